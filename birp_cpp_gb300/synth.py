"""Seeded synthetic workloads with the shapes of the benchmark configurations.

There is no public dataset for this path: cubes are filled from an analytic
magnetosheath model (magnetopause r_mp = r0 (2/(1+cos t))^0.5, bow shock
r_bs = 1.3 r0 (2/(1+cos t))^0.7, sheath 2.5 (10/r)^3 (1 + a N) with N uniform
in [-1, 1] per node, 0.05 (10/r)^3 inside, 0.1 (10/r)^3 outside, 0 for r < 3,
plus two cusp Gaussians of amplitude 3 and sigma 1.5 Re at (4, 0, +-8)).
Values are computed in FP64 (the oracle's copy) and stored FP32 on the GPU.
"""
from __future__ import annotations

import math

import numpy as np

# ------------------------------------------------------------------ axes


def uniform_axis(lo: float, hi: float, n: int) -> np.ndarray:
    return np.linspace(lo, hi, n)


def stretched_axis(lo: float, hi: float, n: int, core: float = 15.0, growth: float = 1.03) -> np.ndarray:
    """n nodes on [lo, hi]: uniform spacing on [-core, core], cells growing
    geometrically by `growth` outward on each side, ending exactly at lo/hi.

    The largest core cell count m whose geometric sides fit in n nodes is
    taken; spare nodes join the core (spacing 2*core/m'), and each side's
    geometric cells are scaled so the side ends exactly at lo / hi."""
    assert lo < -core < core < hi

    def side_cells(length, hc):
        s, k = 0.0, 0
        while s < length - 1e-12:
            k += 1
            s += hc * growth ** k
        return k

    best = None
    for m in range(2, n):
        hc = 2 * core / m
        kl, kr = side_cells(-core - lo, hc), side_cells(hi - core, hc)
        if m + 1 + kl + kr <= n:
            best = (m, kl, kr)
        else:
            break
    m, kl, kr = best
    m += n - (m + 1 + kl + kr)
    hc = 2 * core / m
    coreax = -core + hc * np.arange(m + 1)
    coreax[-1] = core

    def side(length, k):
        steps = hc * growth ** np.arange(1, k + 1)
        steps *= length / steps.sum()
        return np.cumsum(steps)

    left = -core - side(-core - lo, kl)[::-1]
    right = core + side(hi - core, kr)
    ax = np.concatenate([left, coreax, right])
    ax[0], ax[-1] = lo, hi
    assert len(ax) == n and np.all(np.diff(ax) > 0)
    return ax


# ------------------------------------------------------------------ field


def sheath_field(xs, ys, zs, rng, r0: float = 10.0, noise: float = 0.3) -> np.ndarray:
    """FP64 emissivity on the grid, shape (nz, ny, nx)."""
    nz, ny, nx = len(zs), len(ys), len(xs)
    out = np.empty((nz, ny, nx), np.float64)
    X, Y = np.meshgrid(xs, ys, indexing="xy")  # (ny, nx)
    for k, z in enumerate(zs):
        r = np.sqrt(X * X + Y * Y + z * z)
        rs = np.maximum(r, 1e-12)
        cos_t = X / rs
        base = 2.0 / (1.0 + cos_t + 1e-300)
        r_mp = r0 * np.sqrt(base)
        r_bs = 1.3 * r0 * base ** 0.7
        p3 = (10.0 / rs) ** 3
        N = rng.uniform(-1.0, 1.0, size=(ny, nx))
        eta = np.where(r <= r_mp, 0.05 * p3, np.where(r < r_bs, 2.5 * p3 * (1.0 + noise * N), 0.1 * p3))
        for cz in (8.0, -8.0):
            d2 = (X - 4.0) ** 2 + Y ** 2 + (z - cz) ** 2
            eta = eta + 3.0 * np.exp(-d2 / (2 * 1.5 ** 2))
        eta[r < 3.0] = 0.0
        out[k] = eta
    return out


def cube_config0(seed: int = 0):
    """64^3 uniform cube, x in [-10, 20], y, z in [-15, 15]."""
    rng = np.random.default_rng(seed)
    xs, ys, zs = uniform_axis(-10, 20, 64), uniform_axis(-15, 15, 64), uniform_axis(-15, 15, 64)
    return xs, ys, zs, sheath_field(xs, ys, zs, rng)


def cube_config1(seed: int = 1, n: int = 256):
    """n^3 stretched cube: x in [-40, 30], y, z in [-40, 40]."""
    rng = np.random.default_rng(seed)
    xs, ys, zs = stretched_axis(-40, 30, n), stretched_axis(-40, 40, n), stretched_axis(-40, 40, n)
    return xs, ys, zs, sheath_field(xs, ys, zs, rng)


# ------------------------------------------------------------------ cameras

C01_POS = (-2.0, -12.0, 16.0)
C01_AIM = (10.0, 0.0, 0.0)
FOV_W, FOV_H = 27.0, 16.0
SIZES = [(144, 84), (288, 168), (576, 336), (1024, 600)]
STEPS = [0.025, 0.05, 0.1]
RAY_LENGTH = 44.0


def n_samples(step: float) -> int:
    return int(round(RAY_LENGTH / step))


def orbit_positions(n: int, rng) -> np.ndarray:
    """Positions on the elliptical orbit: perigee 1.8 Re, apogee 19 Re,
    inclination 73 deg, argument of perigee 270 deg (node at +x), true
    anomaly uniform."""
    rp, ra = 1.8, 19.0
    a = (rp + ra) / 2
    e = (ra - rp) / (ra + rp)
    inc, argp = math.radians(73.0), math.radians(270.0)
    nu = rng.uniform(0, 2 * math.pi, n)
    r = a * (1 - e * e) / (1 + e * np.cos(nu))
    u = argp + nu
    return np.stack([r * np.cos(u), r * np.sin(u) * math.cos(inc), r * np.sin(u) * math.sin(inc)], 1)


def config2_requests(n: int = 512, seed: int = 2):
    """(pos, aim, nx, ny, step) of the batched config: orbit poses aimed at
    (9, 0, 0), sizes and steps drawn uniformly."""
    rng = np.random.default_rng(seed)
    pos = orbit_positions(n, rng)
    sizes = rng.integers(0, len(SIZES), n)
    steps = rng.integers(0, len(STEPS), n)
    return [(tuple(pos[i]), (9.0, 0.0, 0.0), SIZES[sizes[i]][0], SIZES[sizes[i]][1], STEPS[steps[i]])
            for i in range(n)]


def config2_rolls(n: int = 512, seed: int = 2) -> np.ndarray:
    """Camera roll of each config-2 request in degrees, uniform in [-10, 10]
    (drawn from its own stream, so the poses, sizes and steps of
    config2_requests are unchanged)."""
    return np.random.default_rng(seed + 7919).uniform(-10.0, 10.0, n)


def serving_bases(nx: int, ny: int, nz: int, r0s=(7.5, 9.0, 10.5, 12.0)):
    """Axes and noise-free FP32 base fields of the serving pool's cubes, one
    per standoff r0 group."""
    xs, ys, zs = stretched_axis(-40, 30, nx), stretched_axis(-40, 40, ny), stretched_axis(-40, 40, nz)
    bases = [sheath_field(xs, ys, zs, np.random.default_rng(40 + g), r0=r0, noise=0.0).astype(np.float32)
             for g, r0 in enumerate(r0s)]
    return xs, ys, zs, bases


def serving_cube(i: int, bases) -> np.ndarray:
    """FP32 values of serving cube i: its group's base field times
    (1 + 0.3 N), N uniform in [-1, 1] per node from the cube's own seed,
    computed in FP32 in place (the same values on every call)."""
    base = bases[i % len(bases)]
    v = np.random.default_rng(1000 + i).random(base.shape, dtype=np.float32)
    v *= np.float32(0.6)
    v += np.float32(0.7)
    v *= base
    return v


def cube_stretched(nx: int, ny: int, nz: int, r0: float, seed: int, noise: float = 0.3):
    """A cube with the config-1 axis rule on x in [-40, 30], y, z in [-40, 40]
    and its own magnetopause standoff r0 (bow shock at 1.3 r0)."""
    rng = np.random.default_rng(seed)
    xs, ys, zs = stretched_axis(-40, 30, nx), stretched_axis(-40, 40, ny), stretched_axis(-40, 40, nz)
    return xs, ys, zs, sheath_field(xs, ys, zs, rng, r0=r0, noise=noise)


def config3_specs(n_cubes: int = 48, cams_per_cube: int = 16, n_cmem: int = 8, seed: int = 3):
    """Uneven multi-cube batch: per cube (nx, ny, nz) drawn from multiples of 16
    in [96, 320], standoff r0 in U[7, 12]; each cube gets `cams_per_cube`
    requests from config 2's orbit/size/step sampler; `n_cmem` gridless CMEM
    requests from the same sampler. Returns (cubes, requests) where cubes are
    (nx, ny, nz, r0, seed) and requests are (source, pos, aim, nx, ny, step)
    with source an index into cubes or -1 for CMEM."""
    rng = np.random.default_rng(seed)
    dims = rng.integers(96 // 16, 320 // 16 + 1, size=(n_cubes, 3)) * 16
    r0s = rng.uniform(7.0, 12.0, n_cubes)
    cubes = [(int(d[0]), int(d[1]), int(d[2]), float(r), int(1000 + i)) for i, (d, r) in enumerate(zip(dims, r0s))]
    reqs = []
    cams = config2_requests(n_cubes * cams_per_cube + n_cmem, seed=seed + 1)
    for i in range(n_cubes):
        for j in range(cams_per_cube):
            pos, aim, nx, ny, step = cams[i * cams_per_cube + j]
            reqs.append((i, pos, aim, nx, ny, step))
    for j in range(n_cmem):
        pos, aim, nx, ny, step = cams[n_cubes * cams_per_cube + j]
        reqs.append((-1, pos, aim, nx, ny, step))
    return cubes, reqs
