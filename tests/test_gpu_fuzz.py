"""Seeded random parity sweep against the FP64 oracle: random nonuniform cubes
(2 to 24 nodes per axis), random poses inside and outside the box, random
fields of view, image sizes, sample counts and ray lengths, both march modes,
both interpolations, the three layouts, plain renders and one mixed batch.
Non-negative fields: max relative error <= 1e-5 on pixels above 1e-3 of the
image maximum and the same dark pixels. Sign-only fields in nearest mode
(every run cut at its first negative node): bit for bit."""
import os

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 4


def o_cam(oracle, cam):
    return oracle.camera64(tuple(cam.pos), tuple(cam.aim), cam.fov_w_deg, cam.fov_h_deg, cam.nx, cam.ny,
                           cam.n_samples, cam.ray_length, cam.march)


def random_axis(rng, n):
    widths = rng.uniform(0.2, 2.0, n - 1)
    if rng.random() < 0.3:
        widths[:] = widths[0]  # a uniform axis
    return np.concatenate([[0.0], np.cumsum(widths)]) + rng.uniform(-10, 5)


def random_case(birp, rng):
    dims = rng.integers(2, 25, 3)
    xs, ys, zs = (random_axis(rng, int(n)) for n in dims)
    lo = np.array([xs[0], ys[0], zs[0]])
    hi = np.array([xs[-1], ys[-1], zs[-1]])
    inside = rng.random() < 0.5
    pos = rng.uniform(lo, hi) if inside else rng.uniform(lo - 0.6 * (hi - lo), hi + 0.6 * (hi - lo))
    aim_x = float(rng.uniform(lo[0], hi[0]))
    if abs(aim_x - pos[0]) < 1e-3:
        aim_x += 1.0
    cam = birp.camera(tuple(float(v) for v in pos), (aim_x, 0.0, 0.0), float(rng.uniform(10, 80)),
                      float(rng.uniform(10, 80)), int(rng.integers(3, 25)), int(rng.integers(3, 25)),
                      n_samples=int(rng.integers(20, 3000)), ray_length=float(rng.uniform(5, 80)),
                      trilinear=bool(rng.random() < 0.6), march=int(rng.integers(0, 2)))
    return xs, ys, zs, cam


def test_random_views_nonnegative(birp, oracle):
    rng = np.random.default_rng(20261204)
    items, refs = [], []
    for case in range(48):
        xs, ys, zs, cam = random_case(birp, rng)
        v = rng.uniform(0.0, 5.0, (len(zs), len(ys), len(xs))).astype(np.float32)
        layout = int(rng.integers(0, 3))
        g = birp.Cube(xs, ys, zs, v, layout=layout)
        oc = oracle.Cube64(xs, ys, zs, v.astype(np.float64), int(cam.trilinear))
        ref = oracle.render64(oc, o_cam(oracle, cam), threads=THREADS)
        img = birp.render(g, cam)
        mx, rms, n = rel_err(img, ref)
        assert mx <= 1e-5 and np.array_equal(img == 0, ref == 0), (case, layout, mx, n)
        items.append((g, cam))
        refs.append(ref)
    # the same views in one batch (several cubes, classes and layouts mixed)
    b = birp.Batch(len(items), sum(c.nx * c.ny for _, c in items))
    outs = b.render(items)
    for case, (img, ref) in enumerate(zip(outs, refs)):
        mx, rms, n = rel_err(img, ref)
        assert mx <= 1e-5 and np.array_equal(img == 0, ref == 0), (case, mx, n)
    b.close()
    for g, _ in items:
        g.close()


def test_random_sign_fields_nearest_bitwise(birp, oracle):
    rng = np.random.default_rng(77)
    for case in range(32):
        xs, ys, zs, cam = random_case(birp, rng)
        cam.trilinear = 0
        s = np.where(rng.random((len(zs), len(ys), len(xs))) < 0.15, -1.0, 1.0).astype(np.float32)
        layout = int(rng.integers(0, 3))
        g = birp.Cube(xs, ys, zs, s, layout=layout)
        oc = oracle.Cube64(xs, ys, zs, s.astype(np.float64), 0)
        ref = oracle.render64(oc, o_cam(oracle, cam), threads=THREADS).astype(np.float32)
        img = birp.render(g, cam)
        bad = np.argwhere(img != ref)
        assert len(bad) == 0, (case, layout, len(bad), bad[:4])
        g.close()
