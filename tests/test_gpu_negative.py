"""Cubes holding negative values on the GPU. The reference ends a ray at its
first sample < 0 (src/Camera.cpp:205-209): the -1 it returns outside the box
and a negative field value alike. The GPU path must cut every run at the
same sample as the FP64 oracle (PREFIX: the first negative sample; CLIP:
skip negative samples to the first good one, stop at the next), in every
layout, both interpolations, plain and batched.

Stop decisions are exact: a sign-only field in nearest mode makes every
pixel (run length) * K, bit for bit. Sums: a run now ends at a zero crossing,
where an FP32 interpolation of values near zero has a large relative error
(|error| ~ 1e-7 of the cell's corners, not of the value), so short runs lose
digits in any FP32 arithmetic (the reference's own FP32 render of these views
is 1.3e-5 to 1.8e-5 off the FP64 oracle). The trilinear march of such a cube
therefore sums every cell next to a negative node in the FP64 oracle's own
arithmetic, sample by sample, and signed fields are held to the path's 1e-5
on pixels above 1e-3 of the image maximum, with the same dark pixels (a wrong
stop drops or adds whole run segments).
"""
import os

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-5
TOL_SIGNED = TOL  # cells next to negative nodes are summed in FP64
THREADS = os.cpu_count() or 4


def signed_cube(seed=5, harsh=False):
    """Stretched axes; a positive sheath-like field with a ball of -1 fill
    (a body the rays stop at), a slab of mixed-sign noise (trilinear blends
    that cross zero inside cells) and scattered negative nodes. The slab noise
    scales with the local field, or (harsh) with the field's maximum: then
    runs end at zero crossings of cells whose corners cancel at full
    amplitude, and FP32 sums lose digits (the reference's own FP32 arithmetic
    is 1.8e-5 off the FP64 oracle there)."""
    from birp_cpp_gb300 import synth
    rng = np.random.default_rng(seed)
    xs, ys, zs = synth.stretched_axis(-20, 25, 61), synth.stretched_axis(-22, 22, 53), synth.stretched_axis(-18, 18, 47)
    v = synth.sheath_field(xs, ys, zs, rng, r0=8.0).astype(np.float64)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    v[(X - 3) ** 2 + Y ** 2 + Z ** 2 < 4.0 ** 2] = -1.0
    slab = (X > 12) & (X < 16)
    v[slab] = rng.uniform(-0.5, 1.0, slab.sum()) * (np.abs(v).max() if harsh else v[slab])
    spots = rng.random(v.shape) < 0.0002
    v[spots] = -rng.uniform(0.01, 1.0, spots.sum())
    return xs, ys, zs, v.astype(np.float32)


def o_cam(oracle, cam):
    return oracle.camera64(tuple(cam.pos), tuple(cam.aim), cam.fov_w_deg, cam.fov_h_deg, cam.nx, cam.ny,
                           cam.n_samples, cam.ray_length, cam.march)


POSES = [((-16.0, -3.0, 2.0), (9.0, 0, 0)), ((20.0, 15.0, -10.0), (0.0, 0, 0)), ((-40.0, -30.0, 25.0), (8.0, 0, 0)),
         ((0.5, 0.2, 11.0), (6.0, 0, 0))]


@pytest.fixture(scope="module")
def sc():
    return signed_cube()


@pytest.mark.parametrize("layout", [0, 1, 2])
def test_ill_conditioned_signed_field(birp, oracle, layout):
    """Full-amplitude mixed-sign noise: the stop decisions stay exact (same
    dark pixels), the sums within the signed-field bound."""
    xs, ys, zs, v = signed_cube(harsh=True)
    g = birp.Cube(xs, ys, zs, v, layout=layout)
    for tri in (True, False):
        oc = oracle.Cube64(xs, ys, zs, v.astype(np.float64), int(tri))
        for pos, aim in POSES:
            for march in (birp.PREFIX, birp.CLIP):
                cam = birp.camera(pos, aim, 50.0, 40.0, 61, 47, n_samples=1100, ray_length=55.0, trilinear=tri,
                                  march=march)
                img = birp.render(g, cam)
                ref = oracle.render64(oc, o_cam(oracle, cam), threads=THREADS)
                mx, rms, n = rel_err(img, ref)
                assert mx <= TOL_SIGNED and np.array_equal(img == 0, ref == 0), (tri, pos, march, mx, n)
    g.close()


@pytest.mark.parametrize("layout", [0, 1, 2])
@pytest.mark.parametrize("tri", [True, False])
def test_signed_cube_plain(birp, oracle, sc, layout, tri):
    xs, ys, zs, v = sc
    g = birp.Cube(xs, ys, zs, v, layout=layout)
    oc = oracle.Cube64(xs, ys, zs, v.astype(np.float64), int(tri))
    cut = 0
    for pos, aim in POSES:
        for march in (birp.PREFIX, birp.CLIP):
            cam = birp.camera(pos, aim, 50.0, 40.0, 61, 47, n_samples=1100, ray_length=55.0, trilinear=tri,
                              march=march)
            img = birp.render(g, cam)
            ref = oracle.render64(oc, o_cam(oracle, cam), threads=THREADS)
            mx, rms, n = rel_err(img, ref)
            assert mx <= TOL_SIGNED and np.array_equal(img == 0, ref == 0), (pos, march, mx, n)
            # the same pixels without the negative values differ: runs were cut
            cut += int((ref != oracle.render64(oracle.Cube64(xs, ys, zs, np.abs(v).astype(np.float64), int(tri)),
                                               o_cam(oracle, cam), threads=THREADS)).sum())
    assert cut > 1000
    g.close()


@pytest.mark.parametrize("layout", [0, 1, 2])
def test_signed_cube_batched_and_segments(birp, oracle, sc, layout):
    """One batch mixing the signed cube (every lanes-per-ray split) with a
    non-negative cube; each image against the oracle."""
    xs, ys, zs, v = sc
    g = birp.Cube(xs, ys, zs, v, layout=layout)
    pos_v = np.abs(v)
    gp = birp.Cube(xs, ys, zs, pos_v, layout=layout)
    items, refs = [], []
    for k, (pos, aim) in enumerate(POSES):
        for tri in (True, False):
            for march in (birp.PREFIX, birp.CLIP):
                for cube, vals in ((g, v), (gp, pos_v)):
                    cam = birp.camera(pos, aim, 44.0, 36.0, 37 + k, 29, n_samples=900, ray_length=50.0,
                                      trilinear=tri, march=march)
                    items.append((cube, cam))
                    refs.append(oracle.render64(oracle.Cube64(xs, ys, zs, vals.astype(np.float64), int(tri)),
                                                o_cam(oracle, cam), threads=THREADS))
    b = birp.Batch(len(items), sum(c.nx * c.ny for _, c in items))
    outs = b.render(items)
    for i, (img, ref) in enumerate(zip(outs, refs)):
        mx, rms, n = rel_err(img, ref)
        assert mx <= TOL_SIGNED and np.array_equal(img == 0, ref == 0), (i, mx)
    # lanes-per-ray splits: the scan and the run are split-independent
    for seg in (1, 2, 4, 8):
        cam = birp.camera(POSES[0][0], POSES[0][1], 44.0, 36.0, 40, 30, n_samples=1500, ray_length=50.0,
                          march=birp.CLIP, segments=seg)
        ref = oracle.render64(oracle.Cube64(xs, ys, zs, v.astype(np.float64), 1), o_cam(oracle, cam),
                              threads=THREADS)
        img = birp.render(g, cam)
        mx, rms, n = rel_err(img, ref)
        assert mx <= TOL_SIGNED and np.array_equal(img == 0, ref == 0), (seg, mx)
    b.close()
    g.close()
    gp.close()


@pytest.mark.parametrize("layout", [0, 1, 2])
def test_nearest_sign_decisions_bitwise(birp, oracle, sc, layout):
    """Nearest mode over the signs of the signed cube (+1, -1): a pixel is
    (length of its run) * K, so bitwise equality with the FP64 oracle proves
    every negative stop (and every CLIP restart) lands on the oracle's
    sample."""
    xs, ys, zs, v = sc
    s = np.where(v < 0, -1.0, 1.0).astype(np.float32)
    g = birp.Cube(xs, ys, zs, s, layout=layout)
    oc = oracle.Cube64(xs, ys, zs, s.astype(np.float64), 0)
    for pos, aim in POSES:
        for march in (birp.PREFIX, birp.CLIP):
            for seg in (1, 4):
                cam = birp.camera(pos, aim, 50.0, 40.0, 61, 47, n_samples=1700, ray_length=55.0, trilinear=False,
                                  march=march, segments=seg)
                img = birp.render(g, cam)
                ref = oracle.render64(oc, o_cam(oracle, cam), threads=THREADS).astype(np.float32)
                bad = np.argwhere(img != ref)
                assert len(bad) == 0, (pos, march, seg, len(bad), bad[:4])
    g.close()


def test_zero_crossings_exact(birp, oracle):
    """A field that is exactly 0 on node planes and negative beyond them:
    samples just inside a negative cell must stop the ray exactly where the
    FP64 oracle does (ties and near-zero trilinear values)."""
    xs = np.linspace(-6, 6, 13)
    ys = np.linspace(-5, 5, 11)
    zs = np.linspace(-4, 4, 9)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    v = np.where(X < 2.0, 1.0 + 0.1 * Y * Y, np.where(X == 2.0, 0.0, -(X - 2.0))).astype(np.float32)
    g = birp.Cube(xs, ys, zs, v)
    for tri in (True, False):
        oc = oracle.Cube64(xs, ys, zs, v.astype(np.float64), int(tri))
        for march in (birp.PREFIX, birp.CLIP):
            for pos, aim in [((-5.5, 0.3, 0.2), (5.0, 0, 0)), ((-5.0, -4.0, 3.0), (5.0, 0, 0))]:
                cam = birp.camera(pos, aim, 30.0, 30.0, 41, 41, n_samples=2000, ray_length=20.0, trilinear=tri,
                                  march=march)
                img = birp.render(g, cam)
                ref = oracle.render64(oc, o_cam(oracle, cam), threads=THREADS)
                mx, rms, n = rel_err(img, ref)
                assert mx <= TOL and np.array_equal(img == 0, ref == 0), (tri, march, pos, mx)
    g.close()


def test_flags_only_for_negative_cubes(birp, sc):
    """Only a cube with a value below zero carries the per-node flags (one
    byte per node); -0.0 and NaN are not below zero."""
    xs, ys, zs, v = sc
    neg = birp.Cube(xs, ys, zs, v)
    pos = birp.Cube(xs, ys, zs, np.abs(v))
    zero = np.abs(v)
    zero[0, 0, 0] = -0.0
    zero[1, 2, 3] = np.nan
    mz = birp.Cube(xs, ys, zs, zero)
    nodes = v.size
    assert neg.info().device_bytes - pos.info().device_bytes == nodes
    assert mz.info().device_bytes == pos.info().device_bytes
    for c in (neg, pos, mz):
        c.close()


def test_server_signed_cube(birp, oracle, sc):
    """The server's upload path carries the flags too."""
    xs, ys, zs, v = sc
    srv = birp.Server(birp.server_config(slots=2, max_batch_requests=8, max_wait_ms=0.5))
    sid = srv.add_cube(xs, ys, zs, v)
    oc = oracle.Cube64(xs, ys, zs, v.astype(np.float64), 1)
    cams = [birp.camera(p, a, 44.0, 36.0, 33, 27, n_samples=800, ray_length=50.0) for p, a in POSES]
    outs = [np.zeros(c.nx * c.ny, np.float32) for c in cams]
    tickets = [srv.submit(sid, c, o) for c, o in zip(cams, outs)]
    for t, c, o in zip(tickets, cams, outs):
        r = srv.wait(t, 60000)
        assert r.status == 0
        ref = oracle.render64(oc, o_cam(oracle, c), threads=THREADS)
        mx, rms, n = rel_err(o.reshape(c.ny, c.nx), ref)
        assert mx <= TOL_SIGNED and np.array_equal(o.reshape(c.ny, c.nx) == 0, ref == 0), mx
    srv.close()
