"""The render path at its limits, against the FP64 oracle: the largest sample
count a camera accepts (2^22 per ray), a 16.7-megapixel image, cells 10^4
times thinner than their neighbours, and a cube 1000 Re from the origin with
a cell only 8 FP32 ulps wide, where an FP32 cell index can be off by more
than one (the negative-value scan then tests every sample in FP64)."""
import os

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 4


def o_cam(oracle, cam):
    return oracle.camera64(tuple(cam.pos), tuple(cam.aim), cam.fov_w_deg, cam.fov_h_deg, cam.nx, cam.ny,
                           cam.n_samples, cam.ray_length, cam.march)


def test_max_samples_per_ray_exact(birp, oracle):
    """2^22 samples per ray (the camera's limit) on a constant field: each
    pixel is (in-box samples) * K, bit for bit, both march modes and both
    interpolations; and one sample more is rejected."""
    xs, ys, zs = np.linspace(-6, 6, 25), np.linspace(-5, 5, 21), np.linspace(-4, 4, 17)
    ones = np.ones((17, 21, 25))
    g = birp.Cube(xs, ys, zs, ones.astype(np.float32))
    oc = oracle.Cube64(xs, ys, zs, ones, 1)
    for march in (birp.PREFIX, birp.CLIP):
        for tri in (True, False):
            cam = birp.camera((-5.5, 0.3, 0.2), (3.0, 0, 0), 30.0, 20.0, 3, 2, n_samples=1 << 22, ray_length=20.0,
                              trilinear=tri, march=march)
            img = birp.render(g, cam)
            ref = oracle.render64(oc, o_cam(oracle, cam), threads=THREADS).astype(np.float32)
            assert np.array_equal(img, ref), (march, tri, img, ref)
    with pytest.raises(birp.BirpError):
        birp.render(g, birp.camera((0, 0, 0), (1, 0, 0), 10, 10, 2, 2, n_samples=(1 << 22) + 1))
    g.close()


def test_large_image(birp, oracle):
    """4096 x 4096 pixels (16.7 M rays) through one plain call: 4000 random
    pixels and the four corners bit for bit against the oracle on a constant
    field (each pixel is its in-box sample count * K)."""
    from birp_cpp_gb300 import synth
    xs, ys, zs = synth.stretched_axis(-30, 25, 80), synth.stretched_axis(-30, 30, 72), synth.stretched_axis(-28, 28, 64)
    ones = np.ones((64, 72, 80))
    g = birp.Cube(xs, ys, zs, ones.astype(np.float32))
    oc = oracle.Cube64(xs, ys, zs, ones, 1)
    cam = birp.camera((-2.0, -12.0, 16.0), (10.0, 0, 0), 60.0, 60.0, 4096, 4096, n_samples=300, ray_length=44.0,
                      march=birp.CLIP)
    img = birp.render(g, cam)
    assert img.shape == (4096, 4096) and np.isfinite(img).all()
    rng = np.random.default_rng(3)
    pi = rng.integers(0, 4096, 4000)
    pj = rng.integers(0, 4096, 4000)
    pi = np.concatenate([pi, [0, 4095, 0, 4095]])
    pj = np.concatenate([pj, [0, 0, 4095, 4095]])
    ref = oracle.render64_pixels(oc, o_cam(oracle, cam), pi, pj, threads=THREADS).astype(np.float32)
    bad = np.flatnonzero(img[pj, pi] != ref)
    assert len(bad) == 0, (len(bad), pi[bad[:4]], pj[bad[:4]])
    g.close()


def thin_cell_axis(lo, hi, n, thin_at, width):
    """n nodes on [lo, hi], evenly spaced except one cell of `width` starting
    at node index thin_at."""
    xs = np.linspace(lo, hi, n - 1)
    xs = np.insert(xs, thin_at + 1, xs[thin_at] + width)
    return xs


@pytest.mark.parametrize("layout", [0, 1, 2])
def test_thin_cells_signed_field(birp, oracle, layout):
    """A cell 3.2e-5 wide next to cells ~0.13 wide (span / smallest cell just
    under the index-table limit of 65536): nearest-mode crossings of the thin
    cell are decided in float-float / FP64, and the negative-value flags'
    one-cell margin covers its neighbours. Signed values make rays stop
    inside and around the thin cells."""
    xs = thin_cell_axis(0.0, 2.0, 17, 7, 3.2e-5)
    ys = thin_cell_axis(-1.0, 1.0, 15, 6, 3.2e-5)
    zs = np.linspace(-1.0, 1.0, 11)
    rng = np.random.default_rng(12)
    v = rng.uniform(0.2, 1.0, (len(zs), len(ys), len(xs)))
    v[:, :, 8] = -0.5   # the plane just past the thin x cell
    v[3, 7, 2] = -1.0
    v = v.astype(np.float32)
    g = birp.Cube(xs, ys, zs, v, layout=layout)
    for tri in (True, False):
        oc = oracle.Cube64(xs, ys, zs, v.astype(np.float64), int(tri))
        for march in (birp.PREFIX, birp.CLIP):
            for pos, aim in [((0.05, 0.02, 0.01), (1.9, 0, 0)), ((-1.0, -0.9, 0.5), (1.0, 0, 0))]:
                cam = birp.camera(pos, aim, 40.0, 40.0, 45, 39, n_samples=4000, ray_length=4.0, trilinear=tri,
                                  march=march)
                img = birp.render(g, cam)
                ref = oracle.render64(oc, o_cam(oracle, cam), threads=THREADS)
                mx, rms, n = rel_err(img, ref)
                assert mx <= 1e-5 and np.array_equal(img == 0, ref == 0), (tri, march, pos, mx, n)
    g.close()


@pytest.mark.parametrize("layout", [0, 1, 2])
def test_far_cube_every_sample_exact(birp, oracle, layout):
    """A cube at x in [1000, 1010] Re with a 5e-4 cell (8 FP32 ulps of 1000):
    the FP32 position of a sample is too coarse to trust its cell within one,
    so the negative-value scan tests every sample in FP64. Sign-only values in
    nearest mode make each pixel (run length) * K: bit for bit."""
    xs = thin_cell_axis(1000.0, 1010.0, 21, 9, 5e-4)
    ys = np.linspace(-1.0, 1.0, 9)
    zs = np.linspace(-1.0, 1.0, 7)
    rng = np.random.default_rng(21)
    s = np.where(rng.random((len(zs), len(ys), len(xs))) < 0.08, -1.0, 1.0)
    s[:, :, 10] = -1.0  # the node just past the thin cell
    s = s.astype(np.float32)
    g = birp.Cube(xs, ys, zs, s, layout=layout)
    oc = oracle.Cube64(xs, ys, zs, s.astype(np.float64), 0)
    for march in (birp.PREFIX, birp.CLIP):
        for pos in [(1000.2, 0.1, 0.05), (999.0, -0.7, 0.3)]:
            cam = birp.camera(pos, (1009.0, 0, 0), 20.0, 20.0, 31, 27, n_samples=4000, ray_length=10.0,
                              trilinear=False, march=march)
            img = birp.render(g, cam)
            ref = oracle.render64(oc, o_cam(oracle, cam), threads=THREADS).astype(np.float32)
            bad = np.argwhere(img != ref)
            assert len(bad) == 0, (march, pos, len(bad), bad[:4])
            if march == birp.CLIP or pos[0] >= 1000.0:  # PREFIX from outside the box renders 0
                assert (ref > 0).sum() > 100
    g.close()
