"""The node-value cube layouts against the FP64 oracle and against the records
layout, through the C ABI: compact (FP32 node values, a cell's coefficients
formed from its 8 corners in the kernel) and pairs ({value, z-slope} per
node, a cell's coefficients formed from its 4 z-edges). Plain renders, point
samples, batches mixing the layouts, and a server holding its cubes in them.

Tolerance: max relative error <= 1e-5 on pixels above 1e-3 of the image
maximum; counts and nearest-node choices exact.
"""
import os

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-5
THREADS = os.cpu_count() or 4


@pytest.fixture(scope="module")
def cubes(birp):
    from birp_cpp_gb300 import synth
    xs, ys, zs, v64 = synth.cube_config1(seed=1, n=128)
    v32 = v64.astype(np.float32)
    return dict(xs=xs, ys=ys, zs=zs, v32=v32, v64=v32.astype(np.float64),
                rec=birp.Cube(xs, ys, zs, v32), compact=birp.Cube(xs, ys, zs, v32, layout=birp.CUBE_COMPACT),
                pairs=birp.Cube(xs, ys, zs, v32, layout=birp.CUBE_PAIRS))


LAYOUTS = ["compact", "pairs"]


def code(birp, name):
    return {"compact": birp.CUBE_COMPACT, "pairs": birp.CUBE_PAIRS}[name]


def o_cam(oracle, cam):
    return oracle.camera64(tuple(cam.pos), tuple(cam.aim), cam.fov_w_deg, cam.fov_h_deg, cam.nx, cam.ny,
                           cam.n_samples, cam.ray_length, cam.march)


def test_node_layouts_memory_and_info(birp, cubes):
    ir, ic, ip = cubes["rec"].info(), cubes["compact"].info(), cubes["pairs"].info()
    assert ir.layout == birp.CUBE_RECORDS and ic.layout == birp.CUBE_COMPACT and ip.layout == birp.CUBE_PAIRS
    nodes = 130 ** 3
    assert nodes * 4 <= ic.device_bytes < nodes * 4 * 1.1
    assert nodes * 8 <= ip.device_bytes < nodes * 8 * 1.05
    assert ir.device_bytes > 7 * ic.device_bytes
    assert ir.device_bytes > 3.5 * ip.device_bytes


@pytest.mark.parametrize("layout", LAYOUTS)
def test_node_layout_constant_field_exact(birp, oracle, layout):
    from birp_cpp_gb300 import synth
    xs, ys, zs = synth.stretched_axis(-40, 30, 64), synth.stretched_axis(-40, 40, 48), np.linspace(-40, 40, 33)
    ones = np.ones((len(zs), len(ys), len(xs)))
    g = birp.Cube(xs, ys, zs, ones.astype(np.float32), layout=code(birp, layout))
    oc = oracle.Cube64(xs, ys, zs, ones, 1)
    for pos, aim in [((1, 2, 3), (9, 0, 0)), ((-30, 25, -35), (4, 0, 0)), ((0.0, 0.0, 0.0), (9, 0, 0))]:
        for march in (birp.PREFIX, birp.CLIP):
            for tri in (True, False):
                cam = birp.camera(pos, aim, 40.0, 30.0, 61, 37, n_samples=880, trilinear=tri, march=march)
                img = birp.render(g, cam)
                ref = oracle.render64(oc, o_cam(oracle, cam), threads=THREADS).astype(np.float32)
                assert np.array_equal(img, ref), (pos, march, tri, int((img != ref).sum()))
    g.close()


@pytest.mark.parametrize("layout", LAYOUTS)
@pytest.mark.parametrize("tri", [True, False])
def test_node_layout_parity_vs_oracle(birp, oracle, cubes, tri, layout):
    from birp_cpp_gb300 import synth
    oc = oracle.Cube64(cubes["xs"], cubes["ys"], cubes["zs"], cubes["v64"], int(tri))
    for pos, aim, _, _, step in synth.config2_requests(5, seed=31):
        cam = birp.camera(pos, aim, 27.0, 16.0, 96, 56, n_samples=synth.n_samples(step), trilinear=tri)
        img = birp.render(cubes[layout], cam)
        ref = oracle.render64(oc, o_cam(oracle, cam), threads=THREADS)
        mx, rms, n = rel_err(img, ref)
        assert mx <= TOL, (pos, tri, mx, rms)
        # nearest mode reads the same node values in both layouts: same bits
        if not tri:
            assert np.array_equal(img, birp.render(cubes["rec"], cam))
        else:
            mx2, _, _ = rel_err(img, birp.render(cubes["rec"], cam))
            assert mx2 <= 2 * TOL


@pytest.mark.parametrize("layout", LAYOUTS)
def test_node_layout_point_samples(birp, cubes, layout):
    rng = np.random.default_rng(8)
    pts = rng.uniform(-45, 35, (4000, 3)).astype(np.float32)
    for tri in (False, True):
        a = cubes[layout].sample(pts, trilinear=tri)
        b = cubes["rec"].sample(pts, trilinear=tri)
        assert np.array_equal(a == -1, b == -1)
        if tri:
            assert np.allclose(a, b, rtol=1e-6, atol=1e-7)
        else:
            assert np.array_equal(a, b)


def test_batch_mixing_layouts_equals_plain(birp, cubes):
    from birp_cpp_gb300 import synth
    items = []
    for k, (pos, aim, nx, ny, step) in enumerate(synth.config2_requests(16, seed=33)):
        cam = birp.camera(pos, aim, 27.0, 16.0, max(8, nx // 6), max(6, ny // 6), n_samples=synth.n_samples(step),
                          trilinear=bool(k % 3), march=k % 2, segments=2 ** (k % 4))
        items.append(((cubes["rec"], cubes["compact"], cubes["pairs"])[k % 3], cam))
    b = birp.Batch(32, 1 << 22)
    outs = b.render(items)
    for (sp, cam), img in zip(items, outs):
        assert np.array_equal(img, birp.render(sp, cam))
    b.close()


@pytest.mark.parametrize("layout", LAYOUTS)
def test_server_node_layout_cubes(birp, cubes, layout):
    srv = birp.Server(birp.server_config(cube_layout=code(birp, layout), cube_budget_bytes=1 << 30, slots=2))
    cid = srv.add_cube(cubes["xs"], cubes["ys"], cubes["zs"], cubes["v32"])
    cam = birp.camera((3, -9, 11), (9, 0, 0), 27.0, 16.0, 144, 84, n_samples=880, segments=1)
    out = np.empty((84, 144), np.float32)
    t = srv.submit(cid, cam, out)
    r = srv.wait(t, 60000)
    assert r.status == 0
    assert np.array_equal(out, birp.render(cubes[layout], cam))
    st = srv.stats()
    per_node = 4 if layout == "compact" else 8
    assert 0 < st.resident_bytes < 1.1 * 130 ** 3 * per_node + (1 << 20)
    srv.close()


def test_pinned_values_upload_equals_pageable(birp):
    """Cube values in pinned host memory (as the server keeps them) are read
    by a kernel straight into the device layout; pageable values go by a 3D
    copy. Both give the same cube: renders equal bit for bit, both layouts."""
    import ctypes as C
    torch = pytest.importorskip("torch")
    from birp_cpp_gb300 import synth
    xs, ys, zs, v = synth.cube_config1(seed=5, n=72)
    v32 = v.astype(np.float32)
    pinned = torch.from_numpy(v32.copy()).pin_memory()
    assert pinned.is_pinned()
    cam = birp.camera((-2.0, -12.0, 16.0), (9.0, 0.0, 0.0), 27.0, 16.0, 96, 56, n_samples=880)
    for layout in (birp.CUBE_RECORDS, birp.CUBE_COMPACT, birp.CUBE_PAIRS):
        ref = birp.Cube(xs, ys, zs, v32, layout=layout)
        h = C.c_void_p()
        ax = [np.ascontiguousarray(a, np.float64) for a in (xs, ys, zs)]
        birp.check(birp.lib().birp_cube_create_layout(ax[0].ctypes.data, len(xs), ax[1].ctypes.data, len(ys),
                                                      ax[2].ctypes.data, len(zs), C.c_void_p(pinned.data_ptr()),
                                                      int(layout), C.byref(h)))
        try:
            for tri in (True, False):
                cam.trilinear = int(tri)
                img = np.empty((cam.ny, cam.nx), np.float32)
                birp.check(birp.lib().birp_render(h, None, C.byref(cam), img.ctypes.data, None))
                assert np.array_equal(img, birp.render(ref, cam)), (layout, tri)
        finally:
            birp.lib().birp_cube_destroy(h)
            ref.close()
