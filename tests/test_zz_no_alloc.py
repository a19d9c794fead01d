"""birp_batch_render_noalloc: the batch render that allocates nothing.

It serves callers that cannot call cudaMalloc while rendering (an operator
inside another framework that owns all device memory, or a loop that must
not allocate): they pass requests and their own device output buffers, and
the kernel's scratch lives in a fixed array inside the library. These tests
call it through the C ABI and check its results against the existing
allocating batch entry point and against the FP64 oracle, within the render
tolerance (1e-5 relative): two mixed calls in a row (the general kernel),
one call whose requests share one kernel class (that class's kernel), a call
from a fresh host thread, and the rejected cases (too many requests, a NULL
output, a capturing stream). This file runs last in the suite and also
passes alone in a fresh process."""
import ctypes as C
import os
import threading

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _fn(birp):
    fn = birp.lib().birp_batch_render_noalloc
    fn.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    return fn


def _requests(birp, spaces, seed, trilinear=None):
    from birp_cpp_gb300 import synth
    rng = np.random.default_rng(seed)
    items = []
    for pos, aim, nx, ny, step in synth.config2_requests(12, seed=seed):
        space = spaces[int(rng.integers(0, len(spaces)))]
        tri = bool(rng.integers(0, 2)) if trilinear is None else trilinear
        cam = birp.camera(pos, aim, 27.0, 16.0, max(8, nx // 4), max(6, ny // 4),
                          n_samples=synth.n_samples(step), trilinear=tri)
        items.append((space, cam))
    return items


def _render_noalloc(birp, items, stream=None):
    torch = pytest.importorskip("torch")
    outs = [torch.empty(cam.ny * cam.nx, dtype=torch.float32, device="cuda:0") for _, cam in items]
    for o in outs:
        o.fill_(float("nan"))  # stale contents must be overwritten
    torch.cuda.synchronize()
    arr = birp.Batch._reqs(items)
    ptrs = (C.c_void_p * len(outs))(*[o.data_ptr() for o in outs])
    birp.check(_fn(birp)(arr, len(items), ptrs, stream))
    torch.cuda.synchronize()
    return [o.cpu().numpy().reshape(cam.ny, cam.nx) for o, (_, cam) in zip(outs, items)]


def _match(imgs, refs, what):
    for img, r in zip(imgs, refs):
        assert np.isfinite(img).all(), what
        m = r > 1e-3 * max(r.max(), 1e-30)
        if m.any():
            assert (np.abs(img[m] - r[m]) / r[m]).max() <= TOL, what
        assert np.abs(img - r).max() <= TOL * max(np.abs(r).max(), 1e-30), what


@pytest.fixture(scope="module")
def spaces(birp):
    from birp_cpp_gb300 import synth
    xs, ys, zs, v = synth.cube_config1(seed=1, n=96)
    cube = birp.Cube(xs, ys, zs, v.astype(np.float32))
    return dict(cube=cube, cmem=birp.Cmem(), host=(xs, ys, zs, v.astype(np.float32)))


def test_noalloc_matches_batch_twice(birp, spaces):
    ref_batch = birp.Batch(64, 1 << 22)
    for call, seed in enumerate((31, 32)):
        items = _requests(birp, [spaces["cube"], spaces["cmem"]], seed)
        _match(_render_noalloc(birp, items), ref_batch.render(items), f"mixed call {call}")
    ref_batch.close()


def test_noalloc_one_class_matches_batch_and_oracle(birp, spaces, oracle):
    """Every request trilinear on one records-layout cube: the call takes that
    class's own kernel instead of the general one."""
    items = _requests(birp, [spaces["cube"]], 35, trilinear=True)
    ref_batch = birp.Batch(64, 1 << 22)
    imgs = _render_noalloc(birp, items)
    _match(imgs, ref_batch.render(items), "one class")
    ref_batch.close()
    # the FP64 oracle on every image of the call
    xs, ys, zs, v32 = spaces["host"]
    oc = oracle.Cube64(xs, ys, zs, v32.astype(np.float64), 1)
    for img, (_, cam) in zip(imgs, items):
        ocam = oracle.camera64(tuple(cam.pos), tuple(cam.aim), cam.fov_w_deg, cam.fov_h_deg, cam.nx, cam.ny,
                               cam.n_samples, cam.ray_length, cam.march)
        ref = oracle.render64(oc, ocam, threads=os.cpu_count() or 4)
        mx, _, n = rel_err(img, ref)
        assert mx <= TOL, (mx, n)


def test_noalloc_from_another_thread(birp, spaces):
    """A host thread that never selected a device renders on the library's."""
    items = _requests(birp, [spaces["cube"], spaces["cmem"]], 36)
    ref_batch = birp.Batch(64, 1 << 22)
    ref = ref_batch.render(items)
    ref_batch.close()
    got = {}

    def run():
        try:
            got["imgs"] = _render_noalloc(birp, items)
        except Exception as e:  # reported below, on the test's thread
            got["err"] = e

    t = threading.Thread(target=run)
    t.start()
    t.join()
    assert "err" not in got, got.get("err")
    _match(got["imgs"], ref, "other thread")


def test_noalloc_rejects(birp, spaces):
    torch = pytest.importorskip("torch")
    fn = _fn(birp)
    # nothing to do
    assert fn(None, 0, None, None) == birp.OK
    # more than the fixed limit is rejected before any launch
    items = _requests(birp, [spaces["cube"]], 33) * 22
    arr = birp.Batch._reqs(items)
    dummy = (C.c_void_p * len(items))(*([1] * len(items)))
    assert fn(arr, len(items), dummy, None) == birp.ERR_INVALID
    assert b"256" in birp.lib().birp_last_error()
    # a NULL output
    items = _requests(birp, [spaces["cube"]], 34)[:3]
    arr = birp.Batch._reqs(items)
    buf = torch.empty(items[0][1].nx * items[0][1].ny, dtype=torch.float32, device="cuda:0")
    ptrs = (C.c_void_p * 3)(buf.data_ptr(), None, buf.data_ptr())
    assert fn(arr, 3, ptrs, None) == birp.ERR_INVALID
    # a capturing stream: nothing is recorded, the call is refused
    outs = [torch.empty(c.nx * c.ny, dtype=torch.float32, device="cuda:0") for _, c in items]
    ptrs = (C.c_void_p * 3)(*[o.data_ptr() for o in outs])
    side = torch.cuda.Stream()
    x = torch.zeros(4, device="cuda:0")
    g = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.graph(g, stream=side):
        x.add_(1.0)
        rc = fn(arr, 3, ptrs, side.cuda_stream)
    assert rc == birp.ERR_INVALID
    assert b"capturing" in birp.lib().birp_last_error()
    torch.cuda.synchronize()
    # the library is still usable afterwards
    ref_batch = birp.Batch(8, 1 << 20)
    _match(_render_noalloc(birp, items), ref_batch.render(items), "after refusals")
    ref_batch.close()
