"""birp_batch_render_noalloc: the batch render that allocates nothing.

It serves callers that cannot call cudaMalloc while rendering (an operator
inside another framework that owns all device memory, or a loop that must
not allocate): they pass requests and their own device output buffers, and
the kernel's scratch lives in a fixed array inside the library. This test
calls it through the C ABI twice in a row and checks each result against the
existing allocating batch entry point within the render tolerance (1e-5
relative). It runs last in the suite and also passes alone in a fresh
process."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _requests(birp, spaces, seed):
    from birp_cpp_gb300 import synth
    rng = np.random.default_rng(seed)
    items = []
    for pos, aim, nx, ny, step in synth.config2_requests(12, seed=seed):
        space = spaces[int(rng.integers(0, len(spaces)))]
        cam = birp.camera(pos, aim, 27.0, 16.0, max(8, nx // 4), max(6, ny // 4),
                          n_samples=synth.n_samples(step), trilinear=bool(rng.integers(0, 2)))
        items.append((space, cam))
    return items


def test_noalloc_matches_batch_twice(birp):
    torch = pytest.importorskip("torch")
    from birp_cpp_gb300 import synth
    L = birp.lib()
    fn = L.birp_batch_render_noalloc
    fn.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    xs, ys, zs, v = synth.cube_config1(seed=1, n=96)
    cube = birp.Cube(xs, ys, zs, v.astype(np.float32))
    cmem = birp.Cmem()
    ref_batch = birp.Batch(64, 1 << 22)
    for call, seed in enumerate((31, 32)):
        items = _requests(birp, [cube, cmem], seed)
        ref = ref_batch.render(items)
        outs = [torch.empty(cam.ny * cam.nx, dtype=torch.float32, device="cuda:0") for _, cam in items]
        for o in outs:
            o.fill_(float("nan"))  # stale contents must be overwritten
        torch.cuda.synchronize()
        arr = birp.Batch._reqs(items)
        ptrs = (C.c_void_p * len(outs))(*[o.data_ptr() for o in outs])
        birp.check(fn(arr, len(items), ptrs, None))
        torch.cuda.synchronize()
        for (space, cam), o, r in zip(items, outs, ref):
            img = o.cpu().numpy().reshape(cam.ny, cam.nx)
            assert np.isfinite(img).all(), call
            m = r > 1e-3 * max(r.max(), 1e-30)
            if m.any():
                assert (np.abs(img[m] - r[m]) / r[m]).max() <= TOL, call
            assert np.abs(img - r).max() <= TOL * max(np.abs(r).max(), 1e-30), call
    # more than the fixed limit is rejected before any launch
    items = _requests(birp, [cube], 33) * 22
    arr = birp.Batch._reqs(items)
    dummy = (C.c_void_p * len(items))(*([1] * len(items)))
    assert fn(arr, len(items), dummy, None) == birp.ERR_INVALID
    assert b"256" in L.birp_last_error()
    ref_batch.close()
