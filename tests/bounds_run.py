"""Run by tests/test_gpu_bounds.py in a child process with BIRP_LIB pointing at
the bounds-checking library: renders every kernel class and edge case the
walks have (the three layouts, both interpolations, both march modes, rays from
inside, outside and along the faces, negative values, thin cells, a far cube
that tests every sample, CMEM, one mixed batch, the same mix through the
no-allocation entry point), checks each image against
the FP64 oracle, and exits 0 only if no table access was out of range."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))

import birp_cpp_gb300 as B  # noqa: E402
import pyoracle as O  # noqa: E402
from birp_cpp_gb300 import synth  # noqa: E402
from conftest import rel_err  # noqa: E402
from test_gpu_limits import thin_cell_axis  # noqa: E402

THREADS = os.cpu_count() or 4


def o_cam(cam):
    return O.camera64(tuple(cam.pos), tuple(cam.aim), cam.fov_w_deg, cam.fov_h_deg, cam.nx, cam.ny, cam.n_samples,
                      cam.ray_length, cam.march)


def check(space_o, gpu_space, cam, tol):
    img = B.render(gpu_space, cam)
    ref = O.render64(space_o, o_cam(cam), threads=THREADS)
    mx, _, _ = rel_err(img, ref)
    assert mx <= tol and np.array_equal(img == 0, ref == 0), (mx, tuple(cam.pos))
    return img


def main():
    assert B.lib() and os.environ.get("BIRP_LIB")
    B.init(0)
    B.debug_bounds(reset=True)
    n_img = 0
    # stretched cubes, constant and random fields, every march
    xs, ys, zs = synth.stretched_axis(-20, 25, 41), synth.stretched_axis(-22, 22, 37), synth.stretched_axis(-18, 18, 33)
    rng = np.random.default_rng(3)
    fields = [np.ones((33, 37, 41), np.float32), rng.uniform(0, 5, (33, 37, 41)).astype(np.float32)]
    poses = [((-2.0, -12.0, 16.0), (10.0, 0, 0)), ((1.0, 2.0, 3.0), (9.0, 0, 0)), ((-30.0, 25.0, -35.0), (4.0, 0, 0)),
             ((0.0, 0.0, 0.0), (9.0, 0, 0))]
    for v in fields:
        for layout in (B.CUBE_RECORDS, B.CUBE_COMPACT, B.CUBE_PAIRS):
            g = B.Cube(xs, ys, zs, v, layout=layout)
            for tri in (True, False):
                oc = O.Cube64(xs, ys, zs, v.astype(np.float64), int(tri))
                for pos, aim in poses:
                    for march in (B.PREFIX, B.CLIP):
                        for seg in (1, 8):
                            cam = B.camera(pos, aim, 50.0, 40.0, 33, 25, n_samples=900, ray_length=55.0,
                                           trilinear=tri, march=march, segments=seg)
                            check(oc, g, cam, 1e-5)
                            n_img += 1
            g.close()
    # rays along the faces of a uniform cube
    xe = np.linspace(-8, 8, 17)
    ones = np.ones((17, 17, 17))
    g = B.Cube(xe, xe, xe, ones.astype(np.float32))
    oc = O.Cube64(xe, xe, xe, ones, 1)
    for pos in [(-7.5, 0.0, 0.0), (0.0, -6.0, 0.0), (0.0, 0.0, 7.9)]:
        check(oc, g, B.camera(pos, (5.0, 0, 0), 2.0, 2.0, 17, 17, n_samples=1760, march=B.CLIP), 1e-5)
        n_img += 1
    g.close()
    # negative values (the scan), thin cells, a far cube (every sample exact)
    xt = thin_cell_axis(0.0, 2.0, 17, 7, 3.2e-5)
    yt = thin_cell_axis(-1.0, 1.0, 15, 6, 3.2e-5)
    zt = np.linspace(-1.0, 1.0, 11)
    vt = rng.uniform(0.2, 1.0, (len(zt), len(yt), len(xt)))
    vt[:, :, 8] = -0.5
    vt = vt.astype(np.float32)
    xf = thin_cell_axis(1000.0, 1010.0, 21, 9, 5e-4)
    yf, zf = np.linspace(-1.0, 1.0, 9), np.linspace(-1.0, 1.0, 7)
    sf = np.where(rng.random((len(zf), len(yf), len(xf))) < 0.1, -1.0, 1.0).astype(np.float32)
    for layout in (B.CUBE_RECORDS, B.CUBE_COMPACT, B.CUBE_PAIRS):
        gt = B.Cube(xt, yt, zt, vt, layout=layout)
        gf = B.Cube(xf, yf, zf, sf, layout=layout)
        for tri in (True, False):
            for march in (B.PREFIX, B.CLIP):
                check(O.Cube64(xt, yt, zt, vt.astype(np.float64), int(tri)), gt,
                      B.camera((0.05, 0.02, 0.01), (1.9, 0, 0), 40.0, 40.0, 29, 23, n_samples=3000, ray_length=4.0,
                               trilinear=tri, march=march), 1e-5)
                n_img += 1
            check(O.Cube64(xf, yf, zf, sf.astype(np.float64), 0), gf,
                  B.camera((1000.2, 0.1, 0.05), (1009.0, 0, 0), 20.0, 20.0, 21, 17, n_samples=4000, ray_length=10.0,
                           trilinear=False, march=B.CLIP), 1e-6)  # run lengths exact: only FP32 rounding of the sum
            n_img += 1
        gt.close()
        gf.close()
    # CMEM
    cm = B.Cmem()
    check(O.Cmem64(), cm, B.camera((5.91813, 6.74116, 17.7067), (7.81768, 0, 0), 36.0, 36.0, 40, 40, n_samples=200), 1e-5)
    n_img += 1
    # one batch mixing every class
    gr = B.Cube(xs, ys, zs, fields[1])
    gc = B.Cube(xs, ys, zs, fields[1], layout=B.CUBE_COMPACT)
    gp = B.Cube(xs, ys, zs, fields[1], layout=B.CUBE_PAIRS)
    items = []
    for pos, aim in poses:
        items.append((gr, B.camera(pos, aim, 44.0, 36.0, 31, 23, n_samples=700, ray_length=50.0)))
        items.append((gc, B.camera(pos, aim, 44.0, 36.0, 31, 23, n_samples=700, ray_length=50.0)))
        items.append((gp, B.camera(pos, aim, 44.0, 36.0, 31, 23, n_samples=700, ray_length=50.0)))
        items.append((gr, B.camera(pos, aim, 44.0, 36.0, 31, 23, n_samples=700, ray_length=50.0, trilinear=False)))
        items.append((cm, B.camera(pos, aim, 44.0, 36.0, 15, 11, n_samples=200)))
    b = B.Batch(len(items), sum(c.nx * c.ny for _, c in items))
    outs = b.render(items)
    n_img += len(outs)
    b.close()
    # the same mix through the no-allocation entry point, whose one launch
    # takes the general kernel (every class in one kernel), into device
    # buffers; each image against the FP64 oracle
    import ctypes as C
    import torch
    fn = B.lib().birp_batch_render_noalloc
    fn.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    dev = [torch.full((c.ny * c.nx,), float("nan"), dtype=torch.float32, device="cuda:0") for _, c in items]
    torch.cuda.synchronize()
    ptrs = (C.c_void_p * len(dev))(*[d.data_ptr() for d in dev])
    B.check(fn(B.Batch._reqs(items), len(items), ptrs, None))
    torch.cuda.synchronize()
    o_space = {id(gr): O.Cube64(xs, ys, zs, fields[1].astype(np.float64), 1),
               id(gc): O.Cube64(xs, ys, zs, fields[1].astype(np.float64), 1),
               id(gp): O.Cube64(xs, ys, zs, fields[1].astype(np.float64), 1), id(cm): O.Cmem64()}
    o_nearest = O.Cube64(xs, ys, zs, fields[1].astype(np.float64), 0)
    for (sp, cam), d in zip(items, dev):
        img = d.cpu().numpy().reshape(cam.ny, cam.nx)
        ref = O.render64(o_space[id(sp)] if cam.trilinear else o_nearest, o_cam(cam), threads=THREADS)
        mx, _, _ = rel_err(img, ref)
        assert mx <= 1e-5 and np.array_equal(img == 0, ref == 0), (mx, tuple(cam.pos))
        n_img += 1
    status = B.debug_bounds(reset=False)
    print(f"bounds-checked images: {n_img}; status {status:#x}")
    return 0 if status == 0 else 1


if __name__ == "__main__":
    sys.exit(main())
