"""GPU parity of the plain per-call render (birp_render through the C ABI)
against the FP64 oracle.

Tolerance (from the path's contract): max relative error <= 1e-5 on pixels
above 1e-3 of the image maximum. Sample counts, in-box ranges and nearest-cell
choices are exact: a constant field must give bit-identical pixels.
"""
import os

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-5
THREADS = os.cpu_count() or 4


@pytest.fixture(scope="module")
def cube0(birp):
    from birp_cpp_gb300 import synth
    xs, ys, zs, v64 = synth.cube_config0(seed=0)
    v32 = v64.astype(np.float32)
    return dict(xs=xs, ys=ys, zs=zs, v64=v32.astype(np.float64), gpu=birp.Cube(xs, ys, zs, v32))


@pytest.fixture(scope="module")
def cube1(birp):
    from birp_cpp_gb300 import synth
    xs, ys, zs, v64 = synth.cube_config1(seed=1)
    v32 = v64.astype(np.float32)
    return dict(xs=xs, ys=ys, zs=zs, v64=v32.astype(np.float64), gpu=birp.Cube(xs, ys, zs, v32))


def o_cube(oracle, c, tri):
    return oracle.Cube64(c["xs"], c["ys"], c["zs"], c["v64"], int(tri))


def o_cam(oracle, cam):
    return oracle.camera64(tuple(cam.pos), tuple(cam.aim), cam.fov_w_deg, cam.fov_h_deg, cam.nx, cam.ny,
                           cam.n_samples, cam.ray_length, cam.march, cam.roll_deg)


def test_constant_field_counts_are_exact(birp, oracle):
    """All-ones cube: each pixel is (in-box sample count) * K, so bitwise
    equality proves the in-box ranges match the FP64 oracle exactly."""
    from birp_cpp_gb300 import synth
    axes = [(np.linspace(-10, 20, 31), np.linspace(-15, 15, 25), np.linspace(-15, 15, 41)),
            (synth.stretched_axis(-40, 30, 96), synth.stretched_axis(-40, 40, 80), synth.stretched_axis(-40, 40, 64))]
    poses = [((-2, -12, 16), (10, 0, 0)), ((1, 2, 3), (9, 0, 0)), ((0.0, 0.0, 0.0), (9, 0, 0)),
             ((-30, 25, -35), (4, 0, 0)), ((3.49, 0.0746, 0.244), (9, 0, 0))]
    for xs, ys, zs in axes:
        ones = np.ones((len(zs), len(ys), len(xs)))
        g = birp.Cube(xs, ys, zs, ones.astype(np.float32))
        oc = oracle.Cube64(xs, ys, zs, ones, 1)
        for pos, aim in poses:
            for march in (birp.PREFIX, birp.CLIP):
                for tri in (True, False):
                    cam = birp.camera(pos, aim, 40.0, 30.0, 97, 61, n_samples=880, trilinear=tri, march=march)
                    img = birp.render(g, cam)
                    ref = oracle.render64(oc, o_cam(oracle, cam), threads=THREADS).astype(np.float32)
                    bad = np.argwhere(img != ref)
                    assert len(bad) == 0, (pos, march, tri, len(bad), bad[:5])
        g.close()


def test_axis_parallel_rays_exact(birp, oracle):
    """Rays nearly parallel to the box faces (camera on an axis, narrow field)
    go through the FP64 range path; counts stay exact."""
    xs = np.linspace(-8, 8, 17)
    ones = np.ones((17, 17, 17))
    g = birp.Cube(xs, xs, xs, ones.astype(np.float32))
    oc = oracle.Cube64(xs, xs, xs, ones, 1)
    for pos, aim in [((-7.5, 0.0, 0.0), (5.0, 0, 0)), ((0.0, -6.0, 0.0), (0.0, 0, 0)), ((0.0, 0.0, 7.9), (0.0, 0, 0))]:
        for march in (birp.PREFIX, birp.CLIP):
            cam = birp.camera(pos, aim, 2.0, 2.0, 33, 33, n_samples=1760, march=march)
            img = birp.render(g, cam)
            ref = oracle.render64(oc, o_cam(oracle, cam), threads=THREADS).astype(np.float32)
            assert np.array_equal(img, ref), (pos, march, int((img != ref).sum()))


@pytest.mark.parametrize("layout", [0, 1])
def test_nearest_axis_parallel_random_field(birp, oracle, layout):
    """Nearest mode with rays nearly parallel to grid planes (camera on an
    axis, narrow field) on a random field: a sample counted in the wrong cell
    would move a pixel by ~1/N relative, far above the tolerance, so this
    checks the float-float / FP64 crossing decisions where they are hardest."""
    rng = np.random.default_rng(12)
    xs = np.linspace(-8, 8, 33)
    ys = np.concatenate([np.linspace(-8, -2, 7), np.linspace(-1.5, 8, 20)])
    vals = rng.uniform(0.5, 1.5, (len(xs), len(ys), len(xs)))
    g = birp.Cube(xs, ys, xs, vals.astype(np.float32), layout=layout)
    oc = oracle.Cube64(xs, ys, xs, vals.astype(np.float32).astype(np.float64), 0)
    for pos, aim in [((-7.5, 0.0, 0.0), (5.0, 0, 0)), ((0.0, -6.0, 0.0), (0.0, 0, 0)), ((0.0, 0.0, 7.9), (0.0, 0, 0)),
                     ((-7.75, 0.25, -0.5), (5.0, 0, 0))]:
        for march in (birp.PREFIX, birp.CLIP):
            cam = birp.camera(pos, aim, 2.0, 2.0, 33, 33, n_samples=1760, march=march, trilinear=False)
            img = birp.render(g, cam)
            ref = oracle.render64(oc, o_cam(oracle, cam), threads=THREADS)
            mx, rms, n = rel_err(img, ref)
            assert mx <= TOL, (pos, march, layout, mx)
    g.close()


@pytest.mark.parametrize("march", [0, 1])
@pytest.mark.parametrize("tri", [True, False])
def test_config0_cube(birp, oracle, cube0, march, tri):
    """64^3 uniform cube, 144x84, step 0.1; the reference pose (outside the
    box) and a pose inside."""
    for pos in [(-2, -12, 16), (1.0, -5.0, 4.0)]:
        cam = birp.camera(pos, (10, 0, 0), 27.0, 16.0, 144, 84, n_samples=440, trilinear=tri, march=march)
        img = birp.render(cube0["gpu"], cam)
        ref = oracle.render64(o_cube(oracle, cube0, tri), o_cam(oracle, cam), threads=THREADS)
        mx, rms, n = rel_err(img, ref)
        assert mx <= TOL, (pos, mx, rms, n)
        assert np.array_equal(img == 0, ref == 0)


def test_config1_full_image_sampled(birp, oracle, cube1):
    """256^3 stretched cube, 1024x600 at step 0.05 (the production render);
    20000 pixels checked against the oracle."""
    cam = birp.camera((-2, -12, 16), (10, 0, 0), 27.0, 16.0, 1024, 600, n_samples=880, trilinear=True)
    img = birp.render(cube1["gpu"], cam)
    rng = np.random.default_rng(11)
    pi = rng.integers(0, 1024, 20000)
    pj = rng.integers(0, 600, 20000)
    ref = oracle.render64_pixels(o_cube(oracle, cube1, True), o_cam(oracle, cam), pi, pj, threads=THREADS)
    got = img[pj, pi]
    m = ref > 1e-3 * ref.max()
    r = np.abs(got[m] - ref[m]) / ref[m]
    assert r.max() <= TOL, (r.max(), np.sqrt((r * r).mean()))
    assert np.isfinite(img).all()


@pytest.mark.parametrize("step", [0.025, 0.1])
def test_config1_orbit_poses(birp, oracle, cube1, step):
    from birp_cpp_gb300 import synth
    reqs = synth.config2_requests(6, seed=5)
    for pos, aim, nx, ny, _ in reqs:
        cam = birp.camera(pos, aim, 27.0, 16.0, 96, 56, n_samples=synth.n_samples(step), trilinear=True)
        img = birp.render(cube1["gpu"], cam)
        ref = oracle.render64(o_cube(oracle, cube1, True), o_cam(oracle, cam), threads=THREADS)
        mx, rms, n = rel_err(img, ref)
        assert mx <= TOL, (pos, mx, rms)


def test_nearest_stretched_exact_cells(birp, oracle, cube1):
    """Nearest mode on stretched axes: cell choices near nodes are decided in
    FP64, so the result stays within tolerance everywhere."""
    cam = birp.camera((-2, -12, 16), (10, 0, 0), 27.0, 16.0, 128, 75, n_samples=880, trilinear=False)
    img = birp.render(cube1["gpu"], cam)
    ref = oracle.render64(o_cube(oracle, cube1, False), o_cam(oracle, cam), threads=THREADS)
    mx, rms, n = rel_err(img, ref)
    assert mx <= TOL, (mx, rms, n)


@pytest.mark.parametrize("seg", [1, 2, 4, 8])
def test_lanes_per_ray(birp, oracle, cube1, seg):
    """A ray split over 1..8 interleaved lanes gives the same image within
    the tolerance."""
    cam = birp.camera((3.49, 0.0746, 0.244), (9, 0, 0), 27.0, 16.0, 64, 40, n_samples=1760, segments=seg)
    img = birp.render(cube1["gpu"], cam)
    ref = oracle.render64(o_cube(oracle, cube1, True), o_cam(oracle, cam), threads=THREADS)
    mx, rms, n = rel_err(img, ref)
    assert mx <= TOL, (seg, mx, rms)


def test_cmem_render(birp, oracle):
    m = birp.Cmem()
    om = oracle.Cmem64()
    for pos in [(-2, -12, 16), (5.91813, 6.74116, 17.7067), (3.49, 0.0746, 0.244)]:
        cam = birp.camera(pos, (10, 0, 0), 27.0, 16.0, 72, 42, n_samples=440)
        img = birp.render(m, cam)
        ref = oracle.render64(om, o_cam(oracle, cam), threads=THREADS)
        mx, rms, n = rel_err(img, ref)
        assert mx <= TOL, (pos, mx, rms)


@pytest.mark.parametrize("roll", [-10.0, 6.5])
def test_roll(birp, oracle, cube1, roll):
    """A camera rolled about its view axis (an extension; the benchmark draws
    the roll U[-10, 10] deg): cube and CMEM against the FP64 oracle."""
    for pos in [(-2, -12, 16), (3.49, 0.0746, 0.244)]:
        cam = birp.camera(pos, (9, 0, 0), 27.0, 16.0, 80, 48, n_samples=880, roll=roll)
        img = birp.render(cube1["gpu"], cam)
        ref = oracle.render64(o_cube(oracle, cube1, True), o_cam(oracle, cam), threads=THREADS)
        mx, rms, n = rel_err(img, ref)
        assert mx <= TOL, (pos, roll, mx)
        flat = birp.render(cube1["gpu"], birp.camera(pos, (9, 0, 0), 27.0, 16.0, 80, 48, n_samples=880))
        assert not np.array_equal(img, flat)
    m = birp.Cmem()
    cam = birp.camera((-2, -12, 16), (10, 0, 0), 27.0, 16.0, 72, 42, n_samples=440, roll=roll)
    mx, rms, n = rel_err(birp.render(m, cam), oracle.render64(oracle.Cmem64(), o_cam(oracle, cam), threads=THREADS))
    assert mx <= TOL, (roll, mx)
    m.close()


def test_cmem_near_earth_cusp(birp, oracle):
    """Two orbit views (config 3's CMEM requests 1 and 4) whose rays pass the
    Earth inside the cusps, where the cusp term cancels most of the
    magnetopause radius (down to ~0.2 Re) and the model is ill-conditioned:
    before float-pair sample positions and the FP64 path for such ramp
    samples, their worst pixels were 4e-3 and 6e-5 off the FP64 oracle.
    Whole images, within the path's 1e-5."""
    from birp_cpp_gb300 import synth
    _, specs = synth.config3_specs()
    cmem = [s for s in specs if s[0] < 0]
    m = birp.Cmem()
    om = oracle.Cmem64()
    for _, pos, aim, nx, ny, step in (cmem[1], cmem[4]):
        cam = birp.camera(pos, aim, synth.FOV_W, synth.FOV_H, nx, ny, n_samples=synth.n_samples(step))
        img = birp.render(m, cam)
        ref = oracle.render64(om, o_cam(oracle, cam), threads=THREADS)
        mx, rms, n = rel_err(img, ref)
        assert mx <= TOL, (pos, mx, rms, n)
    m.close()


def test_cmem_margin_holds(birp):
    m = birp.Cmem()
    err, margin = m.margin_check(1 << 20)
    assert err * 4 < margin, (err, margin)


def test_cmem_sample_kats(birp, golden):
    """GetSample at the reference's CMEM known answers (tests/CMEM_test.cpp)."""
    meta = golden["meta"]
    for name, kats in meta["cmem_kats"].items():
        if name == "default":
            p = birp.cmem_params()
        else:
            v, b, dip, p0, p1, p2, p3, B, al, be, bs, A1, A2, ay, az, de = meta["cmem_sets"][name]
            p = birp.cmem_params(v=v, b=b, dipole=dip, p0=p0, p1=p1, p2=p2, p3=p3, B=B, alpha=al, beta=be, bs=bs,
                                 A1=A1, A2=A2, ay_bs=ay, az_bs=az, density=de)
        got = birp.Cmem(p).sample(np.array([k[0] for k in kats], np.float32))
        want = np.array([k[1] for k in kats], np.float32)
        assert np.allclose(got, want, rtol=2e-6, atol=0), (name, got, want)


def test_cmem_samples_vs_oracle(birp, oracle, golden):
    """3000 CMEM points against the FP64 oracle. Shell choices are exact
    (zero vs non-zero agree). Values agree to 1e-5 relative outside the
    0.05 Re ramp shells; inside them the value is proportional to r - r_mp and
    inherits the FP32 error of r_mp (~1e-5 Re), so there the bound is on the
    absolute error (it moves a ray sum by < 1e-8 of itself)."""
    import ctypes as C
    pts = golden["cmem"]["points"]
    got = birp.Cmem().sample(pts).astype(np.float64)
    om = oracle.Cmem64()
    p64 = pts.astype(np.float64)
    ref = om.sample(p64)
    assert np.array_equal(got == 0, ref == 0)
    x, y, z = p64.T
    r = np.sqrt(x * x + y * y + z * z)
    ramp = np.zeros(len(pts), bool)
    for k in range(len(pts)):
        th = np.arccos(x[k] / r[k]) if x[k] != 0 else 0.0
        ph = np.arccos(y[k] / np.hypot(y[k], z[k])) if y[k] != 0 else 0.0
        a, b = C.c_double(), C.c_double()
        oracle.lib().oracle_cmem64_radii(C.byref(om.s), th, ph, C.byref(a), C.byref(b))
        ramp[k] = abs(r[k] - a.value) <= 0.0251 or abs(r[k] - b.value) <= 0.0251
    m = (ref > 0) & ~ramp
    rel = np.abs(got[m] - ref[m]) / ref[m]
    assert rel.max() < 1e-5, rel.max()
    assert np.abs(got - ref).max() < 1e-5 * ref.max()
    # and the reference's FP32 values are within their own accuracy of both
    want = golden["cmem"]["default"].astype(np.float64)
    assert np.quantile(np.abs(want[m] - ref[m]) / ref[m], 0.99) < 1e-5


def test_cube_sample_matches_oracle(birp, oracle, golden, cube1):
    g = golden["cube"]
    c = birp.Cube(g["xs"].astype(np.float64), g["ys"].astype(np.float64), g["zs"].astype(np.float64), g["values"])
    oc = oracle.Cube64(g["xs"].astype(np.float64), g["ys"].astype(np.float64), g["zs"].astype(np.float64),
                       g["values"].astype(np.float64), 1)
    got = c.sample(g["points"], trilinear=True)
    ref = oc.sample(g["points"].astype(np.float64))
    assert np.array_equal(got == -1, ref == -1)
    assert np.allclose(got, ref, rtol=1e-6, atol=1e-7)
    # reference semantics on a uniform cube: the FP32 reference's own samples
    assert np.allclose(got, g["tri1"], rtol=2e-5, atol=1e-6)
    rng = np.random.default_rng(4)
    pts = rng.uniform(-45, 35, (5000, 3)).astype(np.float32)
    oc1 = oracle.Cube64(cube1["xs"], cube1["ys"], cube1["zs"], cube1["v64"], 0)
    got = cube1["gpu"].sample(pts, trilinear=False)
    ref = oc1.sample(pts.astype(np.float64))
    assert np.array_equal(got, ref.astype(np.float32))


def test_reference_golden_renders(birp, golden):
    """The GPU render of the golden uniform cubes (one of them signed: rays end
    at their first negative sample) with the reference's own camera (200
    samples over 44 Re, dims round(fov/pixel)) agrees with the reference's
    FP32 images to FP32 accuracy."""
    g = golden["renders"]
    axes = (g["xs"].astype(np.float64), g["ys"].astype(np.float64), g["zs"].astype(np.float64))
    spaces = {"cube": birp.Cube(*axes, g["values"]), "cube_signed": birp.Cube(*axes, g["values_signed"]),
              "cmem_default": birp.Cmem()}
    for rec in golden["meta"]["renders"]:
        if rec["renders"] != 1 or rec["space"] == "const":
            continue
        want = g[rec["key"]]
        ny, nx = want.shape
        cam = birp.camera(rec["pos"], rec["aim"], rec["fov_w"], rec["fov_h"], nx, ny, trilinear=rec["trilinear"])
        img = birp.render(spaces[rec["space"]], cam)
        mx, rms, n = rel_err(img, want)
        assert mx < 3e-5, (rec["key"], mx)
        assert np.array_equal(img == 0, want == 0), rec["key"]


def test_linearity_full_size(birp, cube1):
    """render(2 V) == 2 render(V) exactly (a power-of-two scale commutes with
    every FP32 operation) at the full 1024x600 size."""
    xs, ys, zs = cube1["xs"], cube1["ys"], cube1["zs"]
    v = cube1["v64"].astype(np.float32)
    c2 = birp.Cube(xs, ys, zs, 2 * v)
    cam = birp.camera((-2, -12, 16), (10, 0, 0), 27.0, 16.0, 1024, 600, n_samples=880)
    a = birp.render(cube1["gpu"], cam)
    b = birp.render(c2, cam)
    assert np.array_equal(2 * a, b)
    c2.close()


def test_edge_cases(birp, oracle):
    # smallest cube, 1x1 image, one sample, camera far outside
    xs = np.array([0.0, 1.0])
    v = np.arange(8, dtype=np.float32).reshape(2, 2, 2)
    c = birp.Cube(xs, xs, xs, v)
    oc = oracle.Cube64(xs, xs, xs, v.astype(np.float64), 1)
    for cam in [birp.camera((0.5, 0.5, 0.5), (0.9, 0, 0), 10, 10, 1, 1, n_samples=1, ray_length=0.2),
                birp.camera((0.5, 0.5, 0.5), (0.9, 0, 0), 60, 60, 7, 5, n_samples=5000, ray_length=3.0, march=1),
                birp.camera((-50, 40, 30), (0.5, 0, 0), 1, 1, 3, 2, n_samples=200, march=1),
                birp.camera((-50, 40, 30), (0.5, 0, 0), 1, 1, 3, 2, n_samples=200, march=0)]:
        img = birp.render(c, cam)
        ref = oracle.render64(oc, o_cam(oracle, cam))
        mx, rms, n = rel_err(img, ref)
        assert mx <= TOL and np.array_equal(img == 0, ref == 0), (mx, img, ref)
    # invalid inputs are rejected before any launch
    with pytest.raises(birp.BirpError):
        birp.Cube(np.array([0.0, 0.0]), xs, xs, v)
    with pytest.raises(birp.BirpError):
        birp.render(c, birp.camera((0, 0, 0), (1, 0, 0), 10, 10, 0, 4))
    with pytest.raises(birp.BirpError):
        birp.Cube(np.array([0.0]), xs, xs, np.zeros((2, 2, 1), np.float32))


def test_concurrent_callers_share_a_cube(birp, cube1):
    """Host threads rendering different views of one cube at once (the
    reference's Cameras may share a read-only cube across threads) get the
    same images, bit for bit, as the same calls one after another; so do two
    batch objects used from two threads."""
    import concurrent.futures as cf
    from birp_cpp_gb300 import synth
    reqs = synth.config2_requests(24, seed=9)
    cams = [birp.camera(p, a, synth.FOV_W, synth.FOV_H, min(nx, 288), min(ny, 168), n_samples=synth.n_samples(s))
            for p, a, nx, ny, s in reqs]
    cube = cube1["gpu"]
    seq = [birp.render(cube, c) for c in cams]
    with cf.ThreadPoolExecutor(8) as ex:
        par = list(ex.map(lambda c: birp.render(cube, c), cams))
    for k, (a, b) in enumerate(zip(seq, par)):
        assert np.array_equal(a, b), k
    halves = [cams[:12], cams[12:]]
    batches = [birp.Batch(12, sum(c.nx * c.ny for c in h)) for h in halves]
    want = [b.render([(cube, c) for c in h]) for b, h in zip(batches, halves)]
    with cf.ThreadPoolExecutor(2) as ex:
        got = list(ex.map(lambda bh: bh[0].render([(cube, c) for c in bh[1]]), zip(batches, halves)))
    for w, g in zip(want, got):
        for a, b in zip(w, g):
            assert np.array_equal(a, b)
    for b in batches:
        b.close()


def test_kernel_stats_readable(birp):
    s = birp.kernel_stats(reset=True)
    assert set(s) == {"exact_range_rays", "exact_nearest", "exact_cmem", "items", "samples", "cells"}
