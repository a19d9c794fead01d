"""Pins the CPU oracle against the reference renderer (CPU only).

The golden fixtures in tests/golden/ were produced by the unmodified
reference (tests/golden/make_golden.py). The FP32 restatement must reproduce
them bit for bit; the FP64 oracle must agree with them to FP32 accuracy.
"""
import numpy as np
import pytest

from conftest import rel_err


def _bits_equal(a, b):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    same = (a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))
    return bool(same.all()), int((~same).sum())


def _cmem_args(oracle, name, meta):
    args = meta["cmem_sets"][name]
    if args is None:
        return oracle.cmem_args()
    v, b, dipole, p0, p1, p2, p3, B, alpha, beta, bs, A1, A2, ay, az, dens = args
    return oracle.cmem_args(v=v, b=b, dipole=dipole, p0=p0, p1=p1, p2=p2, p3=p3, B=B, alpha=alpha, beta=beta,
                            bs=bs, A1=A1, A2=A2, ay_bs=ay, az_bs=az, density=dens)


def test_cmem_reference_kats(oracle, golden):
    """The reference's own CMEM known answers (tests/CMEM_test.cpp:21-89)."""
    meta = golden["meta"]
    for name, kats in meta["cmem_kats"].items():
        m = oracle.Cmem32(_cmem_args(oracle, name, meta))
        pts = np.array([k[0] for k in kats], np.float32)
        want = np.array([k[1] for k in kats], np.float32)
        got = m.sample(pts)
        assert np.array_equal(got, want), (name, got, want)


@pytest.mark.parametrize("name", ["default", "test_shifted", "custom"])
def test_cmem_samples_bitwise(oracle, golden, name):
    m = oracle.Cmem32(_cmem_args(oracle, name, golden["meta"]))
    got = m.sample(golden["cmem"]["points"])
    ok, bad = _bits_equal(got, golden["cmem"][name])
    assert ok, f"{bad} CMEM samples differ from the reference"


@pytest.mark.parametrize("tri", [0, 1])
def test_cube_samples_bitwise(oracle, golden, tri):
    g = golden["cube"]
    c = oracle.Cube32(g["xs"], g["ys"], g["zs"], g["values"], tri, 0)
    ok, bad = _bits_equal(c.sample(g["points"]), g[f"tri{tri}"])
    assert ok, f"{bad} cube samples differ from the reference"
    # reference returns -1 outside [c0, c_{n-1}) on every axis
    assert (g[f"tri{tri}"] == -1).any()


def _space32(oracle, golden, rec):
    g = golden["renders"]
    if rec["space"] in ("cube", "cube_signed"):
        vals = g["values_signed"] if rec["space"] == "cube_signed" else g["values"]
        return oracle.Cube32(g["xs"], g["ys"], g["zs"], vals, rec["trilinear"], 0)
    if rec["space"] == "cmem_default":
        return oracle.Cmem32()
    return oracle.Const()


def test_renders_bitwise(oracle, golden):
    """Camera::Render through the FP32 restatement == the reference, bit for bit
    (cube nearest/trilinear, CMEM, the constant test space, repeated renders)."""
    for rec in golden["meta"]["renders"]:
        want = golden["renders"][rec["key"]]
        ny, nx = want.shape
        cam = oracle.camera32(rec["pos"], rec["aim"], rec["fov_w"], rec["fov_h"], nx, ny)
        img = np.zeros((ny, nx), np.float32)
        space = _space32(oracle, golden, rec)
        for _ in range(rec["renders"]):
            oracle.render32(space, cam, out=img)
        ok, bad = _bits_equal(img, want)
        assert ok, f"{rec['key']}: {bad} pixels differ"


def test_fp64_oracle_vs_reference(oracle, golden):
    """The FP64 oracle agrees with the reference's FP32 render to FP32
    accuracy (the reference sums 200 FP32 samples serially), including the
    signed field whose rays end at their first negative sample."""
    g = golden["renders"]
    for rec in golden["meta"]["renders"]:
        if rec["renders"] != 1:
            continue
        want = g[rec["key"]].astype(np.float64)
        ny, nx = want.shape
        cam = oracle.camera64(rec["pos"], rec["aim"], rec["fov_w"], rec["fov_h"], nx, ny)
        if rec["space"] in ("cube", "cube_signed"):
            vals = g["values_signed"] if rec["space"] == "cube_signed" else g["values"]
            sp = oracle.Cube64(g["xs"].astype(np.float64), g["ys"].astype(np.float64), g["zs"].astype(np.float64),
                               vals.astype(np.float64), rec["trilinear"])
        elif rec["space"] == "cmem_default":
            sp = oracle.Cmem64()
        else:
            sp = oracle.Const()
        img = oracle.render64(sp, cam)
        mx, rms, n = rel_err(img, want)
        assert mx < 2e-5, (rec["key"], mx, rms, n)
        # same set of dark pixels (out-of-box prefix is empty in both)
        assert np.array_equal(img == 0, want == 0), rec["key"]


def test_const_field_counts(oracle):
    """Constant field: every pixel is (samples in box) * K exactly; the FP64
    value of 200 samples is 200 K where the reference's FP32 gives 2204118."""
    cam = oracle.camera64((1, 1, 1), (1, 0, 0), 36, 36, 12, 12)
    img = oracle.render64(oracle.Const(), cam)
    K = oracle.frame64(cam)["K"]
    assert np.all(img == 200 * K)
    assert abs(img[0, 0] - 2204113.131424716) < 1e-6


def test_ray_range_matches_march(oracle):
    """oracle_ray_range64 (first in-box sample, first exit) agrees with the
    per-sample march on a constant-valued cube, both march modes."""
    xs = np.linspace(-3, 5, 9)
    ys = np.linspace(-4, 4, 7)
    zs = np.linspace(-2, 6, 5)
    cube = oracle.Cube64(xs, ys, zs, np.ones((5, 7, 9)), 1)
    for pos in [(0.5, 0.2, 1.0), (-9.0, 0.3, 1.0), (20.0, 10.0, -7.0)]:
        for mode in (oracle.PREFIX, oracle.CLIP):
            cam = oracle.camera64(pos, (2.0, 0, 0), 70, 60, 9, 7, n_samples=300, ray_length=30.0, mode=mode)
            img = oracle.render64(cube, cam)
            K = oracle.frame64(cam)["K"]
            for j in range(7):
                for i in range(9):
                    a, b = oracle.ray_range64(cube, cam, i, j)
                    n = (b - a) if (mode == oracle.CLIP or a == 0) else 0
                    assert img[j, i] == n * K, (pos, mode, i, j, a, b)


def test_prefix_equals_clip_inside_box(oracle):
    xs = np.linspace(-10, 20, 16)
    ys = np.linspace(-15, 15, 16)
    zs = np.linspace(-15, 15, 16)
    v = np.random.default_rng(3).uniform(0, 1, (16, 16, 16))
    cube = oracle.Cube64(xs, ys, zs, v, 1)
    a = oracle.render64(cube, oracle.camera64((1, 2, 3), (8, 0, 0), 27, 16, 24, 14, mode=oracle.PREFIX))
    b = oracle.render64(cube, oracle.camera64((1, 2, 3), (8, 0, 0), 27, 16, 24, 14, mode=oracle.CLIP))
    assert np.array_equal(a, b)
    # the reference's config-0 pose lies outside the box: PREFIX renders zeros
    c = oracle.render64(cube, oracle.camera64((-2, -12, 16), (10, 0, 0), 27, 16, 24, 14, mode=oracle.PREFIX))
    assert not c.any()


def test_negative_values_end_the_run(oracle):
    """A negative field value ends a ray's run like the box edge does
    (src/Camera.cpp:205-209): PREFIX stops at the first negative sample; CLIP
    skips negative samples before its first good one and stops at the next.
    Checked per sample against a march over the oracle's own point samples."""
    xs = np.linspace(-3, 5, 9)
    ys = np.linspace(-4, 4, 7)
    zs = np.linspace(-2, 6, 5)
    v = np.random.default_rng(8).uniform(-0.6, 2.0, (5, 7, 9))
    for tri in (0, 1):
        cube = oracle.Cube64(xs, ys, zs, v, tri)
        for mode in (oracle.PREFIX, oracle.CLIP):
            cam = oracle.camera64((0.5, 0.2, 1.0), (2.0, 0, 0), 70, 60, 9, 7, n_samples=300, ray_length=30.0,
                                  mode=mode)
            img = oracle.render64(cube, cam)
            f = oracle.frame64(cam)
            for j in range(7):
                for i in range(9):
                    d = oracle.ray_dir64(cam, i, j)
                    t = (np.arange(300) + 0.5) * f["dt"]
                    pts = np.asarray(cam.pos)[None, :] + t[:, None] * d[None, :]
                    s = cube.sample(pts)  # -1 outside the box
                    bad = s < 0
                    if mode == oracle.PREFIX:
                        end = int(np.argmax(bad)) if bad.any() else 300
                        want = s[:end].sum()
                    else:
                        good = np.flatnonzero(~bad)
                        if len(good) == 0:
                            want = 0.0
                        else:
                            a = good[0]
                            rest = np.flatnonzero(bad[a:])
                            want = s[a:a + (rest[0] if len(rest) else 300 - a)].sum()
                    assert np.isclose(img[j, i], want * f["K"], rtol=1e-12, atol=0), (tri, mode, i, j)


def test_ref32_matches_reference_build_random(oracle):
    """The FP32 restatement against the reference's own Camera::Render
    (oracle/_ref, built from the reference sources where they are present):
    seeded random uniform cubes, poses and fields of view at the reference's
    native camera (200 samples over 44 Re), both interpolations, signed and
    non-negative fields; bit for bit."""
    import os
    if not os.path.exists(oracle.REF_PATH):
        pytest.skip("oracle/_ref not built (reference tree absent)")
    R = oracle.Reference()
    rng = np.random.default_rng(31)
    for case in range(8):
        n = rng.integers(4, 30, 3)
        lo = rng.uniform(-30, 0, 3)
        span = rng.uniform(10, 60, 3)
        xs, ys, zs = (np.linspace(lo[k], lo[k] + span[k], n[k]).astype(np.float32) for k in range(3))
        v = rng.uniform(-1.0 if case % 2 else 0.0, 5.0, (n[2], n[1], n[0])).astype(np.float32)
        tri = case % 4 < 2
        pos = tuple(float(x) for x in rng.uniform(lo - 5, lo + span + 5))
        aim = (float(rng.uniform(lo[0], lo[0] + span[0])), 0.0, 0.0)
        pix, fh, fw = float(rng.uniform(1.0, 3.0)), float(rng.uniform(15, 50)), float(rng.uniform(15, 50))
        h = R.cube(xs, ys, zs, v, int(tri))
        want = R.render(h, pix, fh, fw, pos, aim)
        R.free(h)
        ny, nx = want.shape
        img = np.zeros((ny, nx), np.float32)
        oracle.render32(oracle.Cube32(xs, ys, zs, v, int(tri), 0), oracle.camera32(pos, aim, fw, fh, nx, ny), out=img)
        ok, bad = _bits_equal(img, want)
        assert ok, (case, bad)
