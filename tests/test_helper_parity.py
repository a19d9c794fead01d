"""The Helper class of the C++ classes (birp_cpp_gb300/cpp, the reference's
src/Helper.cpp) on the CPU: known answers, and agreement with the
reference's own Helper compiled into oracle/_ref/libbirp_ref.so (when the
reference tree was present to build it) on the same inputs, through the
shared C shim oracle/helper_shim.cpp."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "birp_cpp_gb300", "lib")
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libbirp_ref.so")

F = C.POINTER(C.c_float)


def _bind(lib):
    lib.h_julian.restype = C.c_float
    lib.h_julian.argtypes = [C.c_int, C.c_int, C.c_float]
    lib.h_nearest.restype = C.c_int
    lib.h_nearest.argtypes = [C.c_float, F, C.c_int]
    for n in ("h_radec_gsi", "h_radec_gse"):
        getattr(lib, n).argtypes = [C.c_float, C.c_float, F]
    lib.h_xy_radec.argtypes = [C.c_float, C.c_float, F, F, F, F, C.c_int, C.c_float, F]
    lib.h_det.argtypes = [F, C.c_int, C.c_int, F]
    lib.h_explode_float.argtypes = [C.c_char_p, C.c_char, F, C.c_int]
    return lib


@pytest.fixture(scope="module")
def ours(tmp_path_factory):
    from birp_cpp_gb300 import build
    build.build()
    out = str(tmp_path_factory.mktemp("helper") / "libhelper_ours.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", os.path.join(ROOT, "oracle", "helper_shim.cpp"),
                    "-I", os.path.join(ROOT, "birp_cpp_gb300", "cpp", "include", "birp"),
                    "-I", os.path.join(ROOT, "include"), "-L", LIBDIR,
                    "-lbirp_classes", "-lbirp_gb300", f"-Wl,-rpath,{LIBDIR}", "-o", out], check=True)
    return _bind(C.CDLL(out))


@pytest.fixture(scope="module")
def ref():
    if not os.path.exists(REF_LIB):
        pytest.skip("oracle/_ref/libbirp_ref.so not built (reference tree absent)")
    lib = C.CDLL(REF_LIB)
    if not hasattr(lib, "h_julian"):
        pytest.skip("oracle/_ref/libbirp_ref.so predates the Helper shim")
    return _bind(lib)


def fp(a):
    a = np.ascontiguousarray(a, np.float32)
    return a, a.ctypes.data_as(F)


def call_vec(lib, name, n_out, *args):
    out = np.zeros(n_out, np.float32)
    getattr(lib, name)(*args, out.ctypes.data_as(F))
    return out


def test_known_answers(ours):
    assert ours.h_julian(2000, 1, 1.5) == 2451545.0  # J2000.0
    assert ours.h_julian(1582, 10, 15.0) == 2299160.5  # first Gregorian day
    m = call_vec(ours, "h_gei2gse", 16)
    R = m.reshape(4, 4)[:3, :3].astype(np.float64)
    assert np.allclose(R @ R.T, np.eye(3), atol=1e-6)  # a rotation
    v = call_vec(ours, "h_radec_gsi", 3, C.c_float(0.0), C.c_float(0.0))
    assert np.allclose(v, [1, 0, 0], atol=1e-7)
    a, pa = fp([[0, -1, 0], [1, 0, 0], [0, 0, 1]])
    inv = np.zeros(9, np.float32)
    assert ours.h_inverse(pa, 3, inv.ctypes.data_as(F)) == 0
    assert np.allclose(inv.reshape(3, 3), a.T)
    z, pz = fp(np.zeros(9))
    assert ours.h_inverse(pz, 3, inv.ctypes.data_as(F)) == 1  # "Determinant is 0"
    d = C.c_float()
    _, p23 = fp(np.zeros(6))
    assert ours.h_det(p23, 2, 3, C.byref(d)) == 1  # "Matrix is not quadratic"
    buf, pb = fp(np.zeros(8))
    assert ours.h_explode_float(b"1.5,,2,-3e2", b",", pb, 8) == 3 and list(buf[:3]) == [1.5, 2.0, -300.0]
    _, ps = fp([0.1, 0.2, 5.0])
    assert ours.h_equal_distance(ps, 3) == 1  # the reference's check never fails


def test_matches_reference_helper(ours, ref):
    rng = np.random.default_rng(5)
    # Julian dates across the calendar switch and before year 0
    for y, m, d in [(2024, 1, 1.0), (1582, 10, 4.0), (1582, 10, 15.0), (1, 3, 1.0), (-100, 7, 12.25), (1999, 12, 31.5)]:
        assert ours.h_julian(y, m, d) == ref.h_julian(y, m, d), (y, m, d)
    assert np.array_equal(call_vec(ours, "h_gei2gse", 16), call_vec(ref, "h_gei2gse", 16))
    for ra, dec in zip(rng.uniform(0, 360, 300), rng.uniform(-89, 89, 300)):
        for name in ("h_radec_gsi", "h_radec_gse"):
            a = call_vec(ours, name, 3, C.c_float(ra), C.c_float(dec))
            b = call_vec(ref, name, 3, C.c_float(ra), C.c_float(dec))
            assert np.allclose(a, b, rtol=1e-6, atol=1e-7), (name, ra, dec, a, b)
    for xyz in rng.normal(0, 10, (300, 3)):
        _, px = fp(xyz)
        for alt in (0, 1):
            a, b = (call_vec(L, "h_spherical", 3, px, alt) for L in (ours, ref))
            assert np.allclose(a, b, rtol=1e-6, atol=1e-7)
        assert np.allclose(*(call_vec(L, "h_distance", 2, px) for L in (ours, ref)), rtol=1e-6)
    # 1-D interpolation and its nearest-node search (queries above the first node)
    x, px = fp(np.sort(rng.uniform(-5, 5, 20)))
    y, py = fp(rng.normal(0, 1, 20))
    q, pq = fp(rng.uniform(x[0] + 1e-3, 6, 200))
    a, b = (call_vec(L, "h_interp1", 200, px, py, 20, pq, 200) for L in (ours, ref))
    assert np.allclose(a, b, rtol=1e-5, atol=1e-6)
    for v in rng.uniform(-6, 6, 100):
        assert ours.h_nearest(v, px, 20) == ref.h_nearest(v, px, 20)
    # matrices: products, rotation, determinant, inverse
    for n in (2, 3, 4):
        A, pA = fp(rng.normal(0, 1, (n, n)))
        B, pB = fp(rng.normal(0, 1, (n, n)))
        assert np.allclose(*(call_vec(L, "h_matmul", n * n, pA, pB, n) for L in (ours, ref)), rtol=1e-5, atol=1e-6)
        vec, pv = fp(rng.normal(0, 1, n))
        assert np.allclose(*(call_vec(L, "h_matvec", 4, pA, n, n, pv) for L in (ours, ref)), rtol=1e-5, atol=1e-6)
        d1, d2 = C.c_float(), C.c_float()
        assert ours.h_det(pA, n, n, C.byref(d1)) == ref.h_det(pA, n, n, C.byref(d2)) == 0
        assert np.isclose(d1.value, d2.value, rtol=1e-5, atol=1e-6)
        o1, o2 = np.zeros(n * n, np.float32), np.zeros(n * n, np.float32)
        assert ours.h_inverse(pA, n, o1.ctypes.data_as(F)) == ref.h_inverse(pA, n, o2.ctypes.data_as(F)) == 0
        assert np.allclose(o1, o2, rtol=1e-4, atol=1e-5)
    R, pR = fp(rng.normal(0, 1, (3, 3)))
    c3, pc = fp(rng.normal(0, 1, 3))
    assert np.allclose(*(call_vec(L, "h_rotate", 3, pR, pc) for L in (ours, ref)), rtol=1e-6, atol=1e-7)
    # two smallest with a mask, and the sky-grid RA/Dec of image points
    arr, pa = fp(rng.uniform(0, 1, 12))
    mask = np.array([2, 5, 7, 9, 11], np.int32)
    pm = mask.ctypes.data_as(C.POINTER(C.c_int))
    assert np.array_equal(*(call_vec(L, "h_two_min", 2, pa, 12, pm, len(mask)) for L in (ours, ref)))
    ra_g, dec_g = np.meshgrid(np.arange(0.0, 50.0, 5.0), np.arange(-20.0, 25.0, 5.0))
    xs, pxs = fp(ra_g.ravel() * 2.0 + 0.1 * dec_g.ravel())
    ys, pys = fp(dec_g.ravel() * 2.0)
    s1, ps1 = fp(ra_g.ravel())
    s2, ps2 = fp(dec_g.ravel())
    for cx, cy in zip(rng.uniform(5, 85, 50), rng.uniform(-35, 35, 50)):
        a, b = (call_vec(L, "h_xy_radec", 2, C.c_float(cx), C.c_float(cy), pxs, pys, ps1, ps2, len(xs), C.c_float(5.0))
                for L in (ours, ref))
        assert np.allclose(a, b, rtol=1e-5, atol=1e-4), (cx, cy, a, b)
