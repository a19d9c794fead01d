"""The .dat loader of the C++ classes (DataCube::Load, the reference's
src/DataCube.cpp:28-138) on the CPU, against the reference's own loader
compiled into oracle/_ref/libbirp_ref.so (when the reference tree was present
to build it), through the shared C shim oracle/helper_shim.cpp: the same
axes and values bit for bit, including the reference's token rules (each
white-space separated token read by std::stof: '+' signs, hex, nan / inf,
trailing characters ignored), and the same exception for a token without a
number or out of range."""
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
    lib.h_cube_load.restype = C.c_int
    lib.h_cube_load.argtypes = [C.c_char_p, C.POINTER(C.c_int), F, C.c_int, F, C.c_long]
    return lib


@pytest.fixture(scope="module")
def ours(tmp_path_factory):
    from birp_cpp_gb300 import build
    build.build()
    out = str(tmp_path_factory.mktemp("loader") / "libloader_ours.so")
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
    if not hasattr(lib, "h_cube_load"):
        pytest.skip("oracle/_ref/libbirp_ref.so predates the loader shim")
    return _bind(lib)


def load(lib, path, cap=1 << 22):
    dims = (C.c_int * 3)()
    axes = np.zeros(4096, np.float32)
    vals = np.zeros(cap, np.float32)
    rc = lib.h_cube_load(str(path).encode(), dims, axes.ctypes.data_as(F), len(axes), vals.ctypes.data_as(F), cap)
    n = dims[0] * dims[1] * dims[2] if rc == 0 else 0
    return rc, tuple(dims), axes[: sum(dims)] if rc == 0 else None, vals[:n] if rc == 0 else None


def write(path, dims, axes, rows):
    """The reference's layout: 9 header lines, the dims on line 10, the three
    axes, then one line per row of x values, a blank line after each slice."""
    with open(path, "w") as f:
        f.write("synthetic cube\n" + "".join(f"# {i}\n" for i in range(2, 10)))
        f.write(" ".join(str(d) for d in dims) + "\n")
        for ax in axes:
            f.write(" ".join(ax) + "\n")
        for k, slab in enumerate(rows):
            for row in slab:
                f.write("  ".join(row) + "\n")
            f.write("\n")


def same(a, b):
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    return a.shape == b.shape and bool(((a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))).all())


def test_loader_matches_reference(ours, ref, tmp_path):
    axes = [["-1", "0", "1.5"], ["0", "2"], ["5", "6.25"]]
    quirky = [[["+1.5", "2.5abc", "3e0"], ["-4", "nan", "inf"]],
              [["0x1p3", "1.5E+00-2.5E+00", "7"], ["8", "-0", "1e-3"]]]
    write(tmp_path / "q.dat", (3, 2, 2), axes, quirky)
    a, b = load(ours, tmp_path / "q.dat"), load(ref, tmp_path / "q.dat")
    assert a[0] == b[0] == 0 and a[1] == b[1] == (3, 2, 2)
    assert same(a[2], b[2]) and same(a[3], b[3]), (a[3], b[3])
    assert a[3][6] == 8.0 and a[3][7] == 1.5  # hex; the second of two run-together numbers is not read
    # a larger cube written with 9 significant digits
    rng = np.random.default_rng(4)
    nx, ny, nz = 40, 30, 20
    v = rng.normal(0, 3, (nz, ny, nx)).astype(np.float32)
    axes = [[f"{x:.9g}" for x in np.linspace(-10, 20, n, dtype=np.float32)] for n in (nx, ny, nz)]
    rows = [[[f"{x:.9g}" for x in v[k, j]] for j in range(ny)] for k in range(nz)]
    write(tmp_path / "big.dat", (nx, ny, nz), axes, rows)
    a, b = load(ours, tmp_path / "big.dat"), load(ref, tmp_path / "big.dat")
    assert a[0] == b[0] == 0 and same(a[3], b[3]) and same(a[3], v.reshape(-1))


@pytest.mark.parametrize("token,code", [("abc", 1), ("1e400", 2), ("-1e39", 2)])
def test_loader_errors_match_reference(ours, ref, tmp_path, token, code):
    axes = [["0", "1"], ["0", "1"], ["0", "1"]]
    rows = [[["1", "2"], ["3", "4"]], [["5", "6"], ["7", token]]]
    write(tmp_path / "e.dat", (2, 2, 2), axes, rows)
    assert load(ours, tmp_path / "e.dat")[0] == code
    assert load(ref, tmp_path / "e.dat")[0] == code
