"""The reference-API C++ classes (birp_cpp_gb300/cpp): host parts on the CPU
(.dat loader, FITS and CSV writers) and the full GPU path on a GPU."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "birp_cpp_gb300", "lib")


def _compile(src, out):
    from birp_cpp_gb300 import build
    build.build()
    cmd = ["g++", "-O2", "-std=c++17", "-pthread", os.path.join(ROOT, "tests", "cpp", src), "-I",
           os.path.join(ROOT, "birp_cpp_gb300", "cpp", "include"), "-I", os.path.join(ROOT, "include"), "-L", LIBDIR,
           "-lbirp_classes", "-lbirp_gb300",
           f"-Wl,-rpath,{LIBDIR}", "-o", out]
    subprocess.run(cmd, check=True)


def read_fits(path):
    raw = open(path, "rb").read()
    assert len(raw) % 2880 == 0
    cards, off = {}, 0
    while True:
        c = raw[off:off + 80].decode()
        off += 80
        if c.startswith("END"):
            break
        if "=" in c[:10]:
            k, v = c[:8].strip(), c[10:].split("/")[0].strip()
            cards[k] = v
    data_off = (off + 2879) // 2880 * 2880
    nx, ny = int(cards["NAXIS1"]), int(cards["NAXIS2"])
    img = np.frombuffer(raw[data_off:data_off + 4 * nx * ny], ">f4").reshape(ny, nx)
    return cards, img


def test_loader_and_writers_cpu(tmp_path):
    exe = str(tmp_path / "cpu_test")
    _compile("classes_cpu_test.cpp", exe)
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    cards, img = read_fits(str(tmp_path / "t.fits"))
    assert cards["SIMPLE"] == "T" and cards["BITPIX"] == "-32" and cards["NAXIS"] == "2"
    assert float(cards["CRVAL1"]) == -2.0 and float(cards["CRVAL2"]) == -1.5 and float(cards["CDELT1"]) == 1.0
    assert float(cards["POS_X"]) == 1.5 and float(cards["AIM_X"]) == 7.0
    want = np.array([[10 * j + i + 0.5 for i in range(4)] for j in range(3)], np.float32)
    assert np.array_equal(img, want)
    rows = open(tmp_path / "t.dat").read().strip().split("\n")
    assert rows[1] == "10.500000,11.500000,12.500000,13.500000,"


@pytest.mark.gpu
def test_classes_on_gpu(tmp_path, birp, oracle):
    exe = str(tmp_path / "gpu_test")
    _compile("classes_test.cpp", exe)
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    # the CLI-default CMEM render (written to FITS after the first Render)
    # matches the FP64 oracle; the camera stores its pose as float, like the
    # reference, so the oracle gets the same float pose
    cards, img = read_fits(str(tmp_path / "cmem_cli_default.fits"))
    f32 = lambda v: float(np.float32(v))
    cam = oracle.camera64(tuple(map(f32, (5.91813, 6.74116, 17.7067))), (f32(7.81768), 0, 0), 36.0, 36.0, 144, 144)
    ref = oracle.render64(oracle.Cmem64(), cam, threads=os.cpu_count() or 4)
    m = ref > 1e-3 * ref.max()
    assert (np.abs(img[m] - ref[m]) / ref[m]).max() <= 1e-5
    assert np.float32(cards["POS_X"]) == np.float32(5.91813)  # 9 digits round-trip FP32


def test_cell_record_index_arithmetic(tmp_path):
    """The record addressing the kernels share (csrc/cell_index.h), checked on
    the host: in range for cells -1..n-1, equal to the build order, and kept
    in range by unit steps."""
    exe = str(tmp_path / "cell_index_test")
    subprocess.run(["g++", "-O2", "-std=c++17", os.path.join(ROOT, "tests", "cpp", "cell_index_test.cpp"), "-o", exe],
                   check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
