"""The C ABI library without a GPU: it loads, exports every symbol the header
declares, rejects bad arguments and computes the FP64 camera frame on the
host bit for bit like the FP64 oracle."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def B():
    import birp_cpp_gb300 as B
    from birp_cpp_gb300 import build
    build.build()
    return B


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "birp_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(birp_[a-z0-9_]+)\s*\(", src)))


def test_every_declared_symbol_exported(B):
    L = B.lib()
    names = declared_symbols()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_not_initialised_errors(B):
    L = B.lib()
    import ctypes as C
    h = C.c_void_p()
    xs = np.linspace(0, 1, 3)
    v = np.zeros((3, 3, 3), np.float32)
    st = L.birp_cube_create(xs.ctypes.data, 3, xs.ctypes.data, 3, xs.ctypes.data, 3, v.ctypes.data, C.byref(h))
    assert st == B.ERR_NOT_INIT
    assert b"birp_init" in L.birp_last_error()


def test_camera_defaults_match_reference_cli(B):
    c = B.camera_defaults()
    assert (c.nx, c.ny, c.n_samples, c.ray_length) == (144, 144, 200, 44.0)
    assert abs(c.pos[0] - 5.91813) < 1e-6 and abs(c.aim[0] - 7.81768) < 1e-6
    assert c.trilinear == 0 and c.march == B.PREFIX


@pytest.mark.parametrize("bad", [dict(nx=0), dict(fov_w=0.0), dict(fov_h=180.0), dict(n_samples=0),
                                 dict(ray_length=-1.0), dict(segments=3), dict(march=7)])
def test_camera_validation(B, bad):
    kw = dict(pos=(1, 2, 3), aim=(9, 0, 0), fov_w=27.0, fov_h=16.0, nx=32, ny=16)
    kw.update(bad)
    cam = B.camera(**kw)
    with pytest.raises(B.BirpError) as e:
        B.camera_frame(cam)
    assert e.value.status == B.ERR_INVALID


POSES = [((-2, -12, 16), (10, 0, 0)), ((5.91813, 6.74116, 17.7067), (7.81768, 0, 0)), ((1, 1, 1), (1, 0, 0)),
         ((3.49, 0.0746, 0.244), (9, 0, 0)), ((-7, 3, -12), (9, 0, 0)), ((12, -5, 2), (4, 0, 0)),
         ((0.3, 18.2, 5.5), (9, 0, 0))]


@pytest.mark.parametrize("pos,aim", POSES)
def test_frame_bitwise_equals_oracle(B, oracle, pos, aim):
    """The product's host FP64 frame == the FP64 oracle's, bit for bit: the GPU
    rebuilds the oracle's FP64 ray directions from it."""
    cam = B.camera(pos, aim, 27.0, 16.0, 1024, 600, n_samples=880)
    ocam = oracle.camera64(pos, aim, 27.0, 16.0, 1024, 600, n_samples=880)
    f = B.camera_frame(cam)
    g = oracle.frame64(ocam)
    assert np.array_equal(f["rinv"], g["rinv"])
    for k in ("tfx", "tfy", "aspect", "dt", "K", "angle_sun"):
        assert f[k] == g[k], k


@pytest.mark.parametrize("roll", [-10.0, 3.25, 7.5])
def test_frame_with_roll_bitwise_equals_oracle(B, oracle, roll):
    """A roll offset (an extension; 0 is the reference's pose) gives the
    oracle's frame bit for bit too, turns the frame by that angle about the
    view axis, and leaves the Sun angle it is added to unchanged."""
    pos, aim = (-2, -12, 16), (10, 0, 0)
    cam = B.camera(pos, aim, 27.0, 16.0, 288, 168, n_samples=880, roll=roll)
    f = B.camera_frame(cam)
    g = oracle.frame64(oracle.camera64(pos, aim, 27.0, 16.0, 288, 168, 880, 44.0, 0, roll))
    assert np.array_equal(f["rinv"], g["rinv"])
    f0 = B.camera_frame(B.camera(pos, aim, 27.0, 16.0, 288, 168, n_samples=880))
    assert f["angle_sun"] == f0["angle_sun"]
    # the view axis (third column of R^-1, the -z camera axis) is unchanged;
    # the image axes turn by the roll
    assert np.allclose(f["rinv"][:, 2], f0["rinv"][:, 2], atol=1e-12)
    c = float(np.dot(f["rinv"][:, 0], f0["rinv"][:, 0]))
    assert abs(abs(c) - np.cos(np.radians(roll))) < 1e-12


def test_frame_rotation_is_orthonormal(B):
    for pos, aim in POSES:
        f = B.camera_frame(B.camera(pos, aim, 27.0, 16.0, 64, 32))
        R = f["rinv"]
        assert np.allclose(R @ R.T, np.eye(3), atol=1e-12)
