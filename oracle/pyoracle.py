"""ctypes binding of the CPU oracle (oracle/birp_oracle.cpp).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference arm, as the checker or the timed CPU
baseline. The product package never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "libbirp_oracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libbirp_ref.so")

SPACE_CUBE, SPACE_CMEM, SPACE_CONST = 0, 1, 2
PREFIX, CLIP = 0, 1


class O32Cube(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("xs", C.c_void_p), ("ys", C.c_void_p), ("zs", C.c_void_p),
                ("values", C.c_void_p), ("trilinear", C.c_int), ("axis_mode", C.c_int)]


class O64Cube(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("xs", C.c_void_p), ("ys", C.c_void_p), ("zs", C.c_void_p),
                ("values", C.c_void_p), ("trilinear", C.c_int)]


_CMEM_NAMES = ["p0", "p1", "p2", "p3", "bs", "A1", "A2", "B", "alpha", "beta", "ay_bs", "az_bs",
               "dn", "ds", "theta_n", "theta_s", "r0_lin", "charlie", "a5", "a21"]


class O32Cmem(C.Structure):
    _fields_ = [(n, C.c_float) for n in _CMEM_NAMES] + [("beta_c", C.c_float * 4),
                                                        ("pressure_dynamic", C.c_float),
                                                        ("pressure_magnetic", C.c_float)]


class O64Cmem(C.Structure):
    _fields_ = [(n, C.c_double) for n in _CMEM_NAMES] + [("beta_c", C.c_double * 4),
                                                         ("pressure_dynamic", C.c_double),
                                                         ("pressure_magnetic", C.c_double)]


class OCmemArgs(C.Structure):
    _fields_ = [("has_v", C.c_int), ("v", C.c_int * 3), ("has_b", C.c_int), ("b", C.c_int * 3),
                ("dipole", C.c_float), ("p0", C.c_float), ("p1", C.c_int), ("p2", C.c_int),
                ("p3", C.c_int), ("B", C.c_float), ("alpha", C.c_float), ("beta", C.c_float),
                ("bs", C.c_float), ("A1", C.c_float), ("A2", C.c_float), ("ay_bs", C.c_float),
                ("az_bs", C.c_float), ("density", C.c_float)]


class O32Camera(C.Structure):
    _fields_ = [("pos", C.c_float * 3), ("aim", C.c_float * 3), ("fov_w", C.c_float),
                ("fov_h", C.c_float), ("nx", C.c_int), ("ny", C.c_int), ("n_samples", C.c_int),
                ("ray_max", C.c_int), ("mode", C.c_int)]


class O64Camera(C.Structure):
    _fields_ = [("pos", C.c_double * 3), ("aim", C.c_double * 3), ("fov_w", C.c_double),
                ("fov_h", C.c_double), ("nx", C.c_int), ("ny", C.c_int), ("n_samples", C.c_int),
                ("ray_length", C.c_double), ("mode", C.c_int), ("roll", C.c_double)]


def build(quiet: bool = True) -> str:
    """Compiles the oracle library (make in oracle/)."""
    out = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        L.oracle_cmem32_init.argtypes = [P, P]
        L.oracle_cmem64_init.argtypes = [P, P]
        L.oracle_cmem32_sample.argtypes = [P, P, C.c_int, P]
        L.oracle_cmem64_sample.argtypes = [P, P, C.c_int, P]
        L.oracle_cmem64_radii.argtypes = [P, C.c_double, C.c_double, P, P]
        L.oracle_cube32_sample.argtypes = [P, P, C.c_int, P]
        L.oracle_cube64_sample.argtypes = [P, P, C.c_int, P]
        L.oracle_orient32.argtypes = [P, P]
        L.oracle_orient32.restype = C.c_float
        L.oracle_render32.argtypes = [C.c_int, P, P, P, P, C.c_int]
        L.oracle_render32_pixels.argtypes = [C.c_int, P, P, P, P, P, C.c_int, P, C.c_int]
        L.oracle_render64.argtypes = [C.c_int, P, P, P, P, C.c_int]
        L.oracle_render64_pixels.argtypes = [C.c_int, P, P, P, P, P, C.c_int, P, C.c_int]
        L.oracle_frame64.argtypes = [P, P, P, P, P, P, P, P]
        L.oracle_ray_dir64.argtypes = [P, C.c_int, C.c_int, P]
        L.oracle_ray_range64.argtypes = [P, P, C.c_int, C.c_int, P, P]
        _lib = L
    return _lib


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


# ------------------------------------------------------------------ spaces

class Cube32:
    """FP32 cube with the reference's GetSample semantics (axis_mode 0) or a
    per-cell lookup (axis_mode 1)."""

    def __init__(self, xs, ys, zs, values, trilinear=True, axis_mode=0):
        self.xs = np.ascontiguousarray(xs, np.float32)
        self.ys = np.ascontiguousarray(ys, np.float32)
        self.zs = np.ascontiguousarray(zs, np.float32)
        v = np.asarray(values, np.float32)
        assert v.shape == (len(self.zs), len(self.ys), len(self.xs))
        self.values = np.ascontiguousarray(v)
        self.s = O32Cube(len(self.xs), len(self.ys), len(self.zs), _ptr(self.xs), _ptr(self.ys),
                         _ptr(self.zs), _ptr(self.values), int(trilinear), int(axis_mode))
        self.kind = SPACE_CUBE

    def sample(self, pts):
        p = np.ascontiguousarray(pts, np.float32).reshape(-1, 3)
        out = np.empty(len(p), np.float32)
        lib().oracle_cube32_sample(C.byref(self.s), _ptr(p), len(p), _ptr(out))
        return out


class Cube64:
    """The FP64 copy of a cube for the FP64 oracle (per-cell lookup)."""

    def __init__(self, xs, ys, zs, values, trilinear=True):
        self.xs = np.ascontiguousarray(xs, np.float64)
        self.ys = np.ascontiguousarray(ys, np.float64)
        self.zs = np.ascontiguousarray(zs, np.float64)
        v = np.asarray(values, np.float64)
        assert v.shape == (len(self.zs), len(self.ys), len(self.xs))
        self.values = np.ascontiguousarray(v)
        self.s = O64Cube(len(self.xs), len(self.ys), len(self.zs), _ptr(self.xs), _ptr(self.ys),
                         _ptr(self.zs), _ptr(self.values), int(trilinear))
        self.kind = SPACE_CUBE

    def sample(self, pts):
        p = np.ascontiguousarray(pts, np.float64).reshape(-1, 3)
        out = np.empty(len(p), np.float64)
        lib().oracle_cube64_sample(C.byref(self.s), _ptr(p), len(p), _ptr(out))
        return out


def cmem_args(v=None, b=None, dipole=0.0, p0=0.786300004, p1=1, p2=3, p3=4, B=2.0, alpha=2.5,
              beta=-1.6, bs=12.6400003, A1=7.2e-06, A2=3.5000000000000004e-06, ay_bs=0.0,
              az_bs=0.0, density=0.0) -> OCmemArgs:
    """Arguments of CMEM::Init with the reference's defaults (include/Cmem.h:21-41)."""
    a = OCmemArgs()
    a.has_v = int(v is not None)
    a.has_b = int(b is not None)
    for i in range(3):
        a.v[i] = int(v[i]) if v is not None else 0
        a.b[i] = int(b[i]) if b is not None else 0
    a.dipole, a.p0, a.p1, a.p2, a.p3 = dipole, p0, int(p1), int(p2), int(p3)
    a.B, a.alpha, a.beta, a.bs, a.A1, a.A2 = B, alpha, beta, bs, A1, A2
    a.ay_bs, a.az_bs, a.density = ay_bs, az_bs, density
    return a


class Cmem32:
    def __init__(self, args: OCmemArgs | None = None):
        self.args = args if args is not None else cmem_args()
        self.s = O32Cmem()
        lib().oracle_cmem32_init(C.byref(self.args), C.byref(self.s))
        self.kind = SPACE_CMEM

    def sample(self, pts):
        p = np.ascontiguousarray(pts, np.float32).reshape(-1, 3)
        out = np.empty(len(p), np.float32)
        lib().oracle_cmem32_sample(C.byref(self.s), _ptr(p), len(p), _ptr(out))
        return out


class Cmem64:
    def __init__(self, args: OCmemArgs | None = None):
        self.args = args if args is not None else cmem_args()
        self.s = O64Cmem()
        lib().oracle_cmem64_init(C.byref(self.args), C.byref(self.s))
        self.kind = SPACE_CMEM

    def sample(self, pts):
        p = np.ascontiguousarray(pts, np.float64).reshape(-1, 3)
        out = np.empty(len(p), np.float64)
        lib().oracle_cmem64_sample(C.byref(self.s), _ptr(p), len(p), _ptr(out))
        return out


class Const:
    """The reference test's CubeFake: every sample is 1."""
    kind = SPACE_CONST


def _space_ptrs(space):
    if space.kind == SPACE_CUBE:
        return C.byref(space.s), None
    if space.kind == SPACE_CMEM:
        return None, C.byref(space.s)
    return None, None


# ------------------------------------------------------------------ cameras

def camera32(pos, aim, fov_w, fov_h, nx, ny, n_samples=200, ray_max=44, mode=PREFIX) -> O32Camera:
    c = O32Camera()
    for i in range(3):
        c.pos[i] = pos[i]
        c.aim[i] = aim[i]
    c.fov_w, c.fov_h, c.nx, c.ny = fov_w, fov_h, nx, ny
    c.n_samples, c.ray_max, c.mode = n_samples, ray_max, mode
    return c


def camera64(pos, aim, fov_w, fov_h, nx, ny, n_samples=200, ray_length=44.0, mode=PREFIX,
             roll=0.0) -> O64Camera:
    c = O64Camera()
    for i in range(3):
        c.pos[i] = pos[i]
        c.aim[i] = aim[i]
    c.fov_w, c.fov_h, c.nx, c.ny = fov_w, fov_h, nx, ny
    c.n_samples, c.ray_length, c.mode, c.roll = n_samples, ray_length, mode, roll
    return c


def render32(space, cam: O32Camera, threads: int = 1, out=None) -> np.ndarray:
    img = np.zeros((cam.ny, cam.nx), np.float32) if out is None else out
    cb, cm = _space_ptrs(space)
    rc = lib().oracle_render32(space.kind, cb, cm, C.byref(cam), _ptr(img), threads)
    if rc != 0:
        raise RuntimeError(f"oracle_render32 failed ({rc})")
    return img


def render32_pixels(space, cam: O32Camera, pi, pj, threads: int = 1) -> np.ndarray:
    pi = np.ascontiguousarray(pi, np.int32)
    pj = np.ascontiguousarray(pj, np.int32)
    out = np.zeros(len(pi), np.float32)
    cb, cm = _space_ptrs(space)
    rc = lib().oracle_render32_pixels(space.kind, cb, cm, C.byref(cam), _ptr(pi), _ptr(pj), len(pi),
                                      _ptr(out), threads)
    if rc != 0:
        raise RuntimeError(f"oracle_render32_pixels failed ({rc})")
    return out


def render64(space, cam: O64Camera, threads: int = 1) -> np.ndarray:
    img = np.zeros((cam.ny, cam.nx), np.float64)
    cb, cm = _space_ptrs(space)
    rc = lib().oracle_render64(space.kind, cb, cm, C.byref(cam), _ptr(img), threads)
    if rc != 0:
        raise RuntimeError(f"oracle_render64 failed ({rc})")
    return img


def render64_pixels(space, cam: O64Camera, pi, pj, threads: int = 1) -> np.ndarray:
    pi = np.ascontiguousarray(pi, np.int32)
    pj = np.ascontiguousarray(pj, np.int32)
    out = np.zeros(len(pi), np.float64)
    cb, cm = _space_ptrs(space)
    rc = lib().oracle_render64_pixels(space.kind, cb, cm, C.byref(cam), _ptr(pi), _ptr(pj), len(pi),
                                      _ptr(out), threads)
    if rc != 0:
        raise RuntimeError(f"oracle_render64_pixels failed ({rc})")
    return out


def frame64(cam: O64Camera) -> dict:
    rinv = np.zeros(9, np.float64)
    vals = [C.c_double() for _ in range(6)]
    rc = lib().oracle_frame64(C.byref(cam), _ptr(rinv), *[C.byref(v) for v in vals])
    if rc != 0:
        raise RuntimeError("singular pose")
    tfx, tfy, aspect, dt, K, angle_sun = (v.value for v in vals)
    return dict(rinv=rinv.reshape(3, 3), tfx=tfx, tfy=tfy, aspect=aspect, dt=dt, K=K, angle_sun=angle_sun)


def ray_dir64(cam: O64Camera, i: int, j: int) -> np.ndarray:
    d = np.zeros(3, np.float64)
    lib().oracle_ray_dir64(C.byref(cam), i, j, _ptr(d))
    return d


def ray_range64(cube: Cube64, cam: O64Camera, i: int, j: int):
    a, b = C.c_int(), C.c_int()
    lib().oracle_ray_range64(C.byref(cube.s), C.byref(cam), i, j, C.byref(a), C.byref(b))
    return a.value, b.value


def orient32(pos, aim) -> float:
    p = np.ascontiguousarray(pos, np.float32)
    a = np.ascontiguousarray(aim, np.float32)
    return float(lib().oracle_orient32(_ptr(p), _ptr(a)))


# ------------------------------------------------------------------ reference build

class Reference:
    """The unmodified reference renderer built from its own sources
    (oracle/build_ref.sh). Present only where the reference tree exists."""

    def __init__(self):
        if not os.path.exists(REF_PATH):
            raise FileNotFoundError(REF_PATH)
        L = C.CDLL(REF_PATH)
        P = C.c_void_p
        L.ref_cube_new.restype = P
        L.ref_cube_new.argtypes = [P, C.c_int, P, C.c_int, P, C.c_int, P, C.c_int]
        L.ref_cmem_new_default.restype = P
        L.ref_cmem_new.restype = P
        L.ref_cmem_new.argtypes = [P, P, C.c_float, C.c_float, C.c_int, C.c_int, C.c_int] + [C.c_float] * 9
        L.ref_const_new.restype = P
        L.ref_space_free.argtypes = [P, C.c_int]
        L.ref_sample.argtypes = [P, P, C.c_int, P]
        L.ref_render.argtypes = [P, C.c_float, C.c_float, C.c_float] + [C.c_float] * 6 + [C.c_int, P, P, P]
        self.L = L

    def cube(self, xs, ys, zs, values, trilinear):
        xs = np.ascontiguousarray(xs, np.float32)
        ys = np.ascontiguousarray(ys, np.float32)
        zs = np.ascontiguousarray(zs, np.float32)
        v = np.ascontiguousarray(values, np.float32)
        return (self.L.ref_cube_new(_ptr(xs), len(xs), _ptr(ys), len(ys), _ptr(zs), len(zs), _ptr(v),
                                    int(trilinear)), 0)

    def cmem_default(self):
        return (self.L.ref_cmem_new_default(), 1)

    def cmem(self, v, b, dipole, p0, p1, p2, p3, B, alpha, beta, bs, A1, A2, ay_bs, az_bs, density):
        va = (C.c_int * 3)(*v) if v is not None else None
        ba = (C.c_int * 3)(*b) if b is not None else None
        return (self.L.ref_cmem_new(va, ba, dipole, p0, p1, p2, p3, B, alpha, beta, bs, A1, A2, ay_bs,
                                    az_bs, density), 1)

    def const(self):
        return (self.L.ref_const_new(), 2)

    def free(self, h):
        self.L.ref_space_free(h[0], h[1])

    def sample(self, h, pts):
        p = np.ascontiguousarray(pts, np.float32).reshape(-1, 3)
        out = np.empty(len(p), np.float32)
        self.L.ref_sample(h[0], _ptr(p), len(p), _ptr(out))
        return out

    def render(self, h, pixel_size_deg, fov_h, fov_w, pos, aim, renders=1):
        nx = C.c_int(0)
        ny = C.c_int(0)
        self.L.ref_render(h[0], pixel_size_deg, fov_h, fov_w, *pos, *aim, renders, None, C.byref(nx),
                          C.byref(ny))
        img = np.zeros((ny.value, nx.value), np.float32)
        rc = self.L.ref_render(h[0], pixel_size_deg, fov_h, fov_w, *pos, *aim, renders, _ptr(img),
                               C.byref(nx), C.byref(ny))
        assert rc == 0
        return img
