"""GB300-native BIRP render path: Python binding of the C ABI
(include/birp_gb300.h) used by the tests and the benchmark.

The library is built in-tree by birp_cpp_gb300/build.py. There is no CPU
fallback: importing the binding without the built library raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# BIRP_LIB selects another build of the library (the bounds-checking
# lib/libbirp_gb300_debug.so, say)
LIB_PATH = os.environ.get("BIRP_LIB") or os.path.join(HERE, "lib", "libbirp_gb300.so")
HEADER = os.path.join(HERE, "..", "include", "birp_gb300.h")

OK, ERR_INVALID, ERR_CUDA, ERR_NOMEM, ERR_SINGULAR, ERR_NOT_INIT, ERR_TIMEOUT, ERR_BUSY, ERR_DEVICE = range(9)
PREFIX, CLIP = 0, 1


class BirpError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"birp status {status}: {msg}")
        self.status = status


class Camera(C.Structure):
    _fields_ = [("pos", C.c_double * 3), ("aim", C.c_double * 3), ("fov_w_deg", C.c_double),
                ("fov_h_deg", C.c_double), ("nx", C.c_int), ("ny", C.c_int), ("n_samples", C.c_int),
                ("ray_length", C.c_double), ("trilinear", C.c_int), ("march", C.c_int),
                ("segments", C.c_int), ("roll_deg", C.c_double), ("warp_rays_x", C.c_int),
                ("tile_warps_x", C.c_int)]


class CmemParams(C.Structure):
    _fields_ = [("has_v", C.c_int), ("v", C.c_int * 3), ("has_b", C.c_int), ("b", C.c_int * 3),
                ("dipole", C.c_float), ("p0", C.c_float), ("p1", C.c_int), ("p2", C.c_int),
                ("p3", C.c_int), ("B", C.c_float), ("alpha", C.c_float), ("beta", C.c_float),
                ("bs", C.c_float), ("A1", C.c_float), ("A2", C.c_float), ("ay_bs", C.c_float),
                ("az_bs", C.c_float), ("density", C.c_float)]


class Request(C.Structure):
    _fields_ = [("cube", C.c_void_p), ("cmem", C.c_void_p), ("cam", Camera)]


CUBE_RECORDS, CUBE_COMPACT, CUBE_PAIRS = 0, 1, 2  # device layouts of a cube (birp_cube_create_layout)


class CubeInfo(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("uniform", C.c_int * 3),
                ("device_bytes", C.c_size_t), ("layout", C.c_int)]


class ServerConfig(C.Structure):
    _fields_ = [("cube_budget_bytes", C.c_int64), ("slots", C.c_int), ("max_batch_requests", C.c_int),
                ("max_batch_pixels", C.c_int64), ("max_queue", C.c_int), ("max_wait_ms", C.c_double),
                ("cube_layout", C.c_int), ("promoted_layout", C.c_int), ("promoted_budget_bytes", C.c_int64),
                ("uploaders", C.c_int)]


class Result(C.Structure):
    _fields_ = [("ticket", C.c_int64), ("status", C.c_int), ("latency_ms", C.c_double),
                ("queue_ms", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("submitted", "completed", "rejected", "batches", "cube_uploads",
                                         "cube_evictions", "cube_hits", "resident_bytes", "cube_promotions",
                                         "promoted_bytes")]


class KernelStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("exact_range_rays", "exact_nearest", "exact_cmem", "items", "samples",
                                          "cells")]


_lib = None


def lib():
    """The loaded C ABI library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with birp_cpp_gb300/build.py "
                              "(there is no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        P, I, D, F = C.c_void_p, C.c_int, C.c_double, C.c_float
        sig = {
            "birp_version": ([], I),
            "birp_init": ([I], I),
            "birp_shutdown": ([], None),
            "birp_last_error": ([], C.c_char_p),
            "birp_cube_create": ([P, I, P, I, P, I, P, P], I),
            "birp_cube_create_layout": ([P, I, P, I, P, I, P, I, P], I),
            "birp_cube_destroy": ([P], I),
            "birp_cube_get_info": ([P, P], I),
            "birp_cube_sample": ([P, I, P, I, P], I),
            "birp_cmem_default_params": ([P], None),
            "birp_cmem_create": ([P, P], I),
            "birp_cmem_destroy": ([P], I),
            "birp_cmem_sample": ([P, P, I, P], I),
            "birp_camera_defaults": ([P], None),
            "birp_render": ([P, P, P, P, P], I),
            "birp_render_device": ([P, P, P, P, P], I),
            "birp_camera_frame": ([P, P, P, P, P, P, P, P], I),
            "birp_batch_create": ([I, C.c_int64, P], I),
            "birp_batch_destroy": ([P], I),
            "birp_batch_submit": ([P, P, I], I),
            "birp_batch_wait": ([P], I),
            "birp_batch_image": ([P, I], C.POINTER(C.c_float)),
            "birp_batch_render": ([P, P, I, P], I),
            "birp_batch_last_ms": ([P, P, P], I),
            "birp_batch_upload_bytes": ([P, P], I),
            "birp_debug_bounds": ([P, I], I),
            "birp_server_default_config": ([P], None),
            "birp_server_create": ([P, P], I),
            "birp_server_destroy": ([P], I),
            "birp_server_add_cube": ([P, P, I, P, I, P, I, P, P], I),
            "birp_server_add_cmem": ([P, P, P], I),
            "birp_server_submit": ([P, I, P, P, P], I),
            "birp_server_wait": ([P, C.c_int64, D, P], I),
            "birp_server_get_stats": ([P, P], I),
            "birp_get_kernel_stats": ([P, I], I),
            "birp_time_render_device": ([P, P, P, P, I, I, P], I),
            "birp_cmem_margin_check": ([P, I, P, P], I),
            "birp_flush_l2": ([], I),
            "birp_measure_peaks": ([P, P, P], I),
            "birp_fastmath_check": ([I, P, P, I, P, P], I),
        }
        for name, (args, res) in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != OK:
        raise BirpError(status, lib().birp_last_error().decode())


def _p(a: np.ndarray) -> int:
    return a.ctypes.data


def init(device: int = 0) -> None:
    check(lib().birp_init(device))


def shutdown() -> None:
    lib().birp_shutdown()


def camera(pos, aim, fov_w, fov_h, nx, ny, n_samples=200, ray_length=44.0, trilinear=True, march=PREFIX,
           segments=0, roll=0.0, warp_rays_x=0, tile_warps_x=0) -> Camera:
    c = Camera()
    for i in range(3):
        c.pos[i] = float(pos[i])
        c.aim[i] = float(aim[i])
    c.fov_w_deg, c.fov_h_deg, c.nx, c.ny = float(fov_w), float(fov_h), int(nx), int(ny)
    c.n_samples, c.ray_length = int(n_samples), float(ray_length)
    c.trilinear, c.march, c.segments = int(bool(trilinear)), int(march), int(segments)
    c.roll_deg = float(roll)
    c.warp_rays_x, c.tile_warps_x = int(warp_rays_x), int(tile_warps_x)
    return c


def camera_defaults() -> Camera:
    c = Camera()
    lib().birp_camera_defaults(C.byref(c))
    return c


class Cube:
    """A DataCube resident in GPU memory (birp_cube_create_layout; layout
    CUBE_RECORDS, the fastest, CUBE_PAIRS, about 1/4 of its memory, or
    CUBE_COMPACT, about 1/8)."""

    def __init__(self, xs, ys, zs, values, layout: int = CUBE_RECORDS):
        xs = np.ascontiguousarray(xs, np.float64)
        ys = np.ascontiguousarray(ys, np.float64)
        zs = np.ascontiguousarray(zs, np.float64)
        v = np.ascontiguousarray(values, np.float32)
        if v.shape != (len(zs), len(ys), len(xs)):
            raise ValueError(f"values shape {v.shape} != (nz, ny, nx) = {(len(zs), len(ys), len(xs))}")
        h = C.c_void_p()
        check(lib().birp_cube_create_layout(_p(xs), len(xs), _p(ys), len(ys), _p(zs), len(zs), _p(v), int(layout),
                                            C.byref(h)))
        self.h = h
        self.shape = v.shape

    def info(self) -> CubeInfo:
        i = CubeInfo()
        check(lib().birp_cube_get_info(self.h, C.byref(i)))
        return i

    def sample(self, pts, trilinear=True) -> np.ndarray:
        p = np.ascontiguousarray(pts, np.float32).reshape(-1, 3)
        out = np.empty(len(p), np.float32)
        check(lib().birp_cube_sample(self.h, int(bool(trilinear)), _p(p), len(p), _p(out)))
        return out

    def close(self):
        if self.h:
            check(lib().birp_cube_destroy(self.h))
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def cmem_params(**kw) -> CmemParams:
    """CMEM::Init arguments: the reference defaults overridden by kw (v, b are
    3-sequences; the rest scalars, 0 meaning unset as in the reference)."""
    p = CmemParams()
    lib().birp_cmem_default_params(C.byref(p))
    for k, val in kw.items():
        if k in ("v", "b"):
            setattr(p, "has_" + k, int(val is not None))
            if val is not None:
                arr = getattr(p, k)
                for i in range(3):
                    arr[i] = int(val[i])
        else:
            setattr(p, k, val)
    return p


class Cmem:
    """The CMEM analytic emissivity model on the GPU (birp_cmem_create)."""

    def __init__(self, params: CmemParams | None = None):
        self.params = params if params is not None else cmem_params()
        h = C.c_void_p()
        check(lib().birp_cmem_create(C.byref(self.params), C.byref(h)))
        self.h = h

    def sample(self, pts) -> np.ndarray:
        p = np.ascontiguousarray(pts, np.float32).reshape(-1, 3)
        out = np.empty(len(p), np.float32)
        check(lib().birp_cmem_sample(self.h, _p(p), len(p), _p(out)))
        return out

    def margin_check(self, n=1 << 20):
        err, margin = C.c_float(), C.c_float()
        check(lib().birp_cmem_margin_check(self.h, n, C.byref(err), C.byref(margin)))
        return err.value, margin.value

    def close(self):
        if self.h:
            check(lib().birp_cmem_destroy(self.h))
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _src(space):
    if isinstance(space, Cube):
        return space.h, None
    if isinstance(space, Cmem):
        return None, space.h
    raise TypeError("space must be a Cube or a Cmem")


def render(space, cam: Camera, out: np.ndarray | None = None) -> np.ndarray:
    """Plain per-call render into a host array (birp_render)."""
    img = np.empty((cam.ny, cam.nx), np.float32) if out is None else out
    cb, cm = _src(space)
    check(lib().birp_render(cb, cm, C.byref(cam), _p(img), None))
    return img


def camera_frame(cam: Camera) -> dict:
    rinv = np.zeros(9, np.float64)
    vals = [C.c_double() for _ in range(6)]
    check(lib().birp_camera_frame(C.byref(cam), _p(rinv), *[C.byref(v) for v in vals]))
    tfx, tfy, aspect, dt, K, angle = (v.value for v in vals)
    return dict(rinv=rinv.reshape(3, 3), tfx=tfx, tfy=tfy, aspect=aspect, dt=dt, K=K, angle_sun=angle)


def kernel_stats(reset: bool = False) -> dict:
    s = KernelStats()
    check(lib().birp_get_kernel_stats(C.byref(s), int(reset)))
    return {n: getattr(s, n) for n, _ in KernelStats._fields_}


def flush_l2() -> None:
    check(lib().birp_flush_l2())


def fastmath_check(which: int, x, y=None):
    """(fast, library) values of one of the CMEM kernel's fast functions on the
    GPU at the FP32 arguments x (and y): 0 atan2_pos(y, x), 1 pow_pos(x, y),
    2 sqrt_fast(x), 3 ex2_fast(x) (birp_fastmath_check)."""
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(np.zeros_like(x) if y is None else y, np.float32)
    fast, libv = np.empty_like(x), np.empty_like(x)
    check(lib().birp_fastmath_check(int(which), _p(x), _p(y), len(x), _p(fast), _p(libv)))
    return fast, libv


def measure_peaks() -> tuple[float, float, int]:
    """(FP32 TFLOP/s, L2-resident read GB/s, buffer bytes of that read rate)
    measured on this GPU."""
    f, r, n = C.c_double(), C.c_double(), C.c_size_t()
    check(lib().birp_measure_peaks(C.byref(f), C.byref(r), C.byref(n)))
    return f.value, r.value, n.value


class Batch:
    """Many renders in one persistent-kernel launch replayed from a CUDA graph."""

    def __init__(self, max_requests: int, max_pixels: int):
        h = C.c_void_p()
        check(lib().birp_batch_create(int(max_requests), int(max_pixels), C.byref(h)))
        self.h = h

    @staticmethod
    def _reqs(items):
        arr = (Request * len(items))()
        for i, (space, cam) in enumerate(items):
            cb, cm = _src(space)
            arr[i].cube = cb.value if cb is not None else None
            arr[i].cmem = cm.value if cm is not None else None
            arr[i].cam = cam
        return arr

    def render(self, items) -> list[np.ndarray]:
        """items: list of (space, Camera). Returns the images."""
        arr = self._reqs(items)
        outs = [np.empty((cam.ny, cam.nx), np.float32) for _, cam in items]
        ptrs = (C.c_void_p * len(items))(*[o.ctypes.data for o in outs])
        check(lib().birp_batch_render(self.h, arr, len(items), ptrs))
        return outs

    def submit(self, items):
        self._keep = self._reqs(items)
        check(lib().birp_batch_submit(self.h, self._keep, len(items)))

    def wait(self):
        check(lib().birp_batch_wait(self.h))

    def last_ms(self):
        k, t = C.c_float(), C.c_float()
        check(lib().birp_batch_last_ms(self.h, C.byref(k), C.byref(t)))
        return k.value, t.value

    def upload_bytes(self) -> int:
        n = C.c_size_t()
        check(lib().birp_batch_upload_bytes(self.h, C.byref(n)))
        return n.value

    def close(self):
        if self.h:
            check(lib().birp_batch_destroy(self.h))
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def server_config(**kw) -> ServerConfig:
    c = ServerConfig()
    lib().birp_server_default_config(C.byref(c))
    for k, v in kw.items():
        setattr(c, k, v)
    return c


class Server:
    """Continuous-batching render server (birp_server_*)."""

    def __init__(self, cfg: ServerConfig | None = None):
        self.cfg = cfg if cfg is not None else server_config()
        h = C.c_void_p()
        check(lib().birp_server_create(C.byref(self.cfg), C.byref(h)))
        self.h = h

    def add_cube(self, xs, ys, zs, values) -> int:
        xs = np.ascontiguousarray(xs, np.float64)
        ys = np.ascontiguousarray(ys, np.float64)
        zs = np.ascontiguousarray(zs, np.float64)
        v = np.ascontiguousarray(values, np.float32)
        cid = C.c_int()
        check(lib().birp_server_add_cube(self.h, _p(xs), len(xs), _p(ys), len(ys), _p(zs), len(zs), _p(v),
                                         C.byref(cid)))
        return cid.value

    def add_cmem(self, params: CmemParams | None = None) -> int:
        p = params if params is not None else cmem_params()
        sid = C.c_int()
        check(lib().birp_server_add_cmem(self.h, C.byref(p), C.byref(sid)))
        return sid.value

    def submit(self, source: int, cam: Camera, out: np.ndarray) -> int:
        t = C.c_int64()
        check(lib().birp_server_submit(self.h, int(source), C.byref(cam), _p(out), C.byref(t)))
        return t.value

    def wait(self, ticket: int, timeout_ms: float = -1.0) -> Result:
        r = Result()
        st = lib().birp_server_wait(self.h, int(ticket), float(timeout_ms), C.byref(r))
        if st != OK and st != ERR_TIMEOUT:
            r.status = st
            return r
        check(st)
        return r

    def stats(self) -> ServerStats:
        s = ServerStats()
        check(lib().birp_server_get_stats(self.h, C.byref(s)))
        return s

    def close(self):
        if self.h:
            check(lib().birp_server_destroy(self.h))
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def debug_bounds(reset: bool = True) -> int:
    """First out-of-range table access recorded by the bounds-checking build
    (code << 48 | index; 0 if none). Raises BirpError in other builds."""
    st = C.c_ulonglong()
    check(lib().birp_debug_bounds(C.byref(st), int(reset)))
    return st.value

