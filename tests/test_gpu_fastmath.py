"""The CMEM kernel's fast functions (birp_cpp_gb300/csrc/render.cu) against
the true values (FP64 on the host) and against CUDA's own atan2f / powf /
sqrtf / exp2f at the same FP32 arguments, on dense grids over the argument
ranges the CMEM model gives them. The bounds asserted are the ones the
kernel's FP32 shell decisions are budgeted with (its margin is checked
separately by birp_cmem_margin_check):
  atan2_pos   <= 4e-7 rad absolute (degree-8 minimax polynomial, 9.8e-8 rad;
              the hardware-reciprocal division of min/max; the FP32 pi/2
              and pi it is subtracted from and that last rounding)
  sqrt_fast   <= 3 ulp relative (x * rsqrt.approx)
  ex2_fast    <= 2 ulp relative (ex2.approx.ftz)
  pow_pos     relative error <= 5e-7 + 2.5e-7 |y log2 x| + 1.7e-7 |y|
              (ex2.approx of y * log2.approx(x): the log's relative error
              grows with the result's exponent, and near x = 1 its absolute
              error, about 2^-22.5, is scaled by y)"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ULP = 2.0 ** -23


def _grid2(a, b):
    A, Bv = np.meshgrid(a, b, indexing="ij")
    return A.ravel().astype(np.float32), Bv.ravel().astype(np.float32)


def test_atan2_pos(birp):
    # sample-direction angles: y = r_yz >= 0 (0 included) and any x; cusp
    # angles: |u x n| and u . n of unit vectors
    ys = np.concatenate([[0.0, 1e-6, 1e-3], np.linspace(0.0, 60.0, 1201)[1:]])
    xs = np.concatenate([np.linspace(-60.0, 60.0, 1201), [-1e-6, 1e-6]])
    x, y = _grid2(xs, ys)
    t = np.linspace(0.0, np.pi, 200001)
    x = np.concatenate([x, np.cos(t).astype(np.float32)])
    y = np.concatenate([y, np.abs(np.sin(t)).astype(np.float32)])
    keep = (x != 0) | (y != 0)
    x, y = x[keep], y[keep]
    fast, lib = birp.fastmath_check(0, x, y)
    true = np.arctan2(y.astype(np.float64), x.astype(np.float64))
    err = np.abs(fast - true)
    assert err.max() <= 4e-7, (err.max(), x[err.argmax()], y[err.argmax()])
    assert np.abs(fast.astype(np.float64) - lib).max() <= 4.5e-7
    assert fast.min() >= 0.0 and fast.max() <= np.float32(np.pi) + 4e-7


def test_sqrt_fast(birp):
    x = np.concatenate([[0.0], np.geomspace(1e-12, 1e5, 400001)]).astype(np.float32)
    fast, lib = birp.fastmath_check(2, x)
    assert fast[0] == 0.0
    true = np.sqrt(x[1:].astype(np.float64))
    rel = np.abs(fast[1:] - true) / true
    assert rel.max() <= 3 * ULP, rel.max()
    assert np.all(lib[1:] == np.sqrt(x[1:]))  # sqrtf is correctly rounded


def test_ex2_fast(birp):
    x = np.linspace(-40.0, 20.0, 600001).astype(np.float32)
    fast, lib = birp.fastmath_check(3, x)
    true = np.exp2(x.astype(np.float64))
    rel = np.abs(fast - true) / true
    assert rel.max() <= 2 * ULP, rel.max()


def test_pow_pos(birp):
    # bases: the magnetopause base (~0.3-1.5), cusp angles (0-pi], r/10
    # (0.01-10); exponents: the model's (-6..6)
    a = np.concatenate([np.geomspace(1e-3, 20.0, 1501), np.linspace(0.25, 1.6, 500)])
    b = np.linspace(-6.0, 6.0, 601)
    x, y = _grid2(a, b)
    fast, lib = birp.fastmath_check(1, x, y)
    true = np.power(x.astype(np.float64), y.astype(np.float64))
    bound = 5e-7 + 2.5e-7 * np.abs(y * np.log2(x.astype(np.float64))) + 1.7e-7 * np.abs(y)
    rel = np.abs(fast - true) / true
    worst = int(np.argmax(rel / bound))
    assert np.all(rel <= bound), (rel[worst], bound[worst], x[worst], y[worst])
    rel_lib = np.abs(fast.astype(np.float64) - lib) / np.abs(lib)
    assert np.all(rel_lib <= bound + 2 * ULP)
