"""Regenerates the arctangent polynomial of the CMEM kernel's atan2_pos
(birp_cpp_gb300/csrc/render.cu).

atan(a) on a in [0, 1] is approximated as a * P(a^2) with P of degree 8. The
coefficients minimise the largest absolute error on 4000 Chebyshev nodes of
s = a^2 in [0, 1], found by Lawson's algorithm (iteratively reweighted least
squares: each pass solves a weighted least-squares fit and multiplies every
node's weight by its absolute error, which converges to the minimax
polynomial), computed in FP64 and rounded once to FP32. Run as a script it
prints the kernel's lines; tests/test_fastmath_fit.py checks that render.cu
holds exactly these values.

    python tests/fit_atan2.py
"""
from __future__ import annotations

import numpy as np

DEGREE = 8
NODES = 4000
PASSES = 4000  # the FP32-rounded coefficients are stable from ~3000 passes on


def fit(degree: int = DEGREE, nodes: int = NODES, passes: int = PASSES) -> np.ndarray:
    """FP64 coefficients c_0..c_degree of P (atan(a) ~ a * sum c_j a^(2j))."""
    k = np.arange(nodes)
    s = 0.5 - 0.5 * np.cos((2 * k + 1) * np.pi / (2 * nodes))  # Chebyshev nodes on [0, 1]
    a = np.sqrt(s)
    target = np.arctan(a)
    basis = np.stack([a * s ** j for j in range(degree + 1)], 1)
    w = np.full(nodes, 1.0 / nodes)
    c = None
    for _ in range(passes):
        sw = np.sqrt(w)
        c, *_ = np.linalg.lstsq(basis * sw[:, None], target * sw, rcond=None)
        w = w * np.abs(basis @ c - target)
        w /= w.sum()
    return c


def kernel_coefficients() -> list[np.float32]:
    """The FP32 coefficients in the kernel's Horner order (highest first)."""
    return [np.float32(x) for x in fit()[::-1]]


def fp32_max_error(coef) -> float:
    """Largest |a P(a^2) - atan(a)| over a fine grid of a in [0, 1], with the
    polynomial evaluated in FP32 by Horner's rule as the kernel does."""
    a = np.linspace(0.0, 1.0, 400001).astype(np.float32)
    s = a * a
    p = np.full_like(a, coef[0])
    for c in coef[1:]:
        p = (p * s + np.float32(c)).astype(np.float32)
    return float(np.abs((a * p).astype(np.float64) - np.arctan(a.astype(np.float64))).max())


def literal(c) -> str:
    """The shortest decimal that reads back as this FP32 value."""
    return np.format_float_positional(np.float32(c), unique=True, trim="-")


def c_lines(coef) -> list[str]:
    lines = [f"  float p = {literal(coef[0])}f;"]
    lines += [f"  p = fmaf(p, s, {literal(c)}f);" for c in coef[1:]]
    return lines


if __name__ == "__main__":
    coef = kernel_coefficients()
    print("\n".join(c_lines(coef)))
    print(f"// largest error evaluated in FP32: {fp32_max_error(coef):.3g} rad")
