"""The arctangent polynomial of the CMEM kernel (atan2_pos in
birp_cpp_gb300/csrc/render.cu) is exactly what tests/fit_atan2.py computes:
the FP32-rounded minimax fit, coefficient for coefficient."""
import os
import re
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "tests"))


def kernel_literals():
    src = open(os.path.join(ROOT, "birp_cpp_gb300", "csrc", "render.cu")).read()
    body = src[src.index("__device__ __forceinline__ float atan2_pos"):]
    body = body[:body.index("\n}\n")]
    first = re.search(r"float p = ([-0-9.e]+)f;", body).group(1)
    rest = re.findall(r"p = fmaf\(p, s, ([-0-9.e]+)f\);", body)
    return [np.float32(first)] + [np.float32(v) for v in rest]


def test_kernel_holds_the_fit():
    import fit_atan2
    fitted = fit_atan2.kernel_coefficients()
    lits = kernel_literals()
    assert len(lits) == fit_atan2.DEGREE + 1
    assert [float(x) for x in lits] == [float(x) for x in fitted]
    # and the polynomial is as accurate as stated beside it
    assert fit_atan2.fp32_max_error(lits) < 1.0e-7
