import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def birp():
    """The product library, initialised on cuda:0 (GPU tests only)."""
    import birp_cpp_gb300 as B
    from birp_cpp_gb300 import build
    build.build()
    B.init(0)
    yield B


@pytest.fixture(scope="session")
def golden():
    import json
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        meta = json.load(f)
    return dict(meta=meta,
                cmem=np.load(os.path.join(GOLDEN, "cmem_samples.npz")),
                cube=np.load(os.path.join(GOLDEN, "cube_samples.npz")),
                renders=np.load(os.path.join(GOLDEN, "renders.npz")))


def rel_err(img, ref, floor=1e-3):
    """max and RMS relative error on pixels above floor * max|ref|."""
    img = np.asarray(img, np.float64)
    ref = np.asarray(ref, np.float64)
    m = np.abs(ref) > floor * np.abs(ref).max() if np.abs(ref).max() > 0 else np.zeros(ref.shape, bool)
    if not m.any():
        return 0.0, 0.0, 0
    r = np.abs(img[m] - ref[m]) / np.abs(ref[m])
    return float(r.max()), float(np.sqrt(np.mean(r * r))), int(m.sum())
