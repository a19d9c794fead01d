"""The bounds-checking build (BIRP_DEBUG_BOUNDS): every table access of the
render kernels is checked, and the first out-of-range one is recorded
instead of faulting. Every load is in bounds by construction (guard cells,
infinite exit planes, sentinel nodes, clamped start cells); this runs every
kernel class and edge case through that build and requires that nothing was
recorded, with the images still matching the FP64 oracle."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_release_build_is_not_bounds_checking(birp):
    with pytest.raises(birp.BirpError):
        birp.debug_bounds()


def test_every_table_access_in_bounds():
    from birp_cpp_gb300 import build
    lib = build.build_debug_bounds()
    env = dict(os.environ, BIRP_LIB=lib)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "tests", "bounds_run.py")], env=env,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert "status 0x0" in r.stdout
