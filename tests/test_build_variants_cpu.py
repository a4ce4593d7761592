"""Build variants compile without a GPU (nvcc cross-compiles for sm_103a).

The bounds-checked debug build (-DFWI_BOUNDS_CHECK=1) takes code paths the
normal build leaves out; compiling it here catches a break before a GPU host
runs it (tests/test_gpu_bounds_check.py).  The library is built into a
temporary directory and only checked for the C ABI's entry points.
"""
import os
import shutil
import subprocess

import pytest

from cuda_fwi_gb300 import _capi
from cuda_fwi_gb300 import build as B


@pytest.mark.skipif(not os.path.exists(B.nvcc()), reason="nvcc not found")
def test_bounds_checked_build_compiles(tmp_path):
    lib = B.build(defines=["FWI_BOUNDS_CHECK=1"], out=tmp_path / "libfwi_psv_checked.so")
    assert lib.exists()
    nm = shutil.which("nm")
    if nm:
        out = subprocess.run([nm, "-D", "--defined-only", str(lib)], capture_output=True, text=True).stdout
        missing = [s for s in _capi.exported_symbols() if s not in out]
        assert not missing, missing
