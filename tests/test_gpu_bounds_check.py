"""The bounds-checked debug build (-DFWI_BOUNDS_CHECK=1) on valid inputs.

compute-sanitizer is not available on every GPU host; in the checked build the
TMA-staged passes and the fused step guard their global-memory accesses
(fields, CPML memories, gradients, storage; see `inb` in
csrc/fwi_kernels.cuh), recording the first
out-of-range access, skipping it, and making the call fail.  On these valid
cases the checked library must record nothing and give the normal library's
results bit for bit (the guards change no arithmetic).  Only valid inputs run
here: no access is expected to be out of range.
"""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from cuda_fwi_gb300 import _capi
from cuda_fwi_gb300 import build as B

pytestmark = pytest.mark.gpu

HERE = Path(__file__).resolve().parent


@pytest.fixture(scope="module")
def checked_lib(tmp_path_factory):
    return B.build(defines=["FWI_BOUNDS_CHECK=1"], out=tmp_path_factory.mktemp("chk") / "libfwi_psv_checked.so")


def _run(lib, out):
    env = dict(os.environ, FWI_PSV_LIB=str(lib))
    r = subprocess.run([sys.executable, str(HERE / "_bounds_cases.py"), str(out)], env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return np.load(out)


def test_checked_build_records_nothing_and_matches(checked_lib, tmp_path):
    want = _run(_capi.LIB_PATH, tmp_path / "normal.npz")
    got = _run(checked_lib, tmp_path / "checked.npz")
    assert sorted(got.files) == sorted(want.files) and len(want.files) == 3 * 3 * 5 + 1 + 3 * 3
    for k in want.files:
        assert np.array_equal(got[k], want[k]), k
