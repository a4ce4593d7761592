import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU oracle case")


@pytest.fixture(scope="session", autouse=True)
def _built():
    import __graft_entry__ as g
    g.build()


def rel_l2(a, b):
    import numpy as np
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


@pytest.fixture
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return 0


def engine_residual(rec, obs, rows):
    """The engine's adjoint source for traces `rec` (its FP32 seismograms): FP32
    synthetics minus FP32 observed data, differenced in FP64 and rounded to
    FP32 (residual_kernel); zero outside `rows`."""
    import numpy as np
    r = np.zeros_like(np.asarray(obs, np.float64))
    o32 = np.asarray(obs, np.float64)[rows].astype(np.float32).astype(np.float64)
    r[rows] = (np.asarray(rec, np.float64)[rows] - o32).astype(np.float32)
    return r
