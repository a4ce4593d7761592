"""Failure detection on the GPU, in the forms that leave the GPU usable.

* A bounded wait that runs out: the engine's test hook makes one CTA of the
  next forward's first TMA-staged step (the fused step, or the two-pass
  step's stress pass, whose warps release their stages without a CTA
  barrier) expect 16 bytes more than its copies deliver; with a 1 ms wait
  limit the kernel gives up, drains its copies and returns, the rest of the
  call's launches return at once, and the forward returns FWI_ERR_CUDA.  The
  same engine then gives the results of a fresh engine, bit for bit.
* Non-finite values: a NaN placed on the host in a source signal (the forward
  wavefield) or in the observed data (the residual) comes back as
  FWI_ERR_DIVERGED from the device watchdog / the residual check, and the
  engine stays usable.
No kernel faults, traps or waits without a bound.
"""
import numpy as np
import pytest

from cuda_fwi_gb300 import _capi
from cuda_fwi_gb300 import problem as P
from cuda_fwi_gb300.engine import Engine
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _case():
    p = P.small(fdorder=8, nx=150, nz=50, nt=120, npml=8, nrec=6, perturb=0.04, seed=8)
    t = P.small(fdorder=8, nx=150, nz=50, nt=120, npml=8, nrec=6, perturb=0.04, seed=18)
    return p, O.forward(t, 0)["rec"]


def _clean(p, obs, bx=0):
    with Engine(p) as eng:
        eng.set_exec(True, bx, 0)
        eng.set_strategy("binomial", snapshots=6)
        rec, mis = eng.forward([0], obs, keep=True)
        g = eng.backward()
    return rec, mis, g


@pytest.mark.parametrize("bx", [512, 256])  # fused step, two-pass step
def test_wait_that_runs_out_returns_error_and_engine_recovers(bx):
    p, obs = _case()
    want = _clean(p, obs, bx=bx)
    with Engine(p) as eng:
        eng.set_strategy("binomial", snapshots=6)
        eng.set_exec(False, bx, 0)  # direct launches
        eng.set_wait_limit(1e-3)
        eng.debug_stall_next()
        with pytest.raises(_capi.FwiError) as ei:
            eng.forward([0], obs, keep=True)
        assert ei.value.code == "FWI_ERR_CUDA" and "timed out" in str(ei.value)
        # the engine stays usable: the next forward and backward are exact
        eng.set_wait_limit(2.0)
        rec, mis = eng.forward([0], obs, keep=True)
        g = eng.backward()
    assert np.array_equal(rec, want[0]) and np.array_equal(mis, want[1])
    for a, b in zip(g, want[2]):
        assert np.array_equal(a, b)


def test_nan_in_source_signal_is_caught_by_the_watchdog():
    p, obs = _case()
    want = _clean(p, obs)
    bad = P.small(fdorder=8, nx=150, nz=50, nt=120, npml=8, nrec=6, perturb=0.04, seed=8)
    bad.src_signal = bad.src_signal.copy()
    bad.src_signal[0, 30] = np.nan
    with Engine(bad) as eng:
        eng.set_strategy("binomial", snapshots=6)
        with pytest.raises(_capi.FwiError) as ei:
            eng.forward([0], None)
        assert ei.value.code == "FWI_ERR_DIVERGED" and "non-finite" in str(ei.value)
        # a clean acquisition on the same engine gives the clean results
        eng.set_sources(p.src_x, p.src_z, p.src_comp, p.src_shot, p.src_signal)
        rec, mis = eng.forward([0], obs, keep=True)
        g = eng.backward()
    assert np.array_equal(rec, want[0]) and np.array_equal(mis, want[1])
    for a, b in zip(g, want[2]):
        assert np.array_equal(a, b)


def test_nan_in_observed_data_is_caught_by_the_residual_check():
    p, obs = _case()
    bad = obs.copy()
    bad[O.shot_rows(p, 0)[2], 50] = np.nan
    with Engine(p) as eng:
        with pytest.raises(_capi.FwiError) as ei:
            eng.forward([0], bad, keep=True)
        assert ei.value.code == "FWI_ERR_DIVERGED"
        rec, mis = eng.forward([0], obs)
    assert np.isfinite(mis).all() and mis[0] > 0
