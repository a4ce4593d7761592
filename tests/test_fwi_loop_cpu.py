"""Host logic of the FWI optimiser against its restatement (CPU, no GPU).

* fwi_psv_calc_opt_step is bit-identical to the oracle's restatement of
  calc_opt_step + solvelin (float multiplier and accumulator kept).
* fwi_psv_step_search walks the reference's state machine
  (fwi_step_length_estimation.cu:46-223) exactly like the restatement in
  oracle/fwi_loop.py: same trial steps in the same order, same number of
  trials, status and optimum, on misfit curves that take each branch.
"""
import ctypes as C

import numpy as np
import pytest

from cuda_fwi_gb300 import _capi
from oracle import fwi_loop as FL


def test_calc_opt_step_bit_identical():
    rng = np.random.default_rng(0)
    L = _capi.lib()
    for _ in range(200):
        sl = np.sort(rng.uniform(0.0, 0.05, 3))
        sl[0] = 0.0
        L2 = 1.0 + rng.uniform(-0.5, 0.5, 3)
        got = L.fwi_psv_calc_opt_step(_capi.pd(L2), _capi.pd(sl))
        assert got == FL.calc_opt_step(L2, sl)


def _c_search(est, L2_0, f):
    tried = []

    @_capi.TRIAL_FN
    def trial(ctx, step, out):
        tried.append(step)
        out[0] = f(step)
        return 0

    opt = C.c_double()
    trials = C.c_int()
    status = C.c_int()
    st = _capi.lib().fwi_psv_step_search(est, L2_0, trial, None, C.byref(opt), C.byref(trials), C.byref(status))
    _capi.check(st, "step_search")
    return opt.value, trials.value, status.value, tried


CURVES = {
    "bracketed": (0.01, lambda s: (s - 0.03) ** 2 + 1.0),
    "minimum below the first step": (0.01, lambda s: (s - 0.001) ** 2 + 2.0),
    "misfit never reduced": (0.01, lambda s: 1.0 + s),
    "minimum never bracketed": (0.01, lambda s: 1.0 - s),
    "flat then rising": (0.02, lambda s: 5.0 + max(0.0, s - 0.05) ** 2 - 1e-4 * s),
}


@pytest.mark.parametrize("name", list(CURVES))
def test_step_search_follows_the_reference_state_machine(name):
    est, f = CURVES[name]
    L2_0 = f(0.0)
    want = FL.step_search(est, L2_0, f)
    got = _c_search(est, L2_0, f)
    assert got[3] == want[3]            # same trial steps, same order
    assert got[1:3] == want[1:3]        # trials, status
    assert got[0] == want[0]            # optimum (bit-identical fit)


def test_step_search_statuses():
    assert _c_search(0.01, 1.0, lambda s: 1.0 + s)[2] == 1
    assert _c_search(0.01, 1.0, lambda s: 1.0 - s)[2] == 2
    opt, _, st, _ = _c_search(0.01, 1.0009, lambda s: (s - 0.03) ** 2 + 1.0)
    assert st == 0 and opt == pytest.approx(0.03, rel=1e-3)


def test_trial_error_propagates():
    @_capi.TRIAL_FN
    def bad(ctx, step, out):
        return -1

    opt = C.c_double()
    st = _capi.lib().fwi_psv_step_search(0.01, 1.0, bad, None, C.byref(opt), None, None)
    assert st == -1
