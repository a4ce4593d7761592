"""Random-boundary reconstruction (FWI_STORE_RANDOM, experimental) against the FP64 oracle.

The engine takes the residual from the absorbing forward and rebuilds the
random-frame forward wavefield backwards in time; the oracle computes the
reference gradient from the stored wavefield of the frame forward
(oracle/random_boundary.py), here driven by the engine's own residual (its
FP32 syn - obs), so that the comparison measures the reconstruction and the
adjoint, not the conditioning of the gradient with respect to the FP32
seismograms.  Bounds: 1e-4 at nt 220; at nt 1500 the FP32 time reversal's
drift (also measured directly: the state rebuilt back to step 0, which is
zero in exact arithmetic) is reported and bounded.
"""
import numpy as np
import pytest

from conftest import engine_residual, rel_l2
from cuda_fwi_gb300 import _capi
from cuda_fwi_gb300 import problem as P
from cuda_fwi_gb300.engine import Engine
from oracle import oracle as O
from oracle import random_boundary as RB

pytestmark = pytest.mark.gpu


def _case(order, nshots=1, nt=220, fwi=(1, 1, 1)):
    kw = dict(fdorder=order, nx=56, nz=40, nt=nt, npml=10, nshots=nshots, nrec=7, perturb=0.05, fwi=fwi)
    p = P.small(seed=5, **kw)
    t = P.small(seed=15, **kw)
    obs = np.zeros((p.nrec, p.nt))
    for s in range(nshots):
        rows = O.shot_rows(t, s)
        obs[rows] = O.forward(t, s)["rec"][rows]
    return p, obs


@pytest.mark.parametrize("order,fwi", [(2, (1, 1, 1)), (4, (2, 1, 1)), (8, (1, 2, 2))])
def test_random_boundary_matches_oracle(order, fwi):
    p, obs = _case(order, fwi=fwi)
    with Engine(p) as eng:
        eng.set_strategy("random")
        rec, mis = eng.forward([0], obs, keep=True)
        g = eng.backward()
        st = eng.stats()
    J, g_o = RB.gradient(p, obs, 0, residual=engine_residual(rec, obs, O.shot_rows(p, 0)))
    assert mis[0] == pytest.approx(J, rel=1e-4)
    errs = [rel_l2(g[i][0], g_o[i]) for i in range(3)]
    print(f"random boundary, order {order}, nt {p.nt}: gradient rel L2 " + " ".join(f"{e:.2e}" for e in errs))
    for i in range(3):
        assert errs[i] <= 1e-4, i
    assert st["recompute_steps"] == 2 * p.nt


def test_random_boundary_long_record_drift():
    """nt 1500 on a small grid (order 8): the gradient against the oracle's,
    and the drift of the time reversal -- the frame state rebuilt back to
    step 0, which is zero in exact arithmetic, relative to the state at the
    end of the frame forward."""
    kw = dict(fdorder=8, nx=80, nz=60, nt=1500, npml=10, nrec=9, perturb=0.05)
    p, t = P.small(seed=5, **kw), P.small(seed=15, **kw)
    obs = O.forward(t, 0)["rec"]
    with Engine(p) as eng:
        eng.set_strategy("random")
        rec, mis = eng.forward([0], obs, keep=True)
        w_end = eng.wavefield(0)
        g = eng.backward()
        w_0 = eng.wavefield(0)
    J, g_o = RB.gradient(p, obs, 0, residual=engine_residual(rec, obs, O.shot_rows(p, 0)))
    errs = [rel_l2(g[i][0], g_o[i]) for i in range(3)]
    n_end = np.sqrt(sum(np.sum(w_end[k] ** 2) for k in w_end))
    drift = np.sqrt(sum(np.sum(w_0[k] ** 2) for k in w_0)) / n_end
    print(f"random boundary, order 8, nt 1500: gradient rel L2 " + " ".join(f"{e:.2e}" for e in errs) +
          f"; state rebuilt to step 0 / final state {drift:.2e}")
    assert drift <= 1e-3
    for i in range(3):
        assert errs[i] <= 1e-2, i


def test_random_boundary_batched_gradient_and_cost():
    p, obs = _case(8, nshots=3)
    ref = [np.zeros((p.nfz, p.nfx)) for _ in range(3)]
    for s in range(3):
        _, g = RB.gradient(p, obs, s)
        for i in range(3):
            ref[i] += g[i]
    with Engine(p) as eng:
        eng.set_strategy("random")
        g, mis = eng.gradient([0, 1, 2], obs)
        st = eng.stats()
        # the CPML gradient of the same shots: same structure, different boundary model
        eng.set_strategy("binomial", snapshots=8)
        gb, _ = eng.gradient([0, 1, 2], obs)
    for i in range(3):
        assert rel_l2(g[i], ref[i]) <= 1e-3, i
    assert st["device_bytes"] > 0
    # close to the absorbing-boundary gradient: same residual, the source
    # wavefield differs by what the random frame scatters back
    for i in range(3):
        assert rel_l2(g[i], gb[i]) <= 0.5, i


def test_random_boundary_refusals():
    p, obs = _case(4, nt=40)
    with Engine(p) as eng:
        eng.set_strategy("random")
        eng.set_exec(True, 64, 0)  # vectorised cells: no reverse step there
        with pytest.raises(_capi.FwiError) as e:
            eng.forward([0], obs, keep=True)
        assert e.value.code == "FWI_ERR_UNSUPPORTED"
    q = P.small(fdorder=4, nx=40, nz=30, nt=40, npml=6, fsurf=1, nrec=4)
    with Engine(q) as eng:
        eng.set_strategy("random")
        with pytest.raises(_capi.FwiError) as e:
            eng.forward([0], np.zeros((q.nrec, q.nt)), keep=True)
        assert e.value.code == "FWI_ERR_UNSUPPORTED"
