"""The fused forward step (one launch per time step, double-buffered state)
against the two TMA passes per step it replaces: bit-for-bit equal.

The fused kernel runs the two passes' statements in the same order on the
same values, so seismograms, misfits, final wavefields, energies and
gradients must be identical -- over orders 2-8, with and without a free
surface, on grids whose width is below, at and above one 120-column strip and
not a multiple of it, on short grids of one or two 16-row chunks, with full
(sub-sampled) storage, binomial checkpointing (the copy-free plan moving the
state between two working buffers and the slots), the random-boundary
strategy, several shots per launch and wavefield snapshots.  fdorder 10 and
12 (whose stages do not fit shared memory) keep the two passes.
"""
import numpy as np
import pytest

from cuda_fwi_gb300 import problem as P
from cuda_fwi_gb300.engine import Engine
from oracle import oracle as O

pytestmark = pytest.mark.gpu

FUSED, TWO_PASS = 512, 256


def _case(order, nx, nz, nt, fsurf=0, nshots=1, fwi=(1, 1, 1), npml=8, seed=0):
    kw = dict(fdorder=order, nx=nx, nz=nz, nt=nt, npml=npml, fsurf=fsurf, nshots=nshots, nrec=5, perturb=0.05,
              fwi=fwi)
    p, t = P.small(seed=seed, **kw), P.small(seed=seed + 50, **kw)
    obs = np.zeros((p.nrec, p.nt))
    for s in range(nshots):
        rows = O.shot_rows(t, s)
        obs[rows] = O.forward(t, s)["rec"][rows]
    return p, obs


def _run(p, obs, bx, strategy, snapshots=0, snap_interval=0):
    with Engine(p) as eng:
        eng.set_exec(True, bx, 0)
        eng.set_strategy(strategy, snapshots=snapshots)
        if snap_interval:
            eng.set_snapshots(snap_interval)
        shots = list(range(p.nshots))
        rec, mis = eng.forward(shots, obs, keep=True)
        launches = eng.stats()["launches"]  # of the forward sweep
        w = eng.wavefield(0, p.nshots - 1)
        ws, _ = eng.energy(p.nshots - 1)
        snaps = eng.snapshot(p.nshots - 1, 1) if snap_interval else None
        g = eng.backward()
        _, wr = eng.energy(0)
    return dict(rec=rec, mis=mis, w=w, ws=ws, g=g, wr=wr, snaps=snaps, launches=launches)


def _assert_equal(a, b):
    assert np.array_equal(a["rec"], b["rec"])
    assert np.array_equal(a["mis"], b["mis"])
    for k in a["w"]:
        assert np.array_equal(a["w"][k], b["w"][k]), k
    assert np.array_equal(a["ws"], b["ws"]) and np.array_equal(a["wr"], b["wr"])
    for i in range(3):
        assert np.array_equal(a["g"][i], b["g"][i]), i
    if a["snaps"] is not None:
        assert np.array_equal(a["snaps"], b["snaps"])


@pytest.mark.parametrize("order,nx,nz,fsurf", [
    (8, 300, 100, 0),   # 3 strips (the last partial), CPML all round
    (8, 52, 40, 1),     # narrower than one strip, free surface
    (4, 226, 30, 0),    # 2 strips, one 16-row chunk of interior rows
    (2, 119, 57, 1),    # order 2, width one short of a strip boundary
    (6, 150, 70, 0),    # odd half order
    (4, 240, 90, 1),
])
@pytest.mark.parametrize("strategy", ["full", "binomial"])
def test_fused_step_equals_two_passes(order, nx, nz, fsurf, strategy):
    p, obs = _case(order, nx, nz, 130, fsurf=fsurf, fwi=(2, 1, 2) if strategy == "full" else (1, 1, 1))
    a = _run(p, obs, FUSED, strategy, snapshots=6)
    b = _run(p, obs, TWO_PASS, strategy, snapshots=6)
    _assert_equal(a, b)
    assert a["launches"] < b["launches"]  # one stencil launch per forward step instead of two


def test_fused_step_batched_shots_and_snapshots():
    p, obs = _case(8, 180, 60, 110, nshots=3, seed=4)
    a = _run(p, obs, FUSED, "binomial", snapshots=5, snap_interval=25)
    b = _run(p, obs, TWO_PASS, "binomial", snapshots=5, snap_interval=25)
    _assert_equal(a, b)


def test_fused_step_random_boundary():
    p, obs = _case(8, 130, 50, 100, npml=10, seed=6)
    a = _run(p, obs, FUSED, "random")
    b = _run(p, obs, TWO_PASS, "random")
    _assert_equal(a, b)


def test_orders_above_8_keep_the_two_passes():
    p, obs = _case(12, 70, 40, 80, seed=7)
    a = _run(p, obs, FUSED, "binomial", snapshots=4)
    b = _run(p, obs, TWO_PASS, "binomial", snapshots=4)
    _assert_equal(a, b)
    assert a["launches"] == b["launches"]
