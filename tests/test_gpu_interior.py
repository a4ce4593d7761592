"""TMA-staged passes on grids with interior cells, against the FP64 oracle.

In the stress and velocity passes of the TMA mapping a warp covers 64 columns
of two rows; a warp whose cells touch no border column, no CPML strip and no
free-surface row, and that takes no storage sample, runs a branch-free row
loop, the others the general one.  The small parity cases fit in one tile
column with strips on both sides, so here the grid is wide and deep enough for
both kinds of warp (the split is recomputed on the host and checked).
Tolerances as in the other parity tests: seismograms 1e-5, gradients 1e-4
relative L2.
"""
import numpy as np
import pytest

from conftest import rel_l2
from cuda_fwi_gb300 import problem as P
from cuda_fwi_gb300.engine import Engine
from oracle import oracle as O
from oracle import random_boundary as RB

pytestmark = pytest.mark.gpu

SEIS_TOL = 1e-5
GRAD_TOL = 1e-4
TX, TZ, WR = 128, 16, 2  # TMA tile of the forward passes; a warp: 64 columns x WR rows


def _warps(p):
    """(interior, total) warp blocks of the forward passes: the kernel's rule restated."""
    fp = p.fdorder // 2
    cxl, cxh, czl, czh = fp, p.nxt - fp - 1, fp, p.nzt - fp - 1
    if p.npml > 0:
        cxl, cxh = max(cxl, p.ppad + 1), min(cxh, p.nxt - p.ppad - 2)
        czh = min(czh, p.nzt - p.ppad - 2)
        if not p.fsurf:
            czl = max(czl, p.ppad + 1)
    if p.fsurf:
        czl = max(czl, 2 * fp + 1)
    nin = ntot = 0
    for x0 in range(0, p.nxt, TX):
        for z0 in range(fp, p.nzt - fp, TZ):
            for wx in (x0, x0 + 64):
                for wz in range(z0, z0 + TZ, WR):
                    nin += wx >= cxl and wx + 63 <= cxh and wz >= czl and wz + WR - 1 <= czh
                    ntot += 1
    return nin, ntot


def _case(order, fsurf, nt=260, fwi=(1, 1, 1), nshots=1):
    kw = dict(fdorder=order, nx=300, nz=100, nt=nt, npml=8, fsurf=fsurf, nshots=nshots, nrec=9,
              perturb=0.05, fwi=fwi)
    p = P.small(seed=21, **kw)
    t = P.small(seed=31, **kw)
    obs = np.zeros((p.nrec, p.nt))
    for s in range(nshots):
        rows = O.shot_rows(t, s)
        obs[rows] = O.forward(t, s)["rec"][rows]
    return p, obs


@pytest.mark.parametrize("order,fsurf", [(4, 0), (8, 0), (8, 1), (12, 1), (2, 0)])
@pytest.mark.parametrize("strategy", ["binomial", "full"])
def test_interior_tiles_match_oracle(order, fsurf, strategy):
    p, obs = _case(order, fsurf)
    nin, ntot = _warps(p)
    assert 0 < nin < ntot
    J, g_o, fw_o, ad_o = O.gradient(p, obs, 0)
    with Engine(p) as eng:
        if strategy == "binomial":
            eng.set_strategy("binomial", snapshots=6)
        rec, mis = eng.forward([0], obs, keep=True)
        g = eng.backward()
        ws, wr = eng.energy(0)
    assert rel_l2(rec[: p.nrec], fw_o["rec"]) <= SEIS_TOL
    assert mis[0] == pytest.approx(J, rel=1e-4)
    for i in range(3):
        assert rel_l2(g[i][0], g_o[i]) <= GRAD_TOL, i
    assert rel_l2(ws, fw_o["We"]) <= GRAD_TOL
    assert rel_l2(wr, ad_o["We"]) <= GRAD_TOL


def test_interior_tiles_agree_with_vectorised_mapping():
    p, obs = _case(8, 0, nt=200, nshots=2)
    out = []
    for bx in (256, 64):
        with Engine(p) as eng:
            eng.set_exec(True, bx, 0)
            eng.set_strategy("binomial", snapshots=5)
            g, mis = eng.gradient([0, 1], obs)
            out.append((g, mis))
    for i in range(3):
        assert rel_l2(out[0][0][i], out[1][0][i]) <= 3e-5, i
    assert out[0][1] == pytest.approx(out[1][1], rel=1e-5)


def test_interior_tiles_random_boundary():
    """The random-frame sweeps (no CPML, time reversal) on interior tiles."""
    p, obs = _case(8, 0, nt=220)
    J, g_o = RB.gradient(p, obs, 0)
    with Engine(p) as eng:
        eng.set_strategy("random")
        rec, mis = eng.forward([0], obs, keep=True)
        g = eng.backward()
    assert mis[0] == pytest.approx(J, rel=1e-4)
    for i in range(3):
        assert rel_l2(g[i][0], g_o[i]) <= 1e-3, i


@pytest.mark.parametrize("strategy", ["binomial", "random"])
def test_many_tiles_per_cta_batch_equals_single_shots(strategy):
    """16 shots of a 600x200 grid: ~7 forward tiles per CTA, so every stage of
    the TMA pipelines is refilled several times; each shot of the batch must be
    bitwise the shot computed alone (one tile per CTA at most)."""
    p = P.small(fdorder=8, nx=600, nz=200, nt=120, npml=8, nshots=16, nrec=6, perturb=0.04)
    fp = p.fdorder // 2
    tiles = -(-p.nxt // TX) * -(-(p.nzt - 2 * fp) // TZ) * 16
    assert tiles >= 7 * 152
    obs = np.zeros((p.nrec, p.nt))
    shots = list(range(16))
    with Engine(p) as eng:
        eng.set_strategy(strategy, **({"snapshots": 5} if strategy == "binomial" else {}))
        rec_b, mis_b = eng.forward(shots, obs, keep=True)  # one batch: all 16 shots per launch
        g_b = eng.backward()
        for s in (0, 7, 15):
            rec_s, mis_s = eng.forward([s], obs, keep=True)
            g_s = eng.backward()
            rows = O.shot_rows(p, s)
            assert np.array_equal(rec_s[rows], rec_b[rows]), s
            assert mis_s[0] == mis_b[s]
            for i in range(3):
                assert np.array_equal(g_s[i][0], g_b[i][s]), (s, i)
