"""Exact discrete adjoint on the GPU (FWI_GRAD_EXACT).

* Against the FP64 oracle's exact adjoint (orc_exact_gradient, itself checked
  against central finite differences in test_exact_adjoint_cpu.py): relative
  L2 <= 1e-4 per parameter, orders 2/4/8, with and without the free surface,
  a sub-sampled FWI window, and a batch of shots summed.
* Against central finite differences of the FP64 oracle misfit on 32 seeded
  random cells of the config-2 model (6 layers + smoothed perturbation, order
  8) at reduced size and at full size (800x400, nt 4000), eps = 1e-3 relative.
* The checkpoint schedule and graph replay do not change the result (bitwise).
"""
import os

import numpy as np
import pytest

import _fdcheck
from conftest import rel_l2
from cuda_fwi_gb300 import _capi
from cuda_fwi_gb300 import problem as P
from cuda_fwi_gb300.engine import Engine
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _window(p, g):
    """[nzt][nxt] -> the FWI window samples, the engine's [nfz][nfx] layout (the
    engine's extra last row/column, when z2-z1 or x2-x1 divides, stays zero)."""
    w = g[p.z1:p.z2:p.fwi_dz, p.x1:p.x2:p.fwi_dx]
    out = np.zeros((p.nfz, p.nfx))
    out[: w.shape[0], : w.shape[1]] = w
    return out


def _pair(order, fsurf, nshots=1, fwi=(1, 1, 1), nt=150):
    kw = dict(fdorder=order, nx=44, nz=30, nt=nt, npml=6, fsurf=fsurf, nshots=nshots, nrec=6,
              perturb=0.05, fwi=fwi)
    p = P.small(seed=3, **kw)
    t = P.small(seed=13, **kw)
    obs = np.zeros((p.nrec, p.nt))
    for s in range(nshots):
        rows = O.shot_rows(t, s)
        obs[rows] = O.forward(t, s)["rec"][rows]
    return p, obs


def _engine_exact(p, obs, shots, snapshots=8, graphs=True, bx=0):
    with Engine(p) as eng:
        eng.set_gradient_mode("exact")
        eng.set_strategy("binomial", snapshots=snapshots)
        eng.set_exec(graphs, bx, 0, 0)
        g, mis = eng.gradient(list(shots), obs)
        st = eng.stats()
    return g, mis, st


@pytest.mark.parametrize("bx", [64, 256])
@pytest.mark.parametrize("order,fsurf", [(2, 0), (4, 0), (4, 1), (8, 0), (8, 1)])
def test_exact_matches_oracle_exact(order, fsurf, bx):
    p, obs = _pair(order, fsurf)
    J, gl, gm, gr = O.exact_gradient(p, obs)
    g, mis, st = _engine_exact(p, obs, [0], bx=bx)
    assert mis[0] == pytest.approx(J, rel=1e-5)
    for name, gg, go in zip(("lam", "mu", "rho"), g, (gl, gm, gr)):
        assert rel_l2(gg, _window(p, go)) <= 1e-4, name
    assert st["adjoint_steps"] == p.nt


def test_exact_window_and_shot_sum():
    p, obs = _pair(4, 1, nshots=3, fwi=(3, 2, 3))
    ref = [np.zeros((p.nzt, p.nxt)) for _ in range(3)]
    for s in range(3):
        _, *g = O.exact_gradient(p, obs, s)
        for i in range(3):
            ref[i] += g[i]
    g, mis, _ = _engine_exact(p, obs, [0, 1, 2])
    for i in range(3):
        assert rel_l2(g[i], _window(p, ref[i])) <= 1e-4, i


def test_exact_schedule_and_graphs_do_not_change_result():
    p, obs = _pair(8, 0, nt=120)
    a, ma, sa = _engine_exact(p, obs, [0], snapshots=3, graphs=True)
    b, mb, sb = _engine_exact(p, obs, [0], snapshots=119, graphs=False)
    assert sa["recompute_steps"] > sb["recompute_steps"]
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    assert np.array_equal(ma, mb)


def test_exact_rejects_fluid_cells():
    p, obs = _pair(4, 0, nt=40)
    mu = p.mu.copy()
    mu[p.nzt // 2, p.nxt // 2] = 0.0
    q = p.with_model(p.lam, mu, p.rho)
    with Engine(q) as eng:
        eng.set_gradient_mode("exact")
        with pytest.raises(_capi.FwiError) as ei:
            eng.gradient([0], obs)
    assert "mu > 0" in str(ei.value)


def _fd_cells(p, n, seed):
    """n seeded random cells of the physical model (outside the absorbing pads)."""
    rng = np.random.default_rng(seed)
    z0 = p.zoff()
    iz = rng.integers(z0, z0 + p.nz, n)
    ix = rng.integers(p.ppad, p.ppad + p.nx, n)
    return list(zip(iz, ix))


def _fd_check(p, obs, ncells, seed):
    cells = _fd_cells(p, ncells, seed)
    fd = _fdcheck.central_fd(p, obs, cells, rel_eps=1e-3)  # spawn pool: CPU FP64
    g, mis, _ = _engine_exact(p, obs, [0], snapshots=32)
    out = {}
    for name, gg in zip(("lam", "mu", "rho"), g):
        got = np.array([gg[(iz - p.z1) // p.fwi_dz, (ix - p.x1) // p.fwi_dx] for iz, ix in cells])
        out[name] = (got, fd[name])
    return out


def test_exact_gradient_central_fd_config2_reduced():
    t = P.config2(True, nx=120, nz=60, nt=600, npml=10, nrec=24, seed=2)
    p = P.config2(True, nx=120, nz=60, nt=600, npml=10, nrec=24, seed=7)
    obs = O.forward(t, 0)["rec"]
    for name, (got, fd) in _fd_check(p, obs, 32, seed=11).items():
        # relative L2 over the 32 cells; the FD step's own error is ~1e-6
        print(f"config 2 reduced, {name}: rel L2 vs central FD {rel_l2(got, fd):.2e}")
        assert rel_l2(got, fd) <= 1e-4, name


@pytest.mark.skipif(os.environ.get("FWI_SKIP_FULL_FDCHECK") == "1",
                    reason="full-size 800x400 FD check (~8 minutes of host FP64) skipped on request")
def test_exact_gradient_central_fd_config2_full():
    """The FD check at the workload's own size: 800x400, nt 4000, order 8, CPML 30,
    32 seeded cells, eps 1e-3 of each material value (192 FP64 forwards on the
    host cores, one per worker process)."""
    t = P.config2(True, seed=2)
    p = P.config2(True, seed=7)
    obs = O.forward(t, 0)["rec"]
    for name, (got, fd) in _fd_check(p, obs, 32, seed=11).items():
        print(f"config 2 full size, {name}: rel L2 vs central FD {rel_l2(got, fd):.2e}")
        assert rel_l2(got, fd) <= 1e-4, name
