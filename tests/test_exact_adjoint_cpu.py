"""The oracle's exact discrete adjoint against central finite differences (CPU).

orc_exact_gradient transposes the oracle's FP64 time stepping statement by
statement.  Here it is checked against central differences of the oracle's
own FP64 misfit J = sum 0.5 dt (rec - obs)^2:

* per cell, on seeded random cells whose gradient is significant (a cell whose
  gradient is 1e-10 of the largest one is below the FD rounding floor), for
  lam, mu and rho, at orders 2, 4 and 8 with and without the free surface;
* along one seeded random direction over the whole model (every cell, every
  parameter), where the FD signal is large.
"""
import numpy as np
import pytest

from cuda_fwi_gb300 import problem as P
from oracle import oracle as O

CASES = [(2, 0), (4, 0), (4, 1), (8, 0), (8, 1)]


def _case(order, fsurf, nt=90):
    kw = dict(fdorder=order, nx=30, nz=24, nt=nt, npml=5, fsurf=fsurf, nrec=5, perturb=0.05)
    p = P.small(seed=3, **kw)
    t = P.small(seed=13, **kw)
    return p, O.forward(t, 0)["rec"]


def _models(p):
    return {"lam": p.lam, "mu": p.mu, "rho": p.rho}


def _misfit(p, obs, models):
    return O.misfit(p, obs, 0, models["lam"], models["mu"], models["rho"])


@pytest.mark.parametrize("order,fsurf", CASES)
def test_exact_gradient_matches_central_fd_per_cell(order, fsurf):
    p, obs = _case(order, fsurf)
    J, gl, gm, gr = O.exact_gradient(p, obs)
    assert J == pytest.approx(O.misfit(p, obs), rel=1e-12)
    grads = {"lam": gl, "mu": gm, "rho": gr}
    rng = np.random.default_rng(order * 10 + fsurf)
    for name, g in grads.items():
        cand = np.argwhere(np.abs(g) >= 1e-2 * np.abs(g).max())
        pick = cand[rng.choice(len(cand), size=4, replace=False)]
        for iz, ix in pick:
            eps = 1e-4 * _models(p)[name][iz, ix]
            vals = []
            for s in (1.0, -1.0):
                m = {k: v.copy() for k, v in _models(p).items()}
                m[name][iz, ix] += s * eps
                vals.append(_misfit(p, obs, m))
            fd = (vals[0] - vals[1]) / (2.0 * eps)
            assert g[iz, ix] == pytest.approx(fd, rel=1e-4), (name, iz, ix)


@pytest.mark.parametrize("order,fsurf", [(4, 1), (8, 0)])
def test_exact_gradient_directional_derivative(order, fsurf):
    p, obs = _case(order, fsurf)
    J, gl, gm, gr = O.exact_gradient(p, obs)
    rng = np.random.default_rng(5)
    base = _models(p)
    # relative perturbation direction on every cell (the pads included: the
    # gradient there must be zero or carry the pad's real influence)
    dirs = {k: rng.uniform(-1.0, 1.0, v.shape) * v for k, v in base.items()}
    lin = sum(float(np.sum(g * dirs[k])) for k, g in (("lam", gl), ("mu", gm), ("rho", gr)))
    h = 1e-5
    vals = []
    for s in (h, -h):
        vals.append(_misfit(p, obs, {k: base[k] + s * dirs[k] for k in base}))
    fd = (vals[0] - vals[1]) / (2.0 * h)
    assert lin == pytest.approx(fd, rel=1e-6)


def test_exact_gradient_zero_residual_gives_zero():
    p, _ = _case(4, 0, nt=40)
    obs = O.forward(p, 0)["rec"]
    J, gl, gm, gr = O.exact_gradient(p, obs)
    assert J == 0.0
    for g in (gl, gm, gr):
        assert not np.any(g)
