"""GPU tests of the higher-level API: sub-batched gradients, the autograd
wrapper, and the reference-shaped C++ shims through the C ABI."""
import numpy as np
import pytest
import torch

from conftest import rel_l2
from cuda_fwi_gb300 import problem as P
from cuda_fwi_gb300.engine import Engine
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _case(nshots=5, order=8):
    p = P.small(fdorder=order, nx=60, nz=40, nt=140, npml=8, nshots=nshots, nrec=5, perturb=0.04, seed=9)
    t = P.small(fdorder=order, nx=60, nz=40, nt=140, npml=8, nshots=nshots, nrec=5, perturb=0.04, seed=19)
    obs = np.zeros((p.nrec, p.nt))
    for s in range(nshots):
        r = O.forward(t, s)["rec"]
        rows = O.shot_rows(t, s)
        obs[rows] = r[rows]
    return p, obs


@pytest.mark.parametrize("bx", [64, 256])
@pytest.mark.parametrize("batch", [1, 2, 5, 0])
def test_gradient_subbatches_match_oracle(batch, bx):
    p, obs = _case()
    g_ref = [np.zeros((p.nfz, p.nfx)) for _ in range(3)]
    mis_ref = []
    for s in range(p.nshots):
        J, g, _, _ = O.gradient(p, obs, s)
        mis_ref.append(J)
        for i in range(3):
            g_ref[i] += g[i]
    with Engine(p) as eng:
        eng.set_strategy("binomial", snapshots=6)
        eng.set_exec(True, bx, 0, batch)
        g, mis = eng.gradient(list(range(p.nshots)), obs)
        g2, mis2 = eng.gradient(list(range(p.nshots)), None, resident=True)
    np.testing.assert_allclose(mis, mis_ref, rtol=1e-4)
    for i in range(3):
        assert rel_l2(g[i], g_ref[i]) <= 1e-4
        assert np.array_equal(g[i], g2[i])
    assert np.array_equal(mis, mis2)


@pytest.mark.parametrize("mode", ["exact", "reference"])
def test_autograd_wrapper(mode):
    """forward = fwi_psv_forward (misfit only), backward = fwi_psv_backward;
    the gradient equals the engine's fused gradient call in the same mode."""
    from cuda_fwi_gb300.autograd import misfit
    p, obs = _case(nshots=2)
    lam = torch.tensor(p.lam, requires_grad=True)
    mu = torch.tensor(p.mu, requires_grad=True)
    rho = torch.tensor(p.rho, requires_grad=True)
    with Engine(p) as eng:
        J = misfit(lam, mu, rho, eng, [0, 1], obs, mode)
        assert eng.stats()["adjoint_steps"] == 0  # the forward alone runs no adjoint
        (2.0 * J).backward()
        assert eng.stats()["adjoint_steps"] == p.nt
        eng.set_gradient_mode(mode)
        g, mis = eng.gradient([0, 1], obs)
    assert float(J.detach()) == pytest.approx(float(np.sum(mis)), rel=1e-12)
    win = (slice(p.z1, p.z2, p.fwi_dz), slice(p.x1, p.x2, p.fwi_dx))
    for t, gi in zip((lam, mu, rho), g):
        gw = t.grad.numpy()[win]
        # the window loop fills nfz-1 x nfx-1 entries when the range divides evenly
        np.testing.assert_allclose(gw, 2.0 * gi[: gw.shape[0], : gw.shape[1]], rtol=1e-6)


def test_autograd_exact_mode_is_the_misfit_derivative():
    """In exact mode the wrapper's gradient matches the FP64 oracle's discrete
    adjoint of the same misfit (relative L2 <= 1e-4)."""
    from cuda_fwi_gb300.autograd import misfit
    p, obs = _case(nshots=1, order=4)
    lam = torch.tensor(p.lam, requires_grad=True)
    mu = torch.tensor(p.mu, requires_grad=True)
    rho = torch.tensor(p.rho, requires_grad=True)
    with Engine(p) as eng:
        misfit(lam, mu, rho, eng, [0], obs).backward()
    J, gl, gm, gr = O.exact_gradient(p, obs, 0)
    win = (slice(p.z1, p.z2, p.fwi_dz), slice(p.x1, p.x2, p.fwi_dx))
    for t, go in zip((lam, mu, rho), (gl, gm, gr)):
        assert rel_l2(t.grad.numpy()[win], go[win]) <= 1e-4


def test_engine_reuses_graphs_across_shot_ids():
    p, obs = _case(nshots=4, order=4)
    with Engine(p) as eng:
        eng.set_exec(True, 0, 0, 2)
        eng.gradient([0, 1, 2, 3], obs)
        l1 = eng.stats()["launches"]
        eng.gradient([3, 2, 1, 0], obs)
        assert eng.stats()["launches"] == l1
