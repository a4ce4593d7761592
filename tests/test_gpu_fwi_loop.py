"""The FWI optimiser on the GPU against its FP64 restatement.

* fwi_psv_set_model_device (averaging kernel) gives the same materials as the
  host path (bitwise-equal seismograms).
* Energy-weight preconditioned, shot-summed gradients and forward-only trial
  misfits match the oracle (relative L2 <= 1e-4).
* Two iterations of the summed-gradient loop (step-length search with
  batched trial forwards, bounded update) follow oracle/fwi_loop.py: same
  trials and statuses, misfits within 1e-4, step lengths within 1e-3, and the
  model change within 1e-3 (relative L2).
* The reference's own order -- a gradient, step search and update per shot,
  with the last shot's trial misfit (fwi_run's defaults) or the all-shot sum --
  follows the same restatement to the same bounds.
* A run continued from its resume file equals an uninterrupted one.
"""
import numpy as np
import pytest

from conftest import rel_l2
from cuda_fwi_gb300 import _capi
from cuda_fwi_gb300 import problem as P
from cuda_fwi_gb300.engine import Engine
from oracle import fwi_loop as FL
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _case(nshots=2, nt=150):
    kw = dict(fdorder=4, nx=40, nz=30, nt=nt, npml=6, nshots=nshots, nrec=6)
    p = P.small(seed=3, perturb=0.0, **kw)
    t = P.small(seed=21, perturb=0.06, **kw)
    obs = np.zeros((p.nrec, p.nt))
    for s in range(nshots):
        rows = O.shot_rows(t, s)
        obs[rows] = O.forward(t, s)["rec"][rows]
    return p, t, obs


def test_device_materials_equal_host_materials():
    import torch
    p, _, obs = _case(nshots=1, nt=80)
    with Engine(p) as eng:
        rec_h, _ = eng.forward([0], obs)
        dev = [torch.tensor(x, dtype=torch.float64, device="cuda") for x in (p.lam, p.mu, p.rho)]
        eng.set_model_device(*dev)
        rec_d, _ = eng.forward([0], obs)
    assert np.array_equal(rec_h, rec_d)


def test_preconditioned_gradient_and_trial_misfits():
    p, _, obs = _case()
    c = [float(np.mean(x)) for x in (p.lam, p.mu, p.rho)]
    ref = [np.zeros((p.nfz, p.nfx)) for _ in range(3)]
    mis_ref = []
    for s in range(2):
        J, g, fw, ad = O.gradient(p, obs, s)
        mis_ref.append(J)
        g = FL.scale_gradients(p, list(g), fw["We"], ad["We"], c)
        for i in range(3):
            ref[i] += g[i]
    with Engine(p) as eng:
        eng.set_strategy("binomial", snapshots=8)
        eng.set_precondition(True, c)
        g, mis = eng.gradient([0, 1], obs)
        eng.set_precondition(False)
        trial = eng.misfit([0, 1], None, resident=True)
    for i in range(3):
        assert rel_l2(g[i], ref[i]) <= 1e-4, i
    np.testing.assert_allclose(mis, mis_ref, rtol=1e-4)
    np.testing.assert_allclose(trial, mis_ref, rtol=1e-4)


def test_fwi_loop_follows_restatement():
    p, t, obs = _case()
    lam_r, mu_r, rho_r, log_r = FL.fwi_loop(p, obs, [0, 1], iters=2, step0=0.01)
    with Engine(p) as eng:
        eng.set_strategy("binomial", snapshots=8)
        (lam, mu, rho), log = eng.fwi_run([0, 1], obs, max_iter=2, step_length=0.01,
                                          true_model=(t.lam, t.mu, t.rho))
    assert len(log) == len(log_r)
    for a, b in zip(log, log_r):
        assert a["trials"] == b["trials"] and a["status"] == b["status"]
        assert a["misfit"] == pytest.approx(b["misfit"], rel=1e-4)
        assert a["step_length"] == pytest.approx(b["step_length"], rel=1e-3)
        assert a["model_error"] >= 0.0
    for got, want, start in ((lam, lam_r, p.lam), (mu, mu_r, p.mu), (rho, rho_r, p.rho)):
        assert rel_l2(got - start, want - start) <= 1e-3
    assert log[-1]["misfit"] < log[0]["misfit"]


@pytest.mark.parametrize("trial", ["last", "sum"])
def test_fwi_loop_per_shot_order_follows_restatement(trial):
    """FWI_ORDER_PER_SHOT (fd_wave_model.cu:777-955) with FWI_TRIAL_LAST_SHOT
    (fwi_step_length_estimation.cu:136) -- the reference's loop and fwi_run's
    default -- and with the summed trial misfit.  The last shot's observed data
    lie halfway between the starting and the true model's, so the reference's
    comparison (the first shot's misfit against the last shot's trial misfits)
    accepts steps and the loop makes four updates."""
    p, t, obs = _case()
    rows = O.shot_rows(p, 1)
    obs[rows] = 0.5 * (obs[rows] + O.forward(p, 1)["rec"][rows])
    lam_r, mu_r, rho_r, log_r = FL.fwi_loop(p, obs, [0, 1], iters=2, step0=0.01, order="per_shot", trial=trial)
    with Engine(p) as eng:
        eng.set_strategy("binomial", snapshots=8)
        (lam, mu, rho), log = eng.fwi_run([0, 1], obs, max_iter=2, step_length=0.01, order="per_shot",
                                          trial=trial, true_model=(t.lam, t.mu, t.rho))
    assert len(log) == len(log_r) == 4
    for a, b in zip(log, log_r):
        assert a["trials"] == b["trials"] and a["status"] == b["status"]
        assert a["misfit"] == pytest.approx(b["misfit"], rel=1e-4)
        assert a["step_length"] == pytest.approx(b["step_length"], rel=1e-3)
    for got, want, start in ((lam, lam_r, p.lam), (mu, mu_r, p.mu), (rho, rho_r, p.rho)):
        assert rel_l2(got - start, want - start) <= 1e-3


def test_failed_search_retry_follows_restatement():
    """The opt-in continuation (restart_step > 0): a search that finds no step
    lowering the misfit is run once more on the same gradient from restart_step
    before the loop stops.  In this per-shot, last-shot-trial case both searches
    fail (14 trial sweeps in all); the engine's log and model equal the
    restatement's (the model unchanged)."""
    p, t, obs = _case()
    lam_r, mu_r, rho_r, log_r = FL.fwi_loop(p, obs, [0, 1], iters=2, step0=0.01, order="per_shot", trial="last",
                                            restart_step=0.05)
    with Engine(p) as eng:
        eng.set_strategy("binomial", snapshots=8)
        (lam, mu, rho), log = eng.fwi_run([0, 1], obs, max_iter=2, step_length=0.01, order="per_shot",
                                          trial="last", restart_step=0.05)
    assert [(a["trials"], a["status"]) for a in log] == [(b["trials"], b["status"]) for b in log_r] == [(14, 1)]
    assert log[0]["misfit"] == pytest.approx(log_r[0]["misfit"], rel=1e-4)
    assert np.array_equal(lam, p.lam) and np.array_equal(mu, p.mu) and np.array_equal(rho, p.rho)


@pytest.mark.parametrize("order", ["summed", "per_shot"])
def test_resume_file_continues_like_an_uninterrupted_run(order, tmp_path):
    """fwi_psv_fwi_opts.resume_file: a run of one iteration saves the loop
    state, a second run with max_iter 2 finds the file and does the second
    iteration only; log and model equal an uninterrupted two-iteration run bit
    for bit.  A file written under other options is refused."""
    p, t, obs = _case()
    kw = dict(max_iter=2, step_length=0.01, order=order, trial="sum", true_model=(t.lam, t.mu, t.rho))
    with Engine(p) as eng:
        eng.set_strategy("binomial", snapshots=8)
        (lam_a, mu_a, rho_a), log_a = eng.fwi_run([0, 1], obs, **kw)
    path = tmp_path / "fwi.resume"
    with Engine(p) as eng:
        eng.set_strategy("binomial", snapshots=8)
        _, log_1 = eng.fwi_run([0, 1], obs, **dict(kw, max_iter=1), resume_file=path)
    assert path.exists() and 1 <= len(log_1) <= len(log_a)
    with Engine(p) as eng:  # a new engine: the state comes from the file
        eng.set_strategy("binomial", snapshots=8)
        (lam_b, mu_b, rho_b), log_b = eng.fwi_run([0, 1], obs, **kw, resume_file=path)
        with pytest.raises(_capi.FwiError) as ei:
            eng.fwi_run([0, 1], obs, **dict(kw, step_length=0.02), resume_file=path)
        assert ei.value.code == "FWI_ERR_INVALID"
    keys = ("misfit", "step_length", "trials", "status", "model_error")
    assert [[r[k] for k in keys] for r in log_b] == [[r[k] for k in keys] for r in log_a]
    assert np.array_equal(lam_b, lam_a) and np.array_equal(mu_b, mu_a) and np.array_equal(rho_b, rho_a)
