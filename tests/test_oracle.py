"""The CPU oracle is pinned against the reference (CPU only).

1. Golden fixtures made by the reference's own compiled CPU code
   (tests/golden/make_golden.py) must be reproduced bit for bit.
2. Where the reference sources are present, random extra cases are compared
   live against oracle/_ref.
3. The Ricker known-answer vector shipped with the reference.
"""
import numpy as np
import pytest

from _fixtures import load
from cuda_fwi_gb300 import problem as P
from conftest import rel_l2
from oracle import oracle as O
from oracle import reference as R

GOLDEN = ["ref_o2.npz", "ref_o2_fsurf.npz", "ref_o2_multi.npz"]


@pytest.mark.parametrize("name", GOLDEN)
def test_oracle_reproduces_reference_golden(name):
    p, d = load(name)
    shot = int(d["shot"])
    fw = O.forward(p, shot, True)
    assert np.array_equal(fw["rec"], d["out_rec"])
    for k in ("vx", "vz", "sxx", "szx", "szz", "We"):
        assert np.array_equal(fw[k], d["out_fwd_" + k]), k
    for k in ("vx", "vz", "sxx", "szx", "szz"):
        assert np.array_equal(fw["store"][k], d["out_store_" + k]), k
    J, res, blow = O.residual(fw["rec"], d["obs"], p.dt, O.shot_rows(p, shot))
    assert not blow
    assert J == pytest.approx(float(d["out_misfit"]), rel=1e-15)
    ad = O.adjoint(p, shot, res, fw["store"])
    for k in ("grad_lam", "grad_mu", "grad_rho", "We", "vz"):
        assert np.array_equal(ad[k], d["out_adj_" + k]), k


def test_ricker_known_answer():
    kat = np.load(__import__("_fixtures").GOLDEN / "ricker_kat.npz")
    s = O.wavelet(len(kat["signal"]), float(kat["dt"]), float(kat["amp"]), float(kat["fc"]))
    # the CSV holds 6 significant digits
    np.testing.assert_allclose(s, kat["signal"], rtol=5e-6, atol=1e-12)


def test_holberg_table_shape():
    hc = O.holberg(8, 1)
    assert hc[1] == 1.2257 and hc[4] == -0.0026274 and hc[5] == 0.0
    assert O.holberg(2, 0)[1] == 1.0
    with pytest.raises(ValueError):
        O.holberg(14, 1)


def test_calc_opt_step_parabola():
    # L2(s) = (s - 0.3)^2 + 1 sampled at 0, 0.2, 0.5 -> vertex at 0.3
    sl = np.array([0.0, 0.2, 0.5])
    L2 = (sl - 0.3) ** 2 + 1.0
    assert O.calc_opt_step(L2, sl) == pytest.approx(0.3, rel=1e-6)


needs_ref = pytest.mark.skipif(not R.available(), reason="reference sources not present")


@needs_ref
@pytest.mark.parametrize("seed,fsurf", [(3, 0), (4, 1), (5, 0)])
def test_oracle_matches_reference_live(seed, fsurf):
    from cuda_fwi_gb300 import problem as P
    rng = np.random.default_rng(seed)
    p = P.small(fdorder=2, nx=int(rng.integers(24, 50)), nz=int(rng.integers(20, 40)),
                nt=int(rng.integers(60, 140)), npml=int(rng.integers(3, 9)), fsurf=fsurf,
                nshots=2, nrec=3, perturb=0.08, seed=seed,
                fwi=(int(rng.integers(1, 4)), int(rng.integers(1, 3)), int(rng.integers(1, 3))))
    for shot in (0, 1):
        fo, fr = O.forward(p, shot, True), R.forward(p, shot, True)
        for k in ("vx", "vz", "sxx", "szx", "szz", "We", "rec"):
            assert np.array_equal(fo[k], fr[k]), k
        res = O.residual(fo["rec"], 0.5 * fo["rec"], p.dt, O.shot_rows(p, shot))[1]
        ao, ar = O.adjoint(p, shot, res, fo["store"]), R.adjoint(p, shot, res, fr["store"])
        for k in ("grad_lam", "grad_mu", "grad_rho", "We"):
            assert np.array_equal(ao[k], ar[k]), k


@needs_ref
def test_setup_helpers_match_reference():
    for args in [(10, 4.0, 17.0, 2.0, 1.0, 1e-3, 3300.0, 0.6e-3), (30, 5.0, 15.0, 2.0, 2.0, 1e-4, 4500., 0.5e-3)]:
        a, b = O.cpml(*args), R.cpml(*args)
        for k in a:
            assert np.array_equal(a[k], b[k])
    for order in (2, 4, 6, 8, 10, 12):
        for err in range(5):
            assert np.array_equal(O.holberg(order, err), R.holberg(order, err))
    rng = np.random.default_rng(1)
    rho = rng.uniform(1000, 3000, (20, 30))
    rho[2:4, 5:8] = 0.0
    mu = rng.uniform(1e9, 5e9, (20, 30))
    mu[7, 7] = 0.0
    for x, y in zip(O.average(mu, mu, rho), R.average(mu, mu, rho)):
        assert np.array_equal(x, y)
    assert np.array_equal(O.wavelet(300, 1e-3, 2.0, 12.0, 0.01), R.wavelet(300, 1e-3, 2.0, 12.0, 0.01))


def test_restatement_orders_consistent():
    """Higher orders have no reference; the restatement must at least converge:
    a coarse-vs-fine grid pair agrees better at order 8 than at order 2."""
    from cuda_fwi_gb300 import problem as P
    errs = {}
    for order in (2, 8):
        p = P.small(fdorder=order, nx=40, nz=36, nt=150, npml=8, nrec=6, seed=2)
        errs[order] = O.forward(p, 0)["rec"]
    assert np.all(np.isfinite(errs[2])) and np.all(np.isfinite(errs[8]))
    assert 0.0 < rel_l2(errs[8], errs[2]) < 1.0


@pytest.mark.parametrize("order,fsurf,fwi,interval,shot,nshots", [
    (2, 0, (1, 1, 1), 7, 0, 1), (4, 1, (2, 1, 1), 1, 0, 1), (8, 0, (3, 2, 2), 50, 1, 2),
    (8, 1, (1, 1, 1), 13, 0, 1), (6, 0, (1, 2, 3), 120, 0, 1), (12, 0, (2, 1, 1), 9, 2, 3)])
def test_checkpointed_gradient_is_bit_identical(order, fsurf, fwi, interval, shot, nshots):
    """orc_gradient_ckpt (states every `interval` steps, segments recomputed)
    gives the stored-wavefield sequence's seismograms, misfit, gradients and
    energies bit for bit, whatever the interval."""
    kw = dict(fdorder=order, nx=40, nz=30, nt=120, npml=6, fsurf=fsurf, nshots=nshots, nrec=5,
              perturb=0.05, fwi=fwi)
    p, t = P.small(seed=2, **kw), P.small(seed=12, **kw)
    obs = O.forward(t, shot)["rec"]
    J, g, fw, ad = O.gradient(p, obs, shot)
    Jc, gc, rec, wf, wa = O.gradient_ckpt(p, obs, shot, interval=interval)
    rows = O.shot_rows(p, shot)
    assert Jc == J
    assert np.array_equal(rec[rows], fw["rec"][rows])
    for a, b in zip(gc, g):
        assert np.array_equal(a, b)
    assert np.array_equal(wf, fw["We"]) and np.array_equal(wa, ad["We"])


def test_oracle_threads_do_not_change_results():
    p = P.small(fdorder=8, nx=48, nz=36, nt=90, npml=6, fsurf=1, nrec=5, perturb=0.05, seed=5)
    obs = O.forward(P.small(fdorder=8, nx=48, nz=36, nt=90, npml=6, fsurf=1, nrec=5, perturb=0.05,
                            seed=6), 0)["rec"]
    n0 = O.set_threads(0)
    try:
        O.set_threads(1)
        J1, g1, _, _ = O.gradient(p, obs, 0)
        O.set_threads(max(2, n0))
        J2, g2, _, _ = O.gradient(p, obs, 0)
    finally:
        O.set_threads(n0)
    assert J1 == J2
    for a, b in zip(g1, g2):
        assert np.array_equal(a, b)
