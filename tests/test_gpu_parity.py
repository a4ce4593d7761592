"""GPU parity of the sm_103a engine (called through the C ABI) against the
reference's outputs (golden fixtures, fdorder 2) and the FP64 CPU oracle
(fdorder 4..12).  Tolerances (relative L2): seismograms 1e-5, gradients 1e-4.
"""
import numpy as np
import pytest

import _plan
from _fixtures import load
from conftest import rel_l2
from cuda_fwi_gb300 import _capi
from cuda_fwi_gb300 import problem as P
from cuda_fwi_gb300.engine import Engine
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SEIS_TOL = 1e-5
GRAD_TOL = 1e-4


# block_x of set_exec: 64 = vectorised cells, 256 = TMA-staged tiles with two passes per
# forward step (the default mapping), 512 = TMA-staged tiles with the fused forward step
MAPPINGS = [64, 256, 512]


@pytest.mark.parametrize("bx", MAPPINGS)
@pytest.mark.parametrize("name", ["ref_o2.npz", "ref_o2_fsurf.npz", "ref_o2_multi.npz"])
def test_engine_matches_reference_golden(name, bx):
    p, d = load(name)
    shot = int(d["shot"])
    rows = O.shot_rows(p, shot)
    with Engine(p) as eng:
        eng.set_exec(True, bx, 0)
        rec, mis = eng.forward([shot], d["obs"], keep=True)
        assert rel_l2(rec[rows], d["out_rec"][rows]) <= SEIS_TOL
        assert mis[0] == pytest.approx(float(d["out_misfit"]), rel=1e-4)
        w = eng.wavefield(0)
        for k in ("vx", "vz", "sxx", "szx", "szz"):
            assert rel_l2(w[k], d["out_fwd_" + k]) <= SEIS_TOL, k
        ws, _ = eng.energy(0)
        assert rel_l2(ws, d["out_fwd_We"]) <= SEIS_TOL
        g = eng.backward()
        for i, k in enumerate(("grad_lam", "grad_mu", "grad_rho")):
            assert rel_l2(g[i][0], d["out_adj_" + k]) <= GRAD_TOL, k
        _, wr = eng.energy(0)
        assert rel_l2(wr, d["out_adj_We"]) <= GRAD_TOL


def _run_ref_shaped(p, d):
    """fwi_psv_forward_kernel / fwi_psv_adjoint_kernel with the reference's argument list."""
    L = _capi.lib()
    pd, pi = _capi.pd, _capi.pi
    tp = 2 * (p.npml + 1)
    shot = int(d["shot"])
    mz, rz, rx = _capi.average_parameters(p.mu, p.rho)
    wave = [np.zeros((p.nzt, p.nxt)) for _ in range(6)]
    mem = [np.zeros((p.nzt, tp)), np.zeros((tp, p.nxt)), np.zeros((p.nzt, tp)), np.zeros((tp, p.nxt)),
           np.zeros((p.nzt, tp)), np.zeros((p.nzt, tp)), np.zeros((tp, p.nxt)), np.zeros((tp, p.nxt))]
    cp = [np.ascontiguousarray(p.cpml[k]) for k in ("a", "b", "K", "a_half", "b_half", "K_half")]
    rec = np.zeros((p.nrec, p.nt))
    store = [np.zeros((p.nft, p.nfz, p.nfx)) for _ in range(5)]
    fw = (1, p.fwi_dt, p.fwi_dx, p.fwi_dz, p.x1, p.x2, p.z1, p.z2)
    st = L.fwi_psv_forward_kernel(
        shot, p.nt, p.nzt, p.nxt, p.fpad, p.ppad, p.dt, p.dx, p.dz, p.nt, p.fsurf, pd(p.hc), p.fdorder,
        *[pd(x) for x in wave], pd(p.lam), pd(p.mu), pd(mz), pd(rz), pd(rx), p.npml, *[pd(x) for x in cp],
        *[pd(x) for x in mem], p.nsrc, pi(p.src_x), pi(p.src_z), pi(p.src_comp), pd(p.src_signal),
        pi(p.src_shot), p.nrec, pi(p.rec_x), pi(p.rec_z), pi(p.rec_comp), pd(rec), pi(p.rec_shot),
        *fw, *[pd(x) for x in store])
    _capi.check(st, "forward_kernel")
    res = np.zeros_like(rec)
    rows = O.shot_rows(p, shot)
    res[rows] = rec[rows] - d["obs"][rows]
    g = [np.zeros((p.nfz, p.nfx)) for _ in range(3)]
    wave2 = [np.zeros((p.nzt, p.nxt)) for _ in range(6)]
    st = L.fwi_psv_adjoint_kernel(
        shot, p.nt, p.nzt, p.nxt, p.fpad, p.ppad, p.dt, p.dx, p.dz, p.nt, p.fsurf, pd(p.hc), p.fdorder,
        *[pd(x) for x in wave2], pd(p.lam), pd(p.mu), pd(mz), pd(rz), pd(rx), p.npml,
        *[pd(x) for x in cp], *[pd(x) for x in mem], p.nrec, pi(p.rec_x), pi(p.rec_z), pi(p.rec_comp),
        pd(res), pi(p.rec_shot), *fw, *[pd(x) for x in store], *[pd(x) for x in g])
    _capi.check(st, "adjoint_kernel")
    return rec, wave, store, g, wave2


@pytest.mark.parametrize("name", ["ref_o2.npz", "ref_o2_fsurf.npz"])
def test_reference_shaped_entry_points(name):
    p, d = load(name)
    rec, wave, store, g, wave2 = _run_ref_shaped(p, d)
    rows = O.shot_rows(p, int(d["shot"]))
    assert rel_l2(rec[rows], d["out_rec"][rows]) <= SEIS_TOL
    assert rel_l2(wave[5], d["out_fwd_We"]) <= SEIS_TOL
    for i, k in enumerate(("vx", "vz", "sxx", "szx", "szz")):
        assert rel_l2(store[i], d["out_store_" + k]) <= SEIS_TOL, k
    for i, k in enumerate(("grad_lam", "grad_mu", "grad_rho")):
        assert rel_l2(g[i], d["out_adj_" + k]) <= GRAD_TOL, k
    assert rel_l2(wave2[5], d["out_adj_We"]) <= GRAD_TOL


def _oracle_case(order, fsurf=0, fwi=(1, 1, 1), nt=200, seed=0):
    p = P.small(fdorder=order, nx=56, nz=44, nt=nt, npml=10, fsurf=fsurf, nrec=7, perturb=0.05,
                seed=seed, fwi=fwi)
    true = P.small(fdorder=order, nx=56, nz=44, nt=nt, npml=10, fsurf=fsurf, nrec=7, perturb=0.05,
                   seed=seed + 100, fwi=fwi)
    obs = O.forward(true, 0)["rec"]
    return p, obs


@pytest.mark.parametrize("order,fsurf,fwi", [(4, 0, (1, 1, 1)), (6, 0, (2, 1, 1)), (8, 0, (1, 1, 1)),
                                             (8, 1, (3, 2, 2)), (12, 0, (1, 1, 1)), (4, 1, (1, 1, 1)),
                                             (2, 1, (1, 1, 1)), (10, 1, (1, 2, 1))])
@pytest.mark.parametrize("bx", MAPPINGS)
def test_engine_matches_oracle_higher_orders(order, fsurf, fwi, bx):
    p, obs = _oracle_case(order, fsurf, fwi)
    J, g_o, fw_o, ad_o = O.gradient(p, obs, 0)
    with Engine(p) as eng:
        eng.set_exec(True, bx, 0)
        rec, mis = eng.forward([0], obs, keep=True)
        assert rel_l2(rec[: p.nrec], fw_o["rec"]) <= SEIS_TOL
        assert mis[0] == pytest.approx(J, rel=1e-4)
        g = eng.backward()
    for i in range(3):
        assert rel_l2(g[i][0], g_o[i]) <= GRAD_TOL, i


@pytest.mark.parametrize("bx", MAPPINGS)
@pytest.mark.parametrize("order,fsurf,fwi", [(2, 0, (1, 1, 1)), (4, 1, (1, 1, 1)), (8, 0, (2, 1, 1)),
                                             (8, 1, (3, 2, 2)), (12, 0, (1, 1, 1))])
def test_checkpointed_adjoint_matches_oracle(order, fsurf, fwi, bx):
    """Binomial checkpointing: the adjoint stress pass reads the forward fields
    from the recomputed forward state (the TMA mapping stages them)."""
    p, obs = _oracle_case(order, fsurf, fwi, nt=160, seed=8)
    J, g_o, fw_o, ad_o = O.gradient(p, obs, 0)
    with Engine(p) as eng:
        eng.set_exec(True, bx, 0)
        eng.set_strategy("binomial", snapshots=5)
        rec, mis = eng.forward([0], obs, keep=True)
        g = eng.backward()
        ws, wr = eng.energy(0)
    assert rel_l2(rec[: p.nrec], fw_o["rec"]) <= SEIS_TOL
    assert mis[0] == pytest.approx(J, rel=1e-4)
    for i in range(3):
        assert rel_l2(g[i][0], g_o[i]) <= GRAD_TOL, i
    assert rel_l2(wr, ad_o["We"]) <= GRAD_TOL


def test_batch_equals_single_shots_bitwise():
    p = P.small(fdorder=8, nx=64, nz=40, nt=160, npml=10, nshots=4, nrec=5, perturb=0.04)
    obs = np.zeros((p.nrec, p.nt))
    with Engine(p) as eng:
        rec_b, mis_b = eng.forward([0, 1, 2, 3], obs + 0.0, keep=True)
        g_b = eng.backward()
        for s in range(4):
            rec_s, mis_s = eng.forward([s], obs, keep=True)
            g_s = eng.backward()
            rows = O.shot_rows(p, s)
            assert np.array_equal(rec_s[rows], rec_b[rows])
            assert mis_s[0] == mis_b[s]
            for i in range(3):
                assert np.array_equal(g_s[i][0], g_b[i][s])
        _, _ = eng.forward([0, 1, 2, 3], obs, keep=True)
        g_sum = eng.backward(sum_shots=True)
        for i in range(3):
            np.testing.assert_allclose(g_sum[i], g_b[i].sum(0), rtol=1e-5, atol=1e-30)


@pytest.mark.parametrize("bx", MAPPINGS)
@pytest.mark.parametrize("fwi,snaps", [((1, 1, 1), 3), ((3, 2, 2), 2), ((1, 1, 1), 0), ((2, 1, 1), 40)])
def test_binomial_checkpointing_equals_full_storage(fwi, snaps, bx):
    """Same forward; the gradient is bitwise equal where both strategies run
    the same adjoint kernel (vectorised mapping).  The TMA mapping stages the
    checkpointed forward state in its own adjoint kernel, whose rounding
    differs from the full-storage kernel's."""
    p, obs = _oracle_case(8, 0, fwi, nt=150, seed=3)
    with Engine(p) as eng:
        eng.set_exec(True, bx, 0)
        eng.set_strategy("full")
        rec_f, mis_f = eng.forward([0], obs, keep=True)
        g_f = eng.backward()
        eng.set_strategy("binomial", snapshots=min(snaps, p.nft - 1))
        rec_c, mis_c = eng.forward([0], obs, keep=True)
        g_c = eng.backward()
        st = eng.stats()
    assert np.array_equal(rec_f, rec_c) and mis_f[0] == mis_c[0]
    for i in range(3):
        if bx == 64:
            assert np.array_equal(g_f[i], g_c[i]), i
        else:
            assert rel_l2(g_c[i], g_f[i]) <= 3e-5, i
    if snaps:
        # forward steps the backward actually runs (the first sweep placed
        # its checkpoints), in time steps
        want = _plan.recompute_after_first_sweep(p.nft, min(snaps, p.nft - 1)) * p.fwi_dt
        assert st["recompute_steps"] == want > 0


def test_graphs_and_direct_launches_agree():
    p, obs = _oracle_case(4, 0, (1, 1, 1), nt=120, seed=5)
    out = []
    for graphs in (True, False):
        with Engine(p) as eng:
            eng.set_exec(use_graphs=graphs)
            rec, _ = eng.forward([0], obs, keep=True)
            g = eng.backward()
            out.append((rec, g))
    assert np.array_equal(out[0][0], out[1][0])
    for i in range(3):
        assert np.array_equal(out[0][1][i], out[1][1][i])


@pytest.mark.parametrize("bx,tz", [(128, 1), (128, 5), (128, 64), (32, 0), (64, 0), (256, 0)])
def test_thread_mappings_agree(bx, tz):
    """z-march tiles of any height, the scalar and vectorised cell mappings and
    the TMA-staged tiles compute the same stencil (rounding may differ)."""
    p, obs = _oracle_case(8, 0, (1, 1, 1), nt=100, seed=6)
    with Engine(p) as eng:
        rec0, _ = eng.forward([0], obs, keep=True)
        g0 = eng.backward()
        eng.set_exec(True, bx, tz)
        rec1, _ = eng.forward([0], obs, keep=True)
        g1 = eng.backward()
    assert rel_l2(rec1, rec0) <= 1e-6
    # two FP32 roundings of the same 100-step correlation sums (each mapping
    # is within 1e-4 of the FP64 oracle on its own)
    for i in range(3):
        assert rel_l2(g1[i], g0[i]) <= 3e-5


def test_z_march_tile_heights_bitwise_identical():
    p, obs = _oracle_case(8, 0, (1, 1, 1), nt=100, seed=6)
    with Engine(p) as eng:
        eng.set_exec(True, 128, 3)
        rec0, _ = eng.forward([0], obs)
        eng.set_exec(True, 128, 40)
        rec1, _ = eng.forward([0], obs)
    assert np.array_equal(rec0, rec1)


def test_error_paths():
    p, obs = _oracle_case(4, 0, (1, 1, 1), nt=60, seed=7)
    with Engine(p) as eng:
        with pytest.raises(_capi.FwiError) as e:
            eng.backward()
        assert e.value.code == "FWI_ERR_NOFORWARD"
        with pytest.raises(_capi.FwiError) as e:
            eng.set_fwi(1, 1, 1, 0, p.nxt + 5, 0, p.nzt)
        assert e.value.code == "FWI_ERR_INVALID"
        bad_x = p.src_x.copy()
        bad_x[0] = 0
        with pytest.raises(_capi.FwiError) as e:
            eng.set_sources(bad_x, p.src_z, p.src_comp, p.src_shot, p.src_signal)
        assert e.value.code == "FWI_ERR_INVALID"
        with pytest.raises(_capi.FwiError) as e:
            eng.set_exec(True, 48, 0)
        assert e.value.code == "FWI_ERR_INVALID"
        with pytest.raises(_capi.FwiError) as e:
            eng.forward([0], obs * 1e12 + 1e11)
        assert e.value.code == "FWI_ERR_DIVERGED"
        # the engine stays usable after errors
        rec, _ = eng.forward([0], obs)
        assert np.isfinite(rec).all()
