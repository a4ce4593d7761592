"""Independent models of uneven grid size, order and nt in one launch per pass.

Each model's misfit and reference gradient against the FP64 oracle run on
that model alone (relative L2: misfit 1e-4, gradients 1e-4); graph replay and
direct launches agree bitwise; the autotuner writes its choices to the JSON
cache and a second engine reads them back; a forward runs the mappings a
gradient runs.
"""
import json

import numpy as np
import pytest

from conftest import rel_l2
from cuda_fwi_gb300 import problem as P
from cuda_fwi_gb300.multi import MultiEngine
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SPECS = [dict(fdorder=4, nx=40, nz=30, nt=140, npml=6),
         dict(fdorder=8, nx=56, nz=36, nt=100, npml=8),
         dict(fdorder=4, nx=48, nz=40, nt=170, npml=8, fsurf=1),
         dict(fdorder=8, nx=30, nz=26, nt=70, npml=5)]


def _models():
    ps, obs = [], []
    for i, sp in enumerate(SPECS):
        p = P.small(nrec=5, perturb=0.05, seed=30 + i, **sp)
        t = P.small(nrec=5, perturb=0.05, seed=60 + i, **sp)
        ps.append(p)
        obs.append(O.forward(t, 0)["rec"])
    return ps, obs


def _oracle_grid(p, g):
    """oracle [nfz][nfx] window gradient -> [nzt][nxt] grid (rows above the window zero)."""
    out = np.zeros((p.nzt, p.nxt))
    out[p.z1:, :] = g[: p.nzt - p.z1, : p.nxt]
    return out


@pytest.fixture
def tune_cache(tmp_path, monkeypatch):
    path = tmp_path / "autotune.json"
    monkeypatch.setenv("FWI_PSV_TUNE_CACHE", str(path))
    return path


def test_uneven_models_match_oracle(tune_cache):
    ps, obs = _models()
    with MultiEngine(ps, snapshots=6) as m:
        grads, mis = m.gradient(obs)
        tun = m.tuning()
        st = m.stats()
    for k, p in enumerate(ps):
        J, g_o, _, _ = O.gradient(p, obs[k], 0)
        assert mis[k] == pytest.approx(J, rel=1e-4), k
        for i in range(3):
            assert rel_l2(grads[k][i], _oracle_grid(p, g_o[i])) <= 1e-4, (k, i)
    with MultiEngine(ps, snapshots=6) as m:
        recs = m.forward()
    for k, p in enumerate(ps):
        want = O.forward(p, 0)["rec"][m.receiver_rows(k)]
        assert rel_l2(recs[k], want) <= 1e-5, k
    assert sorted(t["half_order"] for t in tun) == [2, 4]
    assert sum(t["models"] for t in tun) == len(ps)
    assert st["forward_steps"] == max(s["nt"] for s in SPECS)
    assert st["recompute_steps"] > 0 and st["batch"] == len(ps)
    data = json.loads(tune_cache.read_text())
    assert len(data) == 2 and all({"fwd_map", "fwd_tz", "adj_map", "adj_tz"} <= set(v) for v in data.values())


def test_graphs_mappings_and_cache(tune_cache):
    ps, obs = _models()
    with MultiEngine(ps, snapshots=4, use_graphs=True, autotune=True) as m:
        g1, m1 = m.gradient(obs)
        g1b, m1b = m.gradient(obs)  # graph replay
    with MultiEngine(ps, snapshots=4, use_graphs=False, autotune=True) as m:
        g2, m2 = m.gradient(obs)    # direct launches, choices read from the cache
        tun = m.tuning()
    assert all(t["cached"] for t in tun)
    for k in range(len(ps)):
        for i in range(3):
            assert np.array_equal(g1[k][i], g1b[k][i])
            assert np.array_equal(g1[k][i], g2[k][i])
    assert np.array_equal(m1, m2)
    with MultiEngine(ps, snapshots=4, autotune=False) as m:  # default mappings
        g3, _ = m.gradient(obs)
    for k in range(len(ps)):
        for i in range(3):
            assert rel_l2(g3[k][i], g1[k][i]) <= 3e-5, (k, i)


def test_tma_tiles_match_oracle(tune_cache):
    """The TMA-staged passes over the uneven work-list (maps per model in device
    memory): the tuner's cache is rewritten to choose them for both passes of
    every order group, and a new engine reads it."""
    ps, obs = _models()
    with MultiEngine(ps, snapshots=5, autotune=True) as m:
        m.gradient(obs)
    data = json.loads(tune_cache.read_text())
    for v in data.values():
        v.update(fwd_map=3, fwd_tz=0, adj_map=3, adj_tz=0)
    # the engine's layout: one entry per line
    lines = [f" {json.dumps(k)}: {json.dumps(v)}" for k, v in data.items()]
    tune_cache.write_text("{\n" + ",\n".join(lines) + "\n}\n")
    with MultiEngine(ps, snapshots=5, autotune=True) as m:
        grads, mis = m.gradient(obs)
        tun = m.tuning()
        grads_r, mis_r = m.gradient(obs)  # graph replay
    assert all(t["cached"] and t["forward_mapping"] == t["adjoint_mapping"] == "TMA-staged tiles" for t in tun)
    for k, p in enumerate(ps):
        J, g_o, _, _ = O.gradient(p, obs[k], 0)
        assert mis[k] == pytest.approx(J, rel=1e-4), k
        for i in range(3):
            assert rel_l2(grads[k][i], _oracle_grid(p, g_o[i])) <= 1e-4, (k, i)
            assert np.array_equal(grads[k][i], grads_r[k][i])


def test_forward_uses_the_gradients_mappings(tune_cache):
    """A forward tunes like a gradient (or reads the same cache), so every
    engine over the same models computes the same traces bit for bit, with the
    choices forced to the TMA tiles or left to the tuner."""
    ps, obs = _models()
    with MultiEngine(ps, snapshots=4, autotune=True) as m:
        m.gradient(obs)
        rec_a = m.forward()
    with MultiEngine(ps, snapshots=4, autotune=True) as m:
        rec_b = m.forward()  # no gradient first: the cache written above
        tun = m.tuning()
    assert all(t["cached"] for t in tun)
    for a, b in zip(rec_a, rec_b):
        assert np.array_equal(a, b)
