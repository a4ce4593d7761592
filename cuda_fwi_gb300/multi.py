"""Many independent models (uneven grids, orders and nt) in one launch per pass.

    with MultiEngine([p0, p1, ...]) as m:
        grads, misfits = m.gradient([obs0, obs1, ...])   # grads[k] = (g_lam, g_mu, g_rho)

Each Problem contributes its shot 0 (vz sources and receivers of that shot).
Wraps fwi_psv_multi_* of include/fwi_psv.h; gradients are [nzt][nxt] per model
(rows above a free surface zero).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi
from ._capi import check, pd, pi
from .problem import Problem

MAPPINGS = {0: "z-march", 1: "scalar cells", 2: "vectorised cells", 3: "TMA-staged tiles"}


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class MultiEngine:
    def __init__(self, problems: list[Problem], device: int = 0, use_graphs: bool = True, snapshots: int = 32,
                 autotune: bool = True):
        self.ps = list(problems)
        self._keep = []
        models = (_capi.Model * len(self.ps))()
        for k, p in enumerate(self.ps):
            m = models[k]
            d = m.grid
            for f in ("nt", "nzt", "nxt", "fpad", "ppad", "npml", "fsurf", "fdorder"):
                setattr(d, f, int(getattr(p, f)))
            d.dt, d.dx, d.dz = p.dt, p.dx, p.dz
            for i in range(7):
                d.hc[i] = float(p.hc[i])
            cp = {f: _f64(v) for f, v in p.cpml.items()}
            for f in ("a", "b", "K", "a_half", "b_half", "K_half"):
                setattr(d, f, pd(cp[f]))
            mats = [_f64(x) for x in (p.lam, p.mu, p.rho)]
            m.lam, m.mu, m.rho = (pd(x) for x in mats)
            sel = (np.asarray(p.src_shot) == 0) & (np.asarray(p.src_comp) == 2)
            sx, sz = _i32(np.asarray(p.src_x)[sel]), _i32(np.asarray(p.src_z)[sel])
            sig = _f64(np.asarray(p.src_signal)[sel]) if sel.any() else np.zeros((1, p.nt))
            rsel = (np.asarray(p.rec_shot) == 0) & (np.asarray(p.rec_comp) == 2)
            rx, rz = _i32(np.asarray(p.rec_x)[rsel]), _i32(np.asarray(p.rec_z)[rsel])
            m.nsrc, m.src_x, m.src_z, m.src_signal = len(sx), pi(sx), pi(sz), pd(sig)
            m.nrec, m.rec_x, m.rec_z = len(rx), pi(rx), pi(rz)
            self._keep.append((cp, mats, sx, sz, sig, rx, rz, rsel))
        h = C.c_void_p()
        check(_capi.lib().fwi_psv_multi_create(len(self.ps), models, device, C.byref(h)), "fwi_psv_multi_create")
        self.h = h
        self.set_exec(use_graphs, snapshots, autotune)

    def set_exec(self, use_graphs=True, snapshots=32, autotune=True):
        check(_capi.lib().fwi_psv_multi_set_exec(self.h, int(use_graphs), int(snapshots), int(autotune)),
              "fwi_psv_multi_set_exec")

    def receiver_rows(self, k):
        """Rows of problem k's [nrec][nt] observed-data array that the engine uses (shot 0, vz)."""
        return np.nonzero(self._keep[k][7])[0]

    def forward(self):
        """vz traces of every model: list of [nrec_k][nt_k] arrays (the receivers of shot 0)."""
        n = len(self.ps)
        recs = [np.zeros((len(self.receiver_rows(k)), p.nt)) for k, p in enumerate(self.ps)]
        arr = (_capi.dp * n)(*[pd(r) for r in recs])
        check(_capi.lib().fwi_psv_multi_forward(self.h, arr), "fwi_psv_multi_forward")
        return recs

    def gradient(self, obs, want=True):
        """obs: list of [nrec][nt] arrays (the problem's receiver order; rows of
        shot 0 are used).  Returns ([(g_lam, g_mu, g_rho)] per model, misfits)."""
        n = len(self.ps)
        ob = [_f64(np.asarray(o)[self.receiver_rows(k)]) for k, o in enumerate(obs)]
        obs_p = (_capi.dp * n)(*[pd(o) for o in ob])
        mis = np.zeros(n)
        outs = [[np.zeros((p.nzt, p.nxt)) for p in self.ps] for _ in range(3)]
        arr = [(_capi.dp * n)(*[pd(g) for g in outs[q]]) if want else None for q in range(3)]
        check(_capi.lib().fwi_psv_multi_gradient(self.h, obs_p, pd(mis), *arr), "fwi_psv_multi_gradient")
        return [(outs[0][k], outs[1][k], outs[2][k]) for k in range(n)], mis

    def tuning(self):
        out = []
        g = 0
        while True:
            info = (C.c_int * 7)()
            ms = (C.c_double * 2)()
            if _capi.lib().fwi_psv_multi_tuning(self.h, g, info, ms) != 0:
                break
            out.append(dict(half_order=info[0], models=info[1], forward_mapping=MAPPINGS[info[2]],
                            forward_tile_rows=info[3], adjoint_mapping=MAPPINGS[info[4]],
                            adjoint_tile_rows=info[5], cached=bool(info[6]), forward_ms=ms[0],
                            adjoint_ms=ms[1]))
            g += 1
        return out

    def stats(self) -> dict:
        s = _capi.Stats()
        check(_capi.lib().fwi_psv_multi_get_stats(self.h, C.byref(s)), "fwi_psv_multi_get_stats")
        return {k: getattr(s, k) for k, _ in _capi.Stats._fields_}

    def close(self):
        if getattr(self, "h", None):
            _capi.lib().fwi_psv_multi_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
