"""Load the self-contained golden fixtures of tests/golden as Problem objects."""
from __future__ import annotations

from pathlib import Path

import numpy as np

from cuda_fwi_gb300.problem import Problem

GOLDEN = Path(__file__).resolve().parent / "golden"

_INT = ("nx", "nz", "nt", "fdorder", "npml", "fsurf", "fpad", "ppad", "nxt", "nzt", "fwi_dt",
        "fwi_dx", "fwi_dz", "x1", "x2", "z1", "z2")
_FLT = ("dx", "dz", "dt")


def load(name: str):
    d = dict(np.load(GOLDEN / name))
    p = Problem(**{k: int(d[k]) for k in _INT if k not in ("fpad", "ppad", "nxt", "nzt", "x1", "x2", "z1", "z2")},
                **{k: float(d[k]) for k in _FLT})
    for k in ("fpad", "ppad", "nxt", "nzt", "x1", "x2", "z1", "z2"):
        setattr(p, k, int(d[k]))
    p.hc = d["hc"]
    p.cpml = {k: d["cpml_" + k] for k in ("a", "b", "K", "a_half", "b_half", "K_half")}
    for k in ("lam", "mu", "rho", "src_signal"):
        setattr(p, k, np.ascontiguousarray(d[k], np.float64))
    for k in ("src_x", "src_z", "src_comp", "src_shot", "rec_x", "rec_z", "rec_comp", "rec_shot"):
        setattr(p, k, np.ascontiguousarray(d[k], np.int32))
    p.nshots = int(p.src_shot.max()) + 1
    return p, d
