"""Central finite differences of the FP64 oracle misfit, run in worker
processes (started with the spawn method, so they are safe after CUDA init)."""
from __future__ import annotations

import multiprocessing as mp
from concurrent.futures import ProcessPoolExecutor

import numpy as np


def _pair(args):
    p, obs, name, iz, ix, eps = args
    from oracle import oracle as O
    O.set_threads(1)  # one core per worker process
    vals = []
    for s in (1.0, -1.0):
        m = {"lam": p.lam.copy(), "mu": p.mu.copy(), "rho": p.rho.copy()}
        m[name][iz, ix] += s * eps
        vals.append(O.misfit(p, obs, 0, m["lam"], m["mu"], m["rho"]))
    return (vals[0] - vals[1]) / (2.0 * eps)


def central_fd(p, obs, cells, rel_eps=1e-3, names=("lam", "mu", "rho"), workers=None):
    """dJ/dm at each (iz, ix) of `cells` for each parameter in `names`, with
    the step rel_eps * m[iz, ix].  Returns {name: array[len(cells)]}."""
    jobs = []
    for name in names:
        base = getattr(p, name)
        for iz, ix in cells:
            jobs.append((p, obs, name, int(iz), int(ix), rel_eps * float(base[iz, ix])))
    with ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
        out = list(ex.map(_pair, jobs, chunksize=1))
    n = len(cells)
    return {name: np.array(out[k * n:(k + 1) * n]) for k, name in enumerate(names)}
