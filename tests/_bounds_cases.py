"""Engine runs whose outputs the bounds-checked build must reproduce (run as a
subprocess by tests/test_gpu_bounds_check.py, with FWI_PSV_LIB naming the
library under test): orders 2, 8 and 4 with a free surface, full storage
(the stress pass's storage writes), binomial checkpointing (the copy-free
backward: reads across checkpoint buffers) and the fused forward step,
forward and reference gradient; then the multi-model engine with its TMA
tiles chosen for both passes.  Usage: python _bounds_cases.py OUT.npz"""
import json
import os
import sys
import tempfile

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
from cuda_fwi_gb300 import problem as P  # noqa: E402
from cuda_fwi_gb300.engine import Engine  # noqa: E402
from cuda_fwi_gb300.multi import MultiEngine  # noqa: E402

CASES = [dict(fdorder=2, nx=40, nz=30, nt=80, npml=5),
         dict(fdorder=8, nx=150, nz=50, nt=100, npml=8),
         dict(fdorder=4, nx=60, nz=40, nt=90, npml=6, fsurf=1)]


def main(path):
    out = {}
    for i, kw in enumerate(CASES):
        p = P.small(nrec=6, nshots=2, perturb=0.04, seed=40 + i, **kw)
        t = P.small(nrec=6, nshots=2, perturb=0.04, seed=70 + i, **kw)
        with Engine(t) as e:
            obs, _ = e.forward([0, 1])
        for strat in ("full", "binomial", "fused"):
            with Engine(p) as e:
                if strat == "fused":
                    e.set_exec(True, 512, 0)
                e.set_strategy("full" if strat == "full" else "binomial", snapshots=6)
                rec, mis = e.forward([0, 1], obs, keep=True)
                g = e.backward()
            out[f"c{i}_{strat}_rec"] = rec
            out[f"c{i}_{strat}_mis"] = mis
            for q, a in zip(("lam", "mu", "rho"), g):
                out[f"c{i}_{strat}_{q}"] = np.asarray(a)
    # multi-model engine, TMA tiles for both passes of both order groups
    ms = [P.small(nrec=5, perturb=0.05, seed=80 + i, **kw) for i, kw in enumerate(CASES)]
    mobs = []
    for i, kw in enumerate(CASES):
        t = P.small(nrec=5, perturb=0.05, seed=90 + i, **kw)
        with Engine(t) as e:
            o, _ = e.forward([0])
        mobs.append(o)
    cache = os.path.join(tempfile.mkdtemp(), "tune.json")
    os.environ["FWI_PSV_TUNE_CACHE"] = cache
    with MultiEngine(ms, snapshots=5, autotune=True) as m:
        m.gradient(mobs)
    data = json.loads(open(cache).read())
    for v in data.values():
        v.update(fwd_map=3, fwd_tz=0, adj_map=3, adj_tz=0)
    open(cache, "w").write("{\n" + ",\n".join(f" {json.dumps(k)}: {json.dumps(v)}" for k, v in data.items())
                           + "\n}\n")
    with MultiEngine(ms, snapshots=5, autotune=True) as m:
        grads, mis = m.gradient(mobs)
        assert all(t["forward_mapping"] == t["adjoint_mapping"] == "TMA-staged tiles" for t in m.tuning())
    out["multi_mis"] = np.asarray(mis)
    for k, g in enumerate(grads):
        for q, a in zip(("lam", "mu", "rho"), g):
            out[f"multi{k}_{q}"] = np.asarray(a)
    np.savez(path, **out)


if __name__ == "__main__":
    main(sys.argv[1])
