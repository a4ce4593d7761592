"""Engine runs whose outputs the bounds-checked build must reproduce (run as a
subprocess by tests/test_gpu_bounds_check.py, with FWI_PSV_LIB naming the
library under test): orders 2, 8 and 4 with a free surface, full storage
(the stress pass's storage writes) and binomial checkpointing (the copy-free
backward: reads across checkpoint buffers), forward and reference gradient
on the default TMA-staged mapping.  Usage: python _bounds_cases.py OUT.npz"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
from cuda_fwi_gb300 import problem as P  # noqa: E402
from cuda_fwi_gb300.engine import Engine  # noqa: E402

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
        for strat in ("full", "binomial"):
            with Engine(p) as e:
                e.set_strategy(strat, snapshots=6)
                rec, mis = e.forward([0, 1], obs, keep=True)
                g = e.backward()
            out[f"c{i}_{strat}_rec"] = rec
            out[f"c{i}_{strat}_mis"] = mis
            for q, a in zip(("lam", "mu", "rho"), g):
                out[f"c{i}_{strat}_{q}"] = np.asarray(a)
    np.savez(path, **out)


if __name__ == "__main__":
    main(sys.argv[1])
