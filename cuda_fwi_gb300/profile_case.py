"""Small, self-terminating case for profiling the stencil kernels under ncu.

    python -m cuda_fwi_gb300.profile_case SHOTS [--nt 40] [--snapshots 4] [--graphs]
                                                [--block-x B] [--time REPS]

Runs the batched-gradient workload's grid (1000x500, 1068x568 padded, order 8,
30-cell CPML) for SHOTS shots with nt cut short: one forward sweep with
binomial checkpoints and one backward, direct kernel launches by default (so
ncu sees each launch).  SHOTS >= 10 keeps the per-step state above the 126 MB
L2 so DRAM counters stay meaningful.  --block-x selects the stencil thread
mapping (set_exec); --time REPS also prints fwi_psv_time_kernels (ms per launch
of forward stress, forward velocity, adjoint stress, adjoint velocity).
"""
from __future__ import annotations

import argparse
from dataclasses import replace

import numpy as np

from . import problem as P
from .engine import Engine


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("shots", type=int)
    ap.add_argument("--nt", type=int, default=40)
    ap.add_argument("--snapshots", type=int, default=4)
    ap.add_argument("--graphs", action="store_true")
    ap.add_argument("--block-x", type=int, default=0)
    ap.add_argument("--time", type=int, default=0)
    a = ap.parse_args(argv)
    p = P.config3(False, nshots=a.shots)
    p = replace(p, nt=a.nt, src_signal=p.src_signal[:, : a.nt].copy())
    obs = np.zeros((p.nrec, a.nt))
    with Engine(p) as e:
        e.set_exec(a.graphs, a.block_x, 0, 0)
        e.set_strategy("binomial", snapshots=min(a.snapshots, a.nt - 1))
        e.forward(list(range(a.shots)), obs, keep=True)
        g = e.backward(sum_shots=True)
        print("ok", a.shots, float(np.abs(g[0]).max()))
        if a.time:
            e.forward(list(range(a.shots)), obs, keep=True, want_rec=False)
            ms = e.time_kernels(a.time)
            print("time_ms", a.shots, a.block_x, " ".join(f"{x:.4f}" for x in ms))


if __name__ == "__main__":
    main()
