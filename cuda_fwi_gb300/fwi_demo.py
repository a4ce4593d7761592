"""The FWI loop on the config-5 workload (2000x600, nt 5000, order 8, 96 shots).

    python -m cuda_fwi_gb300.fwi_demo [--iters 2] [--shots 96] [--nt 5000] [--snapshots 32]
                                      [--restart STEP] [--resume FILE]

Observed data come from the true model (faulted, folded 30-layer medium with
a wedge and a salt body) by a batched forward on the GPU; the inversion starts
from the true model smoothed with sigma = 300 m and runs fwi_psv_fwi_run
(summed shot gradients with energy preconditioning, parabolic step-length
search with batched trial forwards, bounded update).  --restart STEP retries
a search that finds no step lowering the misfit once from STEP (the reference
would stop there; the loop then continues).  --resume FILE saves the loop
state there after each iteration and continues from it when the file exists
(a run cut short picks up where it stopped).  One line per
iteration: misfit, step length, trials, model error against the true model,
seconds; then a JSON summary.
"""
from __future__ import annotations

import argparse
import json
import time
from dataclasses import replace

import numpy as np

from . import problem as P
from .engine import Engine


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--iters", type=int, default=2)
    ap.add_argument("--shots", type=int, default=96)
    ap.add_argument("--nt", type=int, default=0, help="cut the record (0 = the workload's 5000 steps)")
    ap.add_argument("--snapshots", type=int, default=32)
    ap.add_argument("--restart", type=float, default=0.0,
                    help="retry a failed step search once from this step (0 = stop, as the reference)")
    ap.add_argument("--resume", default=None, help="resume file of the FWI loop (saved after each iteration)")
    a = ap.parse_args(argv)
    true = P.config5(True, nshots=a.shots)
    start = P.config5(False, nshots=a.shots)
    if a.nt:
        true = replace(true, nt=a.nt, src_signal=np.ascontiguousarray(true.src_signal[:, : a.nt]))
        start = replace(start, nt=a.nt, src_signal=np.ascontiguousarray(start.src_signal[:, : a.nt]))
    shots = list(range(a.shots))
    t0 = time.perf_counter()
    with Engine(true) as e:
        obs, _ = e.forward(shots)
    t_obs = time.perf_counter() - t0
    with Engine(start) as e:
        e.set_strategy("binomial", snapshots=a.snapshots)
        err0 = float(np.sqrt(np.mean([np.sum((m0 - m1) ** 2) / np.sum(m1 ** 2) for m0, m1 in
                                      zip((start.lam, start.mu, start.rho), (true.lam, true.mu, true.rho))])))
        (lam, mu, rho), log = e.fwi_run(shots, obs, a.iters, step_length=0.01, order="summed", trial="sum",
                                        true_model=(true.lam, true.mu, true.rho), restart_step=a.restart,
                                        resume_file=a.resume)
    for i, r in enumerate(log):
        print(f"iteration {i + 1}: misfit {r['misfit']:.6e}  step {r['step_length']:.4e}  trials {r['trials']}  "
              f"status {r['status']}  model error {r['model_error']:.6f}  {r['seconds']:.1f} s", flush=True)
    print(json.dumps({"workload": f"config 5: {true.nx}x{true.nz} (padded {true.nxt}x{true.nzt}), nt {true.nt}, "
                                  f"order {true.fdorder}, {a.shots} shots x {true.nrec // a.shots} receivers, "
                                  f"binomial {a.snapshots} slots, restart step {a.restart}",
                      "observed_data_seconds": t_obs, "model_error_start": err0, "iterations": log}))


if __name__ == "__main__":
    main()
