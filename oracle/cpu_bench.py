"""CPU baseline timing of the oracle (the FP64 restatement of the reference's
CPU forward/adjoint path).  Used only by bench.py's CPU-baseline leg and its
reference arm.

A *sample* is one shot-gradient (forward with full storage + adjoint with
gradient) on the full padded grid of the workload, run for `nt_sample` time
steps instead of nt; its time is scaled by nt / nt_sample (the cost of the
time loop is linear in nt).  `nproc` samples run concurrently in processes
started with the spawn method, one per host core used.
"""
from __future__ import annotations

import multiprocessing as mp
import os
import time
from dataclasses import replace

import numpy as np


def _one(args):
    p, shot = args
    from oracle import oracle as O
    O.set_threads(1)  # one core per process: the processes fill the host
    obs = np.zeros((p.nrec, p.nt))
    t0 = time.perf_counter()
    O.gradient(p, obs, shot)
    return time.perf_counter() - t0


def sample_problem(p, nt_sample):
    """Same grid/model/acquisition, time loop cut to nt_sample steps."""
    q = replace(p, nt=nt_sample, src_signal=np.ascontiguousarray(p.src_signal[:, :nt_sample]))
    return q


def time_gradient_sample(p, nt_sample=30, nproc=None):
    """Returns dict(shot_gradients_per_s, cores, sample_s, nt_sample, gcell_per_s)."""
    nproc = nproc or (os.cpu_count() or 1)
    q = sample_problem(p, nt_sample)
    shot = int(q.src_shot[0]) if q.nsrc else 0
    ctx = mp.get_context("spawn")
    with ctx.Pool(nproc) as pool:
        pool.map(_one, [(replace(q, nt=2, src_signal=q.src_signal[:, :2]), shot)] * nproc)  # warm/import
        t0 = time.perf_counter()
        times = pool.map(_one, [(q, shot)] * nproc)
        wall = time.perf_counter() - t0
    per = float(np.median(times))
    scale = p.nt / nt_sample
    rate = nproc / (wall * scale)
    cells = p.nxt * p.nzt
    return dict(shot_gradients_per_s=rate, cores=nproc, sample_s=wall, nt_sample=nt_sample,
                per_process_s=per, gcell_per_s=nproc * cells * 2 * nt_sample / wall / 1e9)
