#!/usr/bin/env python
"""Benchmark: batched, checkpointed shot-gradients/s on one GB300.

Workload (the batched multi-shot gradient configuration): 1000x500 grid
(1068x568 padded), dx=dz=10 m, dt=1 ms, nt=3000, 8th-order Holberg, 30-cell
CPML, layered model with a dipping fault (observed data) and without it
(synthetics), 64 shots x 250 receivers, binomial checkpointing with 32 slots
per shot, gradients summed over shots.  One step = one batch of 64 shot
gradients: forward sweep, residual, recompute + adjoint + gradient.

Printed JSON line (rank 0):
  value        shot-gradients/s, device-timed (CUDA events on the engine's
               stream) with the observed data resident in HBM
  e2e          the same through the public API with host buffers: the
               observed data goes host->device and the summed gradient
               device->host inside the timed region
  roofline     the dominant kernel (forward stress pass) timed live with CUDA
               events, algorithmic bytes per launch / duration vs measured HBM peak
  cpu_baseline the FP64 CPU restatement of the reference path on the host cores
  plain        the same gradient as one-shot-per-launch, no CUDA graph

--impl reference times the CPU reference path (the oracle port of the
reference's CPU forward/adjoint; the reference's own code implements only
fdorder 2) on all host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

HBM_FALLBACK_GBS = 6800.0


def parse():
    return parse_args(None)


def parse_args(argv):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--shots", type=int, default=64)
    ap.add_argument("--snapshots", type=int, default=32)
    ap.add_argument("--nt", type=int, default=0, help="override nt (testing only)")
    ap.add_argument("--plain-shots", type=int, default=3)
    ap.add_argument("--batch", type=int, default=0, help="shots per launch (0 = engine default)")
    ap.add_argument("--cpu-nt-sample", type=int, default=200)
    ap.add_argument("--no-uneven", dest="uneven", action="store_false",
                    help="skip the uneven batch of independent models (config 4)")
    ap.add_argument("--uneven-check", type=int, default=8,
                    help="models of the uneven batch compared with the one-model engine")
    ap.add_argument("--no-random-boundary", dest="random_boundary", action="store_false",
                    help="skip the random-boundary comparison")
    ap.add_argument("--block-x", type=int, default=0,
                    help="stencil thread mapping (set_exec block_x; 0 = engine default)")
    ap.add_argument("--no-cpu", action="store_true")
    return ap.parse_args(argv)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK_GBS, "fallback"


def workload(args, setup=None, world=1):
    """(true, synthetic) problems of the workload; `setup` replaces the engine
    library's setup helpers (the reference arm passes the oracle's).  With
    `world` ranks the survey has args.shots shots per rank (weak scaling)."""
    from cuda_fwi_gb300 import problem as P
    P.use_setup_helpers(setup)
    true = P.config3(True, nshots=args.shots * world)
    syn = P.config3(False, nshots=args.shots * world)
    if args.nt:
        from dataclasses import replace
        for name in ("true", "syn"):
            p = locals()[name]
            q = replace(p, nt=args.nt, src_signal=p.src_signal[:, : args.nt].copy())
            if name == "true":
                true = q
            else:
                syn = q
    return true, syn


WORKLOAD_DESC = ("1000x500 (1068x568 padded) elastic P-SV, dx=dz=10 m, dt=1 ms, nt=3000, "
                 "8th-order Holberg, 30-cell CPML, faulted layered model, 64 shots x 250 receivers, "
                 "binomial checkpointing 32 slots/shot, gradients summed over shots")


def bench_config(args, syn, world):
    """The workload's description, printed identically by both arms."""
    return {"workload": WORKLOAD_DESC, "shots_per_step": args.shots, "nt": syn.nt,
            "padded_grid": [syn.nzt, syn.nxt], "fdorder": syn.fdorder,
            "checkpoints_per_shot": args.snapshots,
            "l2": "inputs larger than L2 (per-step working set ~30 GB: 64 shot states, "
                  "checkpoints, 192 MB observed data)",
            "parallelism": f"replicas x{world}, shots batched in one launch per time step"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i].lower() == "active"})
        pw = [float(r[3]) for r in self.rows if r[3].replace(".", "").isdigit()]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows),
                "power_w_median": statistics.median(pw) if pw else None}


def cpu_baseline(syn, args, nproc=None):
    from oracle import cpu_bench
    r = cpu_bench.time_gradient_sample(syn, nt_sample=args.cpu_nt_sample, nproc=nproc)
    return {"value": r["shot_gradients_per_s"], "unit": "shot-gradients/s", "cores": r["cores"],
            "kind": "port",
            "sample": (f"{r['cores']} concurrent single-thread processes, each one shot-gradient "
                       f"(forward with full storage + adjoint + gradient, FP64 order-8 restatement of the "
                       f"reference CPU path) over {r['nt_sample']} of {syn.nt} time steps on the full "
                       f"1068x568 grid, time scaled by nt/{r['nt_sample']}; {r['sample_s']:.1f} s wall"),
            "gcell_upd_s": r["gcell_per_s"],
            # one process = one core (all cores busy at the same time)
            "per_core_value": 1.0 / (r["per_process_s"] * syn.nt / r["nt_sample"])}


def product_library_mapped():
    """Whether this process has the engine library mapped (Linux /proc)."""
    try:
        with open("/proc/self/maps") as f:
            return "libfwi_psv.so" in f.read()
    except OSError:
        return None


def run_reference(args, rank):
    if rank != 0:
        return
    t0 = time.perf_counter()
    # the reference arm never loads the engine library: its problem is set up
    # by the oracle's own helpers (bit-identical to the engine's host code)
    from oracle import oracle as O
    _, syn = workload(args, setup=O.setup_helpers)
    vals = []
    last = None
    for i in range(args.warmup + args.steps):
        last = cpu_baseline(syn, args)
        if i >= args.warmup:
            vals.append(last["value"])
    v = statistics.mean(vals)
    last["value"] = v
    out = {"impl": "reference", "metric": "shot-gradients/s", "value": v, "unit": "shot-gradients/s",
           "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic", "config": bench_config(args, syn, args.gpus),
           "cpu_baseline": last,
           "product_library_mapped": product_library_mapped(),
           "e2e": {"value": v, "unit": "shot-gradients/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "wall_s": time.perf_counter() - t0}
    print(json.dumps(out), flush=True)


def fused_step(block_x, fp):
    """Whether the forward sweeps run the fused one-launch step (block_x 512,
    fdorder <= 8)."""
    return block_x == 512 and fp <= 4


def kernel_names(block_x, fp):
    """The four timed kernels of the thread mapping set_exec(block_x) selects
    (entry 1 is None when the forward step is one fused launch)."""
    if fused_step(block_x, fp):
        return [f"step_fused_kernel<{fp}> (forward/recompute step: stress+velocity+CPML fused, TMA-staged "
                f"120-column strips marched in 16-row chunks)", None,
                f"adjoint_tma_kernel<{fp}> (adjoint stress+CPML+ux/uz+gradient, TMA-staged 128x8 tiles)",
                f"velocity_tma_kernel<{fp}> (adjoint velocity+CPML+energy, TMA-staged 128x16 tiles)"]
    if block_x in (0, 256, 512):  # TMA-staged tiles, two passes per forward step
        return [f"stress_tma_kernel<{fp}> (forward/recompute stress+CPML, TMA-staged 128x16 tiles)",
                f"velocity_tma_kernel<{fp}> (forward/recompute velocity+CPML, TMA-staged 128x16 tiles)",
                f"adjoint_tma_kernel<{fp}> (adjoint stress+CPML+ux/uz+gradient, TMA-staged 128x8 tiles)",
                f"velocity_tma_kernel<{fp}> (adjoint velocity+CPML+energy, TMA-staged 128x16 tiles)"]
    amap = 1 if block_x in (32, 64) else 0
    vmap = {32: 1, 64: 2}.get(block_x, 0)
    return [f"stress_kernel<{fp},false,{vmap}> (forward/recompute stress+CPML)",
            f"velocity_kernel<{fp},{vmap}> (forward/recompute velocity+CPML)",
            f"stress_kernel<{fp},true,{amap}> (adjoint stress+CPML+ux/uz+gradient)",
            f"velocity_kernel<{fp},{vmap}> (adjoint velocity+CPML+energy)"]


def algorithmic_bytes(p, B, fused=False):
    """Minimal DRAM bytes of one launch over B shots (FP32): per-shot fields
    once, shared materials once per launch, CPML memory of strip cells.  With
    the fused step, entry 0 is the whole forward step (read and write the five
    fields once, 40 B, the four CPML memories of a strip cell, 32 B, and all
    five materials, 20 B) and entry 1 is 0."""
    fp = p.fpad
    nxi, nzi = p.nxt - 2 * fp, p.nzt - 2 * fp
    cells = nxi * nzi
    cpml_cells = 2 * p.npml * nzi + 2 * p.npml * nxi
    stress_fwd = B * (cells * (8 + 24) + cpml_cells * 16) + cells * 12
    vel_fwd = B * (cells * (12 + 16) + cpml_cells * 16) + cells * 8  # recompute sweeps: no energy
    if fused:
        stress_fwd, vel_fwd = B * (cells * 40 + cpml_cells * 32) + cells * 20, 0
    # adjoint: + ux,uz r/w (16) + 5 forward fields (20) + 3 gradients r/w (24) at a sampled step
    stress_adj = B * (cells * (8 + 24 + 16 + 20 + 24) + cpml_cells * 16) + cells * 12
    vel_adj = B * (cells * (12 + 16 + 8) + cpml_cells * 16) + cells * 8
    return stress_fwd, vel_fwd, stress_adj, vel_adj


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank)

    true, syn = workload(args, world=world)
    # CPU baseline first: its spawn pool starts before any CUDA call.
    cpu = None
    if rank == 0 and not args.no_cpu:
        try:
            cpu = cpu_baseline(syn, args)
        except Exception as e:  # reported, never silently replaced
            cpu = {"value": None, "error": repr(e)}

    import numpy as np
    import torch
    from cuda_fwi_gb300.engine import Engine

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    # this rank's shots: every rank takes args.shots of the survey's args.shots * world
    # (cuda_fwi_gb300.distributed.shard_shots, the sharding its gloo test covers)
    from cuda_fwi_gb300 import distributed as D
    all_shots = list(range(args.shots * world))
    shots = D.shard_shots(all_shots, rank, world)
    with Engine(true, device=local) as e:
        e.set_exec(use_graphs=True)
        obs, _ = e.forward(shots)
    obs = np.ascontiguousarray(obs)

    stream = torch.cuda.Stream(device=local)
    eng = Engine(syn, device=local)
    eng.set_stream(stream.cuda_stream)
    eng.set_strategy("binomial", snapshots=args.snapshots)
    eng.set_exec(True, args.block_x, 0, args.batch)

    def step_resident():
        # one batch of shot gradients, observed data resident in HBM, summed gradient left on the device
        eng.gradient(shots, None, resident=True, want=False)

    def step_e2e():
        # public API with host buffers: FP64 observed data in, summed FP64 gradient out;
        # with several ranks, the survey's gradient: this rank's shots, then one all-reduce
        if dist is None:
            g, mis = eng.gradient(shots, obs)
            return mis
        g, mis = D.distributed_gradient(lambda s: eng.gradient(s, obs), all_shots, len(all_shots), rank, world,
                                        device=f"cuda:{local}")
        return mis

    # warm-up (captures the CUDA graphs; the first call uploads the observed data)
    eng.gradient(shots, obs)
    for _ in range(args.warmup):
        step_resident()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    # ---- device-timed region (observed data resident) ----
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        ev0.record(stream)
        launches = 0
        for _ in range(args.steps):
            step_resident()
            launches += eng.stats()["launches"]
        ev1.record(stream)
        barrier()
    dev_s = ev0.elapsed_time(ev1) / 1e3
    st = eng.stats()
    launches_per_step = launches / args.steps

    # ---- end to end through the public API with host buffers ----
    barrier()
    t0 = time.perf_counter()
    h2d = d2h = 0
    for _ in range(args.steps):
        step_e2e()
    barrier()
    e2e_s = time.perf_counter() - t0
    est = eng.stats()
    h2d, d2h = est["h2d_bytes"], est["d2h_bytes"]

    def maxr(x):
        if dist is None:
            return x
        t = torch.tensor([x], dtype=torch.float64, device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    dev_s, e2e_s = maxr(dev_s), maxr(e2e_s)
    B = args.shots
    cells = syn.nxt * syn.nzt
    recompute = st["recompute_steps"]  # per shot
    steps_per_batch = syn.nt + recompute + syn.nt
    sub = int(st["batch"])
    value = world * B * args.steps / dev_s
    gcell = world * B * cells * steps_per_batch * args.steps / dev_s / 1e9
    # "useful" rate: 2 nt propagation steps per shot-gradient (no recompute counted)
    gcell_useful = world * B * cells * 2 * syn.nt * args.steps / dev_s / 1e9

    # ---- roofline: live per-kernel timing on one full sub-batch ----
    eng.forward(shots[:sub], obs, keep=True, want_rec=False)  # lays out a batch of `sub` shots
    ms = eng.time_kernels(reps=20)
    fused = fused_step(args.block_x, syn.fpad)
    b_sf, b_vf, b_sa, b_va = algorithmic_bytes(syn, sub, fused)
    counts = [syn.nt + recompute, 0 if fused else syn.nt + recompute, syn.nt, syn.nt]
    shares = [c * t for c, t in zip(counts, ms)]
    names = kernel_names(args.block_x, syn.fpad)
    dom = max(range(4), key=lambda i: shares[i])
    peak, peak_kind = peaks()
    achieved = [b / (t / 1e3) / 1e9 if t > 0 else 0.0 for b, t in zip((b_sf, b_vf, b_sa, b_va), ms)]
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tfile):
        try:
            traffic = json.load(open(tfile)).get(names[dom].split(" ")[0] + f"@B{sub}")
        except Exception:
            traffic = None

    # ---- plain path: one shot per launch, no graph, same kernels/checkpointing ----
    plain = None
    if rank == 0 and args.plain_shots > 0:
        pe = Engine(syn, device=local)
        pe.set_exec(False, args.block_x, 0, 1)
        pe.set_strategy("binomial", snapshots=args.snapshots)
        pe.gradient([0], obs)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for s in range(args.plain_shots):
            pe.gradient([s], obs)
        torch.cuda.synchronize()
        ps = (time.perf_counter() - t0) / args.plain_shots
        plain = {"shot_gradients_s": 1.0 / ps, "batched_over_plain": (value / world) * ps,
                 "how": f"{args.plain_shots} shot(s), one shot per launch, direct launches (no graph), "
                        f"same kernels and binomial checkpointing; host wall clock"}
        pe.close()
        # context: the same one-shot path on the scalar one-thread-per-cell kernels
        # (the reference's GPU kernel design), and the bound the roofline puts on
        # any batched path: algorithmic bytes per shot-gradient / measured HBM peak
        pc = Engine(syn, device=local)
        pc.set_exec(False, 32, 0, 1)
        pc.set_strategy("binomial", snapshots=args.snapshots)
        pc.gradient([0], obs)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pc.gradient([0], obs)
        torch.cuda.synchronize()
        pcs = time.perf_counter() - t0
        pc.close()
        fb = [x / sub for x in algorithmic_bytes(syn, sub, fused)]  # per shot, materials shared by a launch
        per_grad = (syn.nt + recompute) * (fb[0] + fb[1]) + syn.nt * (fb[2] + fb[3]) + \
            syn.nt * (syn.nxt - 2 * syn.fpad) * (syn.nzt - 2 * syn.fpad) * 8  # + energy of the recording sweep
        bound = peak * 1e9 / per_grad
        plain.update({"scalar_cells_shot_gradients_s": 1.0 / pcs,
                      "batched_over_plain_scalar_cells": (value / world) * pcs,
                      "roofline_bound_shot_gradients_s": bound,
                      "roofline_bound_over_plain": bound * ps})

    # ---- the other strategy of the workload: random-boundary reconstruction ----
    rbinfo = None
    if rank == 0 and args.random_boundary:
        g_bin, _ = eng.gradient(shots, None, resident=True)
        rb = Engine(syn, device=local)
        rb.set_strategy("random")
        rb.set_exec(True, args.block_x, 0, args.batch)
        rb.gradient(shots, obs)  # warm-up, graphs
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g_rb, _ = rb.gradient(shots, None, resident=True)
        torch.cuda.synchronize()
        rs = time.perf_counter() - t0
        rst = rb.stats()
        diff = float(np.sqrt(sum(np.sum((a - b) ** 2) for a, b in zip(g_rb, g_bin)) /
                             sum(np.sum(b ** 2) for b in g_bin)))
        # per parameter over the model interior (the padding, where the frame replaces the CPML, left out)
        inner = (slice(max(0, syn.ppad - syn.z1), g_bin[0].shape[0] - syn.ppad),
                 slice(syn.ppad, g_bin[0].shape[1] - syn.ppad))
        per = {k: float(np.linalg.norm(a[inner] - b[inner]) / np.linalg.norm(b[inner]))
               for k, a, b in zip(("lam", "mu", "rho"), g_rb, g_bin)}
        rbinfo = {"shot_gradients_s": B / rs, "time_steps_per_shot_gradient": 2 * syn.nt + int(rst["recompute_steps"]),
                  "device_bytes": int(rst["device_bytes"]),
                  "grad_rel_l2_vs_binomial": diff,
                  "grad_rel_l2_vs_binomial_interior": per,
                  "how": "same workload and batches, FWI_STORE_RANDOM (residual from the CPML forward, one state "
                         "per shot, random-frame forward rebuilt in reverse), host wall clock over one step; the "
                         "difference to the binomial gradient is the random frame's scattering in the source "
                         "wavefield, not an error"}
        rb.close()

    # ---- config 4: uneven batch of independent models in one launch per pass ----
    unev = None
    if rank == 0 and args.uneven:
        from cuda_fwi_gb300 import problem as P
        from cuda_fwi_gb300.multi import MultiEngine
        specs = P.config4_specs()
        trues = [P.config4_model(sp, True) for sp in specs]
        syns = [P.config4_model(sp, False) for sp in specs]
        with MultiEngine(trues, device=local) as mt:
            obs_u = mt.forward()
        mu = MultiEngine(syns, device=local, snapshots=args.snapshots)
        mu.gradient(obs_u)  # warm-up: autotuning (or its cache) and graph capture
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g_u, mis_u = mu.gradient(obs_u)
        torch.cuda.synchronize()
        tu = time.perf_counter() - t0
        tuning = mu.tuning()
        mst = mu.stats()
        mu.close()
        # the batch against the one-model engine running the same kernels (the
        # order group's tuned mapping): only the batching differs
        bx = {"vectorised cells": 64, "scalar cells": 32, "z-march": 128, "TMA-staged tiles": 256}
        errs = []
        for k in range(min(args.uneven_check, len(syns))):
            t = next(t_ for t_ in tuning if t_["half_order"] == syns[k].fpad)
            se = Engine(syns[k], device=local)
            se.set_exec(True, bx[t["forward_mapping"]], t["forward_tile_rows"], 0)
            se.set_strategy("binomial", snapshots=args.snapshots)
            gs, _ = se.gradient([0], obs_u[k])
            se.close()
            num = sum(float(np.sum((g_u[k][q] - gs[q][: syns[k].nzt, : syns[k].nxt]) ** 2)) for q in range(3))
            den = sum(float(np.sum(gs[q] ** 2)) for q in range(3))
            errs.append(float(np.sqrt(num / den)) if den > 0 else 0.0)
        useful = sum(p_.nxt * p_.nzt * 2 * p_.nt for p_ in syns)
        unev = {"models": len(syns), "shot_gradients_s": len(syns) / tu, "seconds": tu,
                "gcell_upd_s_useful": useful / tu / 1e9,
                "grid_range": [[min(p_.nx for p_ in syns), min(p_.nz for p_ in syns)],
                               [max(p_.nx for p_ in syns), max(p_.nz for p_ in syns)]],
                "nt_range": [min(p_.nt for p_ in syns), max(p_.nt for p_ in syns)],
                "orders": sorted({p_.fdorder for p_ in syns}),
                "launches": int(mst["launches"]), "tuning": tuning,
                "grad_rel_l2_vs_single_model_engine_same_kernels": errs,
                "misfit": [float(x) for x in mis_u],
                "how": "config-4 models from seed 4 (anomaly-free starting models, observed data from the models "
                       "with their anomaly), one shot each, binomial checkpointing with a common plan over the "
                       "longest nt, one launch per pass per order group, CUDA graphs; host wall clock over one "
                       "gradient of all models; the error column compares the first models with the one-model "
                       "engine running the same kernels on the same data (only the batching differs); per-model "
                       "parity with the FP64 oracle: tests/test_gpu_multi.py (small models) and "
                       "tests/test_gpu_fullsize.py (three of these models at their drawn sizes; models whose "
                       "records miss the anomaly have a near-zero residual, whose gradient is FP32 noise)"}

    if rank == 0:
        out = {
            "metric": "shot-gradients/s", "value": value, "unit": "shot-gradients/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dev_s / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": bench_config(args, syn, world),
            "shots_per_launch": sub,
            "gcell_upd_s": gcell,
            "gcell_upd_s_useful": gcell_useful,
            "time_steps_per_shot_gradient": steps_per_batch,
            "e2e": {"value": world * B * args.steps / e2e_s, "unit": "shot-gradients/s",
                    "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": int(launches_per_step * args.steps),
            "roofline": {"bound": "hbm", "kernel": names[dom], "achieved": achieved[dom],
                         "peak": peak, "unit": "GB/s", "frac": achieved[dom] / peak,
                         "peak_source": peak_kind, "traffic": traffic,
                         "launch_ms": ms[dom], "algorithmic_bytes_per_launch": [b_sf, b_vf, b_sa, b_va][dom],
                         "all_kernels": {n.split(" ")[0] + ("_adj" if i >= 2 else "_fwd"):
                                         {"ms": ms[i], "GBps": achieved[i], "count_per_step": counts[i]}
                                         for i, n in enumerate(names) if n}},
            "plain": plain,
            "random_boundary": rbinfo,
            "uneven_batch": unev,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
        }
        print(json.dumps(out), flush=True)
    eng.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
