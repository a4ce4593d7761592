"""Shot-parallel FWI gradients over several processes (one GPU each).

The path shards naturally by shot: each rank computes the summed gradient of
its own shots with the engine, then one all-reduce adds the three gradient
grids (and the per-shot misfits are gathered).  This is the only exchange of
an FWI iteration (the reference runs shots sequentially in one process,
CUDA_week2/fd_wave_model.cu:484, 777).

Works with any torch.distributed backend: NCCL between GPUs, gloo on CPU
(used by the tests).  The gradient function is injected, so the host logic is
testable without a GPU.
"""
from __future__ import annotations

from typing import Callable, Sequence

import numpy as np


def shard_shots(shots: Sequence[int], rank: int, world: int) -> list[int]:
    """Round-robin shard: every shot lands on exactly one rank."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("bad rank/world")
    return list(shots)[rank::world]


def allreduce_sum(arrays, device=None):
    """Element-wise sum of a list of float64 arrays over all ranks."""
    import torch
    import torch.distributed as dist
    flat = np.concatenate([np.ravel(a) for a in arrays]).astype(np.float64)
    t = torch.from_numpy(flat)
    if device is not None:
        t = t.to(device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    out = t.cpu().numpy()
    res, o = [], 0
    for a in arrays:
        n = np.size(a)
        res.append(out[o:o + n].reshape(np.shape(a)))
        o += n
    return res


def gather_misfits(shots: Sequence[int], misfit: Sequence[float], nshots_total: int, device=None):
    """Per-shot misfits of all ranks placed at their shot ids."""
    full = np.zeros(nshots_total)
    full[list(shots)] = misfit
    return allreduce_sum([full], device)[0]


def distributed_gradient(grad_fn: Callable, shots: Sequence[int], nshots_total: int, rank: int,
                         world: int, device=None):
    """grad_fn(my_shots) -> ((g_lam, g_mu, g_rho) summed over my_shots, misfit[len(my_shots)]).
    Returns the gradient summed over all shots of all ranks and the full misfit vector."""
    mine = shard_shots(shots, rank, world)
    if mine:
        g, mis = grad_fn(mine)
    else:
        g, mis = None, np.zeros(0)
    if g is None:  # a rank without shots still joins the collectives
        g = grad_fn(None)[0]
    total = allreduce_sum(list(g), device)
    misfit = gather_misfits(mine, mis, nshots_total, device)
    return tuple(total), misfit
