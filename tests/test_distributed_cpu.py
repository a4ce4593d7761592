"""Multi-rank shot-parallel gradient (host logic) on CPU with gloo, world 2.

Each rank computes the gradients of its shard of shots (here with the CPU
oracle standing in for a GPU) and one all-reduce sums them; the result must
equal the single-process sum over all shots.  A rank that raises before the
collective is detected by the others through the process-group timeout.
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as tmp

from cuda_fwi_gb300 import distributed as D


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _problem():
    from cuda_fwi_gb300 import problem as P
    return P.small(fdorder=4, nx=36, nz=28, nt=90, npml=6, nshots=3, nrec=4, perturb=0.05, seed=3)


def _grad_fn_factory(p, obs):
    from oracle import oracle as O

    def grad_fn(shots):
        if shots is None:
            z = np.zeros((p.nfz, p.nfx))
            return (z, z.copy(), z.copy()), np.zeros(0)
        tot = [np.zeros((p.nfz, p.nfx)) for _ in range(3)]
        mis = []
        for s in shots:
            J, g, _, _ = O.gradient(p, obs, s)
            for i in range(3):
                tot[i] += g[i]
            mis.append(J)
        return tuple(tot), np.array(mis)
    return grad_fn


def _worker(rank, world, port, q, fail_rank):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import datetime
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=20))
    try:
        p = _problem()
        obs = np.zeros((p.nrec, p.nt))
        if rank == fail_rank:
            raise RuntimeError("rank failed before the collective")
        g, mis = D.distributed_gradient(_grad_fn_factory(p, obs), list(range(p.nshots)), p.nshots,
                                        rank, world)
        q.put((rank, "ok", [x.copy() for x in g], mis.copy()))
    except Exception as e:
        q.put((rank, "error", repr(e), None))
    finally:
        try:
            dist.destroy_process_group()
        except Exception:
            pass


def _run(world, fail_rank=-1):
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q, fail_rank)) for r in range(world)]
    for pr in procs:
        pr.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for pr in procs:
        pr.join(timeout=60)
    return sorted(out, key=lambda t: t[0])


def test_shard_covers_every_shot_once():
    shots = list(range(11))
    parts = [D.shard_shots(shots, r, 3) for r in range(3)]
    assert sorted(sum(parts, [])) == shots
    with pytest.raises(ValueError):
        D.shard_shots(shots, 3, 3)


def test_two_rank_gradient_equals_single_process():
    res = _run(2)
    assert all(r[1] == "ok" for r in res), res
    p = _problem()
    obs = np.zeros((p.nrec, p.nt))
    g_all, mis_all = _grad_fn_factory(p, obs)(list(range(p.nshots)))
    for rank, _, g, mis in res:
        for i in range(3):
            np.testing.assert_allclose(g[i], g_all[i], rtol=1e-12, atol=0)
        np.testing.assert_allclose(mis, mis_all, rtol=1e-12)


def test_failed_rank_is_reported_not_hung():
    res = _run(2, fail_rank=1)
    status = {r[0]: r[1] for r in res}
    assert status[1] == "error"
    # the surviving rank's collective ends with an error (peer gone), not a hang
    assert status[0] == "error"
