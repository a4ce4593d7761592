"""Device memory through an injected allocator (fwi_psv_set_device_allocator).

* A pool allocator (PyTorch's caching allocator, counted): the engine's
  results equal those of cudaMalloc'd memory bit for bit, every buffer it got
  is handed back by the time the engine is closed, and buffers made before a
  change of allocator go back to the allocator that made them.
* A failing allocator (host-side fault injection: it returns NULL after a few
  allocations): creating or growing an engine, and the FWI loop's buffers,
  give FWI_ERR_NOMEM; the engine that hit it stays usable once memory is
  available again, and nothing leaks.
No GPU fault is involved: the failure is made on the host.
"""
import numpy as np
import pytest

from cuda_fwi_gb300 import _capi
from cuda_fwi_gb300 import allocator as A
from cuda_fwi_gb300 import problem as P
from cuda_fwi_gb300.engine import Engine
from oracle import oracle as O

pytestmark = pytest.mark.gpu


class Pool:
    """torch's caching allocator, counted; fails once `budget` allocations are spent."""

    def __init__(self, budget=None):
        import torch
        self.torch = torch
        self.budget = budget
        self.live = {}
        self.calls = 0

    def alloc(self, nbytes):
        self.calls += 1
        if self.budget is not None:
            if self.budget <= 0:
                return 0
            self.budget -= 1
        ptr = self.torch.cuda.caching_allocator_alloc(nbytes)
        self.live[ptr] = nbytes
        return ptr

    def free(self, ptr):
        assert ptr in self.live, "freed a pointer this pool did not hand out"
        del self.live[ptr]
        self.torch.cuda.caching_allocator_delete(ptr)


def _case():
    p = P.small(fdorder=4, nx=60, nz=40, nt=120, npml=6, nshots=2, nrec=6, perturb=0.04, seed=5)
    t = P.small(fdorder=4, nx=60, nz=40, nt=120, npml=6, nshots=2, nrec=6, perturb=0.04, seed=15)
    obs = np.zeros((p.nrec, p.nt))
    for s in range(2):
        rows = O.shot_rows(t, s)
        obs[rows] = O.forward(t, s)["rec"][rows]
    return p, obs


def _run(p, obs, shots=(0, 1)):
    with Engine(p) as eng:
        eng.set_strategy("binomial", snapshots=6)
        g, mis = eng.gradient(list(shots), obs)
    return g, mis


@pytest.fixture(autouse=True)
def _restore_allocator():
    yield
    A.set_device_allocator(None, None)


def test_pool_allocator_same_results_and_nothing_leaks():
    p, obs = _case()
    want = _run(p, obs)
    pool = Pool()
    A.set_device_allocator(pool.alloc, pool.free)
    got = _run(p, obs)
    assert pool.calls > 0 and not pool.live, (pool.calls, len(pool.live))
    for a, b in zip(got[0], want[0]):
        assert np.array_equal(a, b)
    assert np.array_equal(got[1], want[1])
    # buffers made under the pool go back to it after the allocator is reset
    eng = Engine(p)
    try:
        eng.set_strategy("binomial", snapshots=6)
        eng.gradient([0], obs)
        n_live = len(pool.live)
        assert n_live > 0
        A.set_device_allocator(None, None)
        eng.gradient([0, 1], obs)  # grows its buffers with cudaMalloc, returns the pool's
    finally:
        eng.close()
    assert not pool.live


def test_failing_allocator_gives_nomem_and_engine_recovers():
    p, obs = _case()
    want = _run(p, obs)
    # creation runs out
    A.set_device_allocator(*_spent(Pool(budget=2)))
    with pytest.raises(_capi.FwiError) as ei:
        _run(p, obs)
    assert ei.value.code == "FWI_ERR_NOMEM"
    # an engine that runs out while growing its batch stays usable
    A.set_device_allocator(None, None)
    pool = Pool(budget=0)
    with Engine(p) as eng:
        eng.set_strategy("binomial", snapshots=6)
        A.set_device_allocator(pool.alloc, pool.free)
        with pytest.raises(_capi.FwiError) as ei:
            eng.gradient([0, 1], obs)
        assert ei.value.code == "FWI_ERR_NOMEM"
        A.set_device_allocator(None, None)
        g, mis = eng.gradient([0, 1], obs)
    assert not pool.live
    for a, b in zip(g, want[0]):
        assert np.array_equal(a, b)
    assert np.array_equal(mis, want[1])


def test_failing_allocator_in_the_fwi_loop():
    p, obs = _case()
    with Engine(p) as eng:
        eng.set_strategy("binomial", snapshots=6)
        eng.gradient([0, 1], obs)  # the engine's own buffers exist
        pool = Pool(budget=1)
        A.set_device_allocator(pool.alloc, pool.free)
        with pytest.raises(_capi.FwiError) as ei:
            eng.fwi_run([0, 1], obs, max_iter=1)
        assert ei.value.code == "FWI_ERR_NOMEM"
        A.set_device_allocator(None, None)
        _, log = eng.fwi_run([0, 1], obs, max_iter=1)
    assert not pool.live and len(log) == 1


def _spent(pool):
    return pool.alloc, pool.free
