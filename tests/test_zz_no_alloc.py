"""fwi_psv_misfit_noalloc: the allocation-free residual/misfit entry point.

It serves callers that cannot allocate device memory where they evaluate the
misfit (an application whose HBM is reserved by its own pool allocator, or a
time-critical loop where cudaMalloc/cudaFree would synchronise the device).
The test feeds it the synthetic seismograms produced by the engine's own
forward entry point (fwi_psv_forward) and checks, on two calls in a row, that
its misfit equals the engine's and its residual equals syn - obs.  The file
name makes pytest collect it last.
"""
import ctypes as C

import numpy as np
import pytest

from cuda_fwi_gb300 import _capi
from cuda_fwi_gb300 import problem as P
from cuda_fwi_gb300.engine import Engine
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _case():
    p = P.small(fdorder=4, nx=50, nz=36, nt=160, npml=8, nrec=9, perturb=0.04, seed=4)
    t = P.small(fdorder=4, nx=50, nz=36, nt=160, npml=8, nrec=9, perturb=0.04, seed=14)
    return p, O.forward(t, 0)["rec"]


def test_noalloc_misfit_matches_engine_on_two_calls():
    import torch
    p, obs = _case()
    with Engine(p) as eng:
        rec, mis = eng.forward([0], obs)  # the existing entry point
    rows = O.shot_rows(p, 0)
    dev = torch.device("cuda", 0)
    syn32 = torch.tensor(rec[rows], dtype=torch.float32, device=dev)  # engine output, exact in FP32
    obs32 = torch.tensor(obs[rows].astype(np.float32), device=dev)    # the engine's FP32 rounding
    resid = torch.empty_like(syn32)
    want_resid = (syn32.double() - obs32.double()).float()
    stream = torch.cuda.current_stream(dev).cuda_stream
    L = _capi.lib()
    for call in range(2):
        resid.fill_(float("nan"))
        m = C.c_double(-1.0)
        st = L.fwi_psv_misfit_noalloc(C.c_void_p(syn32.data_ptr()), C.c_void_p(obs32.data_ptr()),
                                      len(rows), p.nt, p.dt, C.c_void_p(resid.data_ptr()),
                                      C.byref(m), C.c_void_p(stream))
        assert st == 0, L.fwi_psv_last_error()
        # same per-trace FP64 partial sums, summed in trace order
        assert m.value == pytest.approx(float(mis[0]), rel=1e-12), call
        assert torch.equal(resid, want_resid), call


def test_noalloc_rejects_more_traces_than_its_scratch():
    import torch
    L = _capi.lib()
    buf = torch.zeros(4, device="cuda")
    m = C.c_double()
    st = L.fwi_psv_misfit_noalloc(C.c_void_p(buf.data_ptr()), C.c_void_p(buf.data_ptr()), 65537, 1, 1e-3,
                                  C.c_void_p(buf.data_ptr()), C.byref(m), None)
    assert st == -1  # FWI_ERR_INVALID, raised before anything is launched
    assert b"FWI_NOALLOC_MAX_ROWS" in L.fwi_psv_last_error()
