"""ctypes binding of ``include/fwi_psv.h`` (libfwi_psv.so, built in-tree).

There is no CPU fallback: if the library is missing, importing the engine
raises ``FwiLibraryMissing``.  Host-side helpers (Holberg table, CPML
profile, grid padding, Ricker wavelet, material averaging) run on the CPU
inside the same library.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_lib" / "libfwi_psv.so"

ABI_VERSION = 2  # FWI_PSV_ABI_VERSION of include/fwi_psv.h this binding follows
FWI_OK = 0
ERRORS = {
    -1: "FWI_ERR_INVALID", -2: "FWI_ERR_UNSUPPORTED", -3: "FWI_ERR_NOMEM", -4: "FWI_ERR_CUDA",
    -5: "FWI_ERR_STATE", -6: "FWI_ERR_DIVERGED", -7: "FWI_ERR_NOFORWARD", -8: "FWI_ERR_NODEVICE",
    -9: "FWI_ERR_IO",
}
FWI_STORE_FULL, FWI_STORE_BINOMIAL, FWI_STORE_RANDOM = 0, 1, 2
FWI_GRAD_REFERENCE, FWI_GRAD_EXACT = 0, 1
FWI_FWD_KEEP, FWI_FWD_RESIDENT_OBS = 1, 2


class FwiLibraryMissing(RuntimeError):
    pass


class FwiError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str):
        self.status = status
        self.code = ERRORS.get(status, str(status))
        super().__init__(f"{where}: {self.code} ({detail})")


dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int)


class Desc(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("nt", "nzt", "nxt", "fpad", "ppad", "npml", "fsurf", "fdorder")] + [
        ("dt", C.c_double), ("dx", C.c_double), ("dz", C.c_double), ("hc", C.c_double * 7),
        ("a", dp), ("b", dp), ("K", dp), ("a_half", dp), ("b_half", dp), ("K_half", dp)]


class Stats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("launches", "forward_steps", "recompute_steps",
                                          "adjoint_steps", "device_bytes", "snapshots")] + [
        ("last_forward_ms", C.c_double), ("last_backward_ms", C.c_double),
        ("h2d_bytes", C.c_int64), ("d2h_bytes", C.c_int64), ("batch", C.c_int64)]


class Layout(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("nt", "nzt", "nxt", "fpad", "ppad", "npml", "fsurf", "fdorder",
                                        "fwi_dt", "fwi_dx", "fwi_dz", "x1", "x2", "z1", "z2", "nfz", "nfx",
                                        "device")]


class FwiOpts(C.Structure):
    _fields_ = [("max_iter", C.c_int), ("max_error", C.c_double), ("step_length", C.c_double),
                ("order", C.c_int), ("trial_misfit", C.c_int), ("precondition", C.c_int),
                ("true_lam", dp), ("true_mu", dp), ("true_rho", dp), ("restart_step", C.c_double),
                ("resume_file", C.c_char_p)]


class FwiIter(C.Structure):
    _fields_ = [("misfit", C.c_double), ("step_length", C.c_double), ("trials", C.c_int), ("status", C.c_int),
                ("model_error", C.c_double), ("seconds", C.c_double)]


TRIAL_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_double, dp)
ALLOC_FN = C.CFUNCTYPE(C.c_void_p, C.c_size_t, C.c_void_p)
FREE_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_void_p)


class Model(C.Structure):
    _fields_ = [("grid", Desc), ("lam", dp), ("mu", dp), ("rho", dp), ("nsrc", C.c_int), ("src_x", ip),
                ("src_z", ip), ("src_signal", dp), ("nrec", C.c_int), ("rec_x", ip), ("rec_z", ip)]

_lib = None

# (name, restype, argtypes); every int-returning function is a status call.
_SIGS = {
    "fwi_psv_abi_version": (C.c_int, []),
    "fwi_psv_strerror": (C.c_char_p, [C.c_int]),
    "fwi_psv_last_error": (C.c_char_p, []),
    "fwi_psv_holberg": (C.c_int, [C.c_int, C.c_int, dp]),
    "fwi_psv_cpml_profile": (C.c_int, [C.c_int] + [C.c_double] * 7 + [dp] * 6),
    "fwi_psv_total_grid": (C.c_int, [C.c_int] * 5 + [ip] * 4),
    "fwi_psv_wavelet": (C.c_int, [dp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]),
    "fwi_psv_average_parameters": (C.c_int, [C.c_int, C.c_int, dp, dp, dp, dp, dp]),
    "fwi_psv_create": (C.c_int, [C.POINTER(Desc), C.c_int, C.POINTER(C.c_void_p)]),
    "fwi_psv_destroy": (C.c_int, [C.c_void_p]),
    "fwi_psv_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fwi_psv_set_model": (C.c_int, [C.c_void_p, dp, dp, dp, dp, dp]),
    "fwi_psv_set_model_lmr": (C.c_int, [C.c_void_p, dp, dp, dp]),
    "fwi_psv_set_sources": (C.c_int, [C.c_void_p, C.c_int, ip, ip, ip, ip, dp]),
    "fwi_psv_set_receivers": (C.c_int, [C.c_void_p, C.c_int, ip, ip, ip, ip]),
    "fwi_psv_set_fwi": (C.c_int, [C.c_void_p] + [C.c_int] * 7),
    "fwi_psv_set_strategy": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_size_t]),
    "fwi_psv_set_gradient_mode": (C.c_int, [C.c_void_p, C.c_int]),
    "fwi_psv_set_exec": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]),
    "fwi_psv_gradient": (C.c_int, [C.c_void_p, C.c_int, ip, dp, dp, dp, dp, dp, C.c_int]),
    "fwi_psv_checkpoint_plan": (C.c_int, [C.c_int, C.c_int, ip, C.c_int, ip, C.POINTER(C.c_longlong)]),
    "fwi_psv_forward": (C.c_int, [C.c_void_p, C.c_int, ip, dp, dp, dp, C.c_int]),
    "fwi_psv_backward": (C.c_int, [C.c_void_p, dp, dp, dp, C.c_int]),
    "fwi_psv_energy": (C.c_int, [C.c_void_p, C.c_int, dp, dp]),
    "fwi_psv_wavefield": (C.c_int, [C.c_void_p, C.c_int, C.c_int, dp, dp, dp, dp, dp]),
    "fwi_psv_get_stats": (C.c_int, [C.c_void_p, C.POINTER(Stats)]),
    "fwi_psv_time_kernels": (C.c_int, [C.c_void_p, C.c_int, dp]),
    "fwi_psv_set_wait_limit": (C.c_int, [C.c_void_p, C.c_double]),
    "fwi_psv_set_device_allocator": (C.c_int, [ALLOC_FN, FREE_FN, C.c_void_p]),
    "fwi_psv_debug_stall_next": (C.c_int, [C.c_void_p]),
    "fwi_psv_misfit_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_double,
                                         C.c_void_p, dp, C.c_void_p]),
    "fwi_psv_set_snapshots": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "fwi_psv_snapshot": (C.c_int, [C.c_void_p, C.c_int, C.c_int, dp]),
    "fwi_psv_get_layout": (C.c_int, [C.c_void_p, C.POINTER(Layout)]),
    "fwi_psv_multi_create": (C.c_int, [C.c_int, C.POINTER(Model), C.c_int, C.POINTER(C.c_void_p)]),
    "fwi_psv_multi_destroy": (C.c_int, [C.c_void_p]),
    "fwi_psv_multi_set_exec": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "fwi_psv_multi_forward": (C.c_int, [C.c_void_p, C.POINTER(dp)]),
    "fwi_psv_multi_gradient": (C.c_int, [C.c_void_p, C.POINTER(dp), dp, C.POINTER(dp), C.POINTER(dp),
                                         C.POINTER(dp)]),
    "fwi_psv_multi_tuning": (C.c_int, [C.c_void_p, C.c_int, ip, dp]),
    "fwi_psv_multi_get_stats": (C.c_int, [C.c_void_p, C.POINTER(Stats)]),
    "fwi_psv_set_model_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "fwi_psv_set_precondition": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double]),
    "fwi_psv_misfit": (C.c_int, [C.c_void_p, C.c_int, ip, dp, dp, C.c_int]),
    "fwi_psv_fwi_run": (C.c_int, [C.c_void_p, C.POINTER(FwiOpts), C.c_int, ip, dp, dp, dp, dp,
                                  C.POINTER(FwiIter), ip]),
    "fwi_psv_calc_opt_step": (C.c_double, [dp, dp]),
    "fwi_psv_step_search": (C.c_int, [C.c_double, C.c_double, TRIAL_FN, C.c_void_p, dp, ip, ip]),
    "fwi_psv_forward_kernel": (C.c_int, [C.c_int] * 6 + [C.c_double] * 3 + [C.c_int, C.c_int, dp, C.c_int]
                               + [dp] * 6 + [dp] * 5 + [C.c_int] + [dp] * 6 + [dp] * 8
                               + [C.c_int, ip, ip, ip, dp, ip] + [C.c_int, ip, ip, ip, dp, ip]
                               + [C.c_int] * 8 + [dp] * 5),
    "fwi_psv_adjoint_kernel": (C.c_int, [C.c_int] * 6 + [C.c_double] * 3 + [C.c_int, C.c_int, dp, C.c_int]
                               + [dp] * 6 + [dp] * 5 + [C.c_int] + [dp] * 6 + [dp] * 8
                               + [C.c_int, ip, ip, ip, dp, ip]
                               + [C.c_int] * 8 + [dp] * 5 + [dp] * 3),
}


def lib():
    """Load libfwi_psv.so (raises FwiLibraryMissing if it has not been built)."""
    global _lib
    if _lib is None:
        path = Path(os.environ.get("FWI_PSV_LIB", LIB_PATH))
        if not path.exists():
            raise FwiLibraryMissing(
                f"{path} not found: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(str(path))
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        if L.fwi_psv_abi_version() != ABI_VERSION:
            raise FwiLibraryMissing(f"{path} has ABI version {L.fwi_psv_abi_version()}, this binding "
                                    f"{ABI_VERSION}: rebuild it")
        _lib = L
    return _lib


def exported_symbols():
    return list(_SIGS)


def check(status: int, where: str) -> None:
    if status != FWI_OK:
        detail = lib().fwi_psv_last_error().decode(errors="replace")
        raise FwiError(status, where, detail)


def pd(a):
    """double* of a C-contiguous float64 array (None -> NULL)."""
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous, "need C-contiguous float64"
    return a.ctypes.data_as(dp)


def pi(a):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags.c_contiguous, "need C-contiguous int32"
    return a.ctypes.data_as(ip)


# ---- host helpers --------------------------------------------------------

def holberg(fdorder: int, max_rel_err: int = 1) -> np.ndarray:
    hc = np.zeros(7)
    check(lib().fwi_psv_holberg(fdorder, max_rel_err, pd(hc)), "holberg")
    return hc


def cpml_profile(npml, dh, fpml, npower, k_max_pml, rcoef, damp_v_pml, dt):
    n = 2 * (npml + 1)
    arr = [np.zeros(n) for _ in range(6)]
    check(lib().fwi_psv_cpml_profile(npml, dh, fpml, npower, k_max_pml, rcoef, damp_v_pml, dt,
                                     *[pd(a) for a in arr]), "cpml_profile")
    return dict(zip(("a", "b", "K", "a_half", "b_half", "K_half"), arr))


def total_grid(nx, nz, fdorder, npml, fsurf):
    out = [C.c_int() for _ in range(4)]
    check(lib().fwi_psv_total_grid(nx, nz, fdorder, npml, int(fsurf), *[C.byref(o) for o in out]),
          "total_grid")
    fpad, ppad, nxt, nzt = (o.value for o in out)
    return fpad, ppad, nxt, nzt


def wavelet(nt, dt, amp, fc, ts=0.0, shape=1):
    s = np.zeros(nt)
    check(lib().fwi_psv_wavelet(pd(s), nt, dt, amp, fc, ts, shape), "wavelet")
    return s


def checkpoint_plan(nsteps: int, slots: int):
    """The binomial schedule as a list of (kind, a, b) and its advance cost."""
    n, cost = C.c_int(), C.c_longlong()
    lib().fwi_psv_checkpoint_plan(nsteps, slots, None, 0, C.byref(n), C.byref(cost))
    buf = np.zeros((max(n.value, 1), 3), np.int32)
    check(lib().fwi_psv_checkpoint_plan(nsteps, slots, pi(buf), n.value, C.byref(n), C.byref(cost)),
          "checkpoint_plan")
    return [tuple(int(v) for v in row) for row in buf[: n.value]], int(cost.value)


def average_parameters(mu: np.ndarray, rho: np.ndarray):
    nzt, nxt = mu.shape
    out = [np.zeros((nzt - 1, nxt - 1)) for _ in range(3)]
    check(lib().fwi_psv_average_parameters(nzt, nxt, pd(np.ascontiguousarray(mu, np.float64)),
                                           pd(np.ascontiguousarray(rho, np.float64)),
                                           *[pd(o) for o in out]), "average_parameters")
    return out  # mu_zx, rho_zp, rho_xp
