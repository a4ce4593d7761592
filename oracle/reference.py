"""Binding of the reference's own CPU path, compiled by ``oracle/build.py``
into ``oracle/_ref/libfwi_ref.so`` (test infrastructure only; available where
the reference sources were present at build time).

Functions mirror ``oracle.oracle``; they return None-raising errors when the
library is absent so callers can skip.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build as _build

dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int)


class RefCall(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("nt", "nzt", "nxt", "fpad", "ppad", "fsurf", "fdorder", "npml")] + [
        ("dt", C.c_double), ("dx", C.c_double), ("dz", C.c_double), ("hc", C.c_double * 7)]


_lib = None


class ReferenceUnavailable(RuntimeError):
    pass


def available() -> bool:
    try:
        lib()
        return True
    except ReferenceUnavailable:
        return False


def lib():
    global _lib
    if _lib is None:
        path = _build.build_ref()
        if path is None or not path.exists():
            if _build.REF_SO.exists():
                path = _build.REF_SO
            else:
                raise ReferenceUnavailable("reference sources not present; oracle/_ref not built")
        try:
            L = C.CDLL(str(path))
        except OSError as e:  # e.g. a library built for another architecture
            raise ReferenceUnavailable(str(e))
        L.ref_holberg.argtypes = [C.c_int, C.c_int, dp]
        L.ref_holberg.restype = None
        L.ref_cpml.argtypes = [C.c_int] + [C.c_double] * 7 + [dp] * 6
        L.ref_cpml.restype = None
        L.ref_average.argtypes = [C.c_int, C.c_int] + [dp] * 6
        L.ref_average.restype = None
        L.ref_wavelet.argtypes = [dp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]
        L.ref_wavelet.restype = None
        PP = C.POINTER(dp)
        L.ref_forward.argtypes = [C.c_int, C.POINTER(RefCall), PP, PP, PP, PP, C.c_int, ip, ip, ip, ip,
                                  dp, C.c_int, ip, ip, ip, ip, dp, ip, PP]
        L.ref_adjoint.argtypes = [C.c_int, C.POINTER(RefCall), PP, PP, PP, PP, C.c_int, ip, ip, ip, ip,
                                  dp, ip, PP, dp, dp, dp]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(dp)


def _i(a):
    return a.ctypes.data_as(ip)


def _pp(arrs):
    t = (dp * len(arrs))(*[_d(a) for a in arrs])
    return t


def holberg(fdorder, max_rel_err=1):
    hc = np.zeros(7)
    lib().ref_holberg(fdorder, max_rel_err, _d(hc))
    return hc


def cpml(npml, dh, fpml, npower, kmax, rcoef, damp, dt):
    n = 2 * (npml + 1)
    arr = [np.zeros(n) for _ in range(6)]
    lib().ref_cpml(npml, dh, fpml, npower, kmax, rcoef, damp, dt, *[_d(a) for a in arr])
    return dict(zip(("a", "b", "K", "a_half", "b_half", "K_half"), arr))


def average(lam, mu, rho):
    nzt, nxt = mu.shape
    a = [np.ascontiguousarray(x, np.float64).copy() for x in (lam, mu, rho)]
    out = [np.zeros((nzt - 1, nxt - 1)) for _ in range(3)]
    lib().ref_average(nzt, nxt, *[_d(x) for x in a], *[_d(o) for o in out])
    return out


def wavelet(nt, dt, amp, fc, ts=0.0, shape=1):
    s = np.zeros(nt)
    lib().ref_wavelet(_d(s), nt, dt, amp, fc, ts, shape)
    return s


def _call(p):
    c = RefCall()
    for k in ("nt", "nzt", "nxt", "fpad", "ppad", "fsurf", "fdorder", "npml"):
        setattr(c, k, int(getattr(p, k)))
    c.dt, c.dx, c.dz = p.dt, p.dx, p.dz
    for i in range(7):
        c.hc[i] = float(p.hc[i])
    return c


def _state(p):
    tp = 2 * (p.npml + 1)
    wave = [np.zeros((p.nzt, p.nxt)) for _ in range(6)]
    mem = [np.zeros((p.nzt, tp)), np.zeros((tp, p.nxt)), np.zeros((p.nzt, tp)), np.zeros((tp, p.nxt)),
           np.zeros((p.nzt, tp)), np.zeros((p.nzt, tp)), np.zeros((tp, p.nxt)), np.zeros((tp, p.nxt))]
    return wave, mem


def _mats(p, lam, mu, rho):
    lam = p.lam if lam is None else lam
    mu = p.mu if mu is None else mu
    rho = p.rho if rho is None else rho
    lam = np.ascontiguousarray(lam, np.float64)
    mu = np.ascontiguousarray(mu, np.float64)
    return [lam, mu] + average(lam, mu, rho)


def _fwi(p, fwinv):
    return np.array([int(fwinv), p.fwi_dt, p.fwi_dx, p.fwi_dz, p.x1, p.x2, p.z1, p.z2], np.int32)


def forward(p, shot=0, fwinv=False, lam=None, mu=None, rho=None):
    """forward_kernel_PSV (fdorder 2 only)."""
    if p.fdorder != 2:
        raise ValueError("the reference implements fdorder 2 only")
    wave, mem = _state(p)
    mats = _mats(p, lam, mu, rho)
    cp = [np.ascontiguousarray(p.cpml[k], np.float64) for k in ("a", "b", "K", "a_half", "b_half", "K_half")]
    s = [np.ascontiguousarray(a, np.int32) for a in (p.src_x, p.src_z, p.src_comp, p.src_shot)]
    r = [np.ascontiguousarray(a, np.int32) for a in (p.rec_x, p.rec_z, p.rec_comp, p.rec_shot)]
    sig = np.ascontiguousarray(p.src_signal, np.float64)
    recs = np.zeros((max(p.nrec, 1), p.nt))
    store = [np.zeros((p.nft, p.nfz, p.nfx)) for _ in range(5)] if fwinv else [np.zeros(1)] * 5
    f = _fwi(p, fwinv)
    rc = lib().ref_forward(shot, C.byref(_call(p)), _pp(wave), _pp(mem), _pp(mats), _pp(cp), len(s[0]),
                           *[_i(a) for a in s], _d(sig), len(r[0]), *[_i(a) for a in r], _d(recs),
                           _i(f), _pp(store))
    if rc != 0:
        raise ValueError(f"ref_forward failed ({rc})")
    names = ("vx", "vz", "sxx", "szx", "szz", "We")
    out = dict(zip(names, wave))
    out.update(zip(("mem_vx_x", "mem_vx_z", "mem_vz_x", "mem_vz_z", "mem_sxx_x", "mem_szx_x",
                    "mem_szz_z", "mem_szx_z"), mem))
    out["rec"] = recs[: p.nrec]
    out["store"] = dict(zip(("vx", "vz", "sxx", "szx", "szz"), store)) if fwinv else None
    return out


def adjoint(p, shot, residual, store, lam=None, mu=None, rho=None):
    """adjoint_kernel_PSV (fdorder 2 only), residual injected at the receivers."""
    if p.fdorder != 2:
        raise ValueError("the reference implements fdorder 2 only")
    wave, mem = _state(p)
    mats = _mats(p, lam, mu, rho)
    cp = [np.ascontiguousarray(p.cpml[k], np.float64) for k in ("a", "b", "K", "a_half", "b_half", "K_half")]
    r = [np.ascontiguousarray(a, np.int32) for a in (p.rec_x, p.rec_z, p.rec_comp, p.rec_shot)]
    res = np.ascontiguousarray(residual, np.float64)
    st = [np.ascontiguousarray(store[k], np.float64) for k in ("vx", "vz", "sxx", "szx", "szz")]
    g = [np.zeros((p.nfz, p.nfx)) for _ in range(3)]
    f = _fwi(p, True)
    rc = lib().ref_adjoint(shot, C.byref(_call(p)), _pp(wave), _pp(mem), _pp(mats), _pp(cp), len(r[0]),
                           *[_i(a) for a in r], _d(res), _i(f), _pp(st), *[_d(x) for x in g])
    if rc != 0:
        raise ValueError(f"ref_adjoint failed ({rc})")
    out = dict(zip(("vx", "vz", "sxx", "szx", "szz", "We"), wave))
    out.update(grad_lam=g[0], grad_mu=g[1], grad_rho=g[2])
    return out
