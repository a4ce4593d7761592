"""Python binding of the CPU parity oracle (``oracle/fwi_oracle.c``).

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and the
CPU-baseline leg of bench.py, always as the checker.  The product never
imports it.

``problem`` arguments are duck-typed objects with the attributes of
``cuda_fwi_gb300.problem.Problem`` (grid, hc, cpml dict, lam/mu/rho,
acquisition arrays, FWI window).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int)


class Grid(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("nt", "nzt", "nxt", "fpad", "ppad", "npml", "fsurf", "fdorder")] + [
        ("dt", C.c_double), ("dx", C.c_double), ("dz", C.c_double), ("hc", C.c_double * 7)] + [
        (n, dp) for n in ("a", "b", "K", "a_half", "b_half", "K_half")]


class Medium(C.Structure):
    _fields_ = [(n, dp) for n in ("lam", "mu", "mu_zx", "rho_zp", "rho_xp")]


class Wave(C.Structure):
    _fields_ = [(n, dp) for n in ("vx", "vz", "sxx", "szx", "szz", "We", "mem_vx_x", "mem_vz_x",
                                  "mem_sxx_x", "mem_szx_x", "mem_vx_z", "mem_vz_z", "mem_szz_z",
                                  "mem_szx_z")]


class Seis(C.Structure):
    _fields_ = [("n", C.c_int), ("x", ip), ("z", ip), ("comp", ip), ("shot", ip)]


class Fwi(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("fwinv", "fwi_dt", "fwi_dx", "fwi_dz", "x1", "x2", "z1", "z2")] + [
        (n, dp) for n in ("vx", "vz", "sxx", "szx", "szz")]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(str(path))
        L.orc_holberg.argtypes = [C.c_int, C.c_int, dp]
        L.orc_cpml.argtypes = [C.c_int] + [C.c_double] * 7 + [dp] * 6
        L.orc_cpml.restype = None
        L.orc_average.argtypes = [C.c_int, C.c_int, dp, dp, dp, dp, dp, dp]
        L.orc_average.restype = None
        L.orc_wavelet.argtypes = [dp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]
        L.orc_wavelet.restype = None
        L.orc_total_grid.argtypes = [C.c_int] * 5 + [ip] * 4
        L.orc_total_grid.restype = None
        L.orc_forward.argtypes = [C.c_int, C.POINTER(Grid), C.POINTER(Medium), C.POINTER(Wave),
                                  C.POINTER(Seis), dp, C.POINTER(Seis), dp, C.POINTER(Fwi)]
        L.orc_adjoint.argtypes = [C.c_int, C.POINTER(Grid), C.POINTER(Medium), C.POINTER(Wave),
                                  C.POINTER(Seis), dp, C.POINTER(Fwi), dp, dp, dp]
        L.orc_l2_adjoint_sources.argtypes = [C.c_int, C.c_int, C.c_double, dp, dp, ip]
        L.orc_l2_adjoint_sources.restype = C.c_double
        L.orc_medium_average.argtypes = [C.c_int, C.c_int, dp, dp, dp, dp, dp, dp]
        L.orc_medium_average.restype = None
        L.orc_scale_gradients.argtypes = [C.c_int, dp, dp, C.c_double, C.c_double, C.c_double] + \
            [C.c_int] * 7 + [dp] * 3
        L.orc_scale_gradients.restype = None
        L.orc_grad_update.argtypes = [dp, dp, dp, C.c_int, C.c_int, C.c_double] + [C.c_int] * 8
        L.orc_grad_update.restype = None
        L.orc_calc_opt_step.argtypes = [dp, dp]
        L.orc_calc_opt_step.restype = C.c_double
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_set_threads.restype = C.c_int
        L.orc_gradient_ckpt.argtypes = [C.c_int, C.POINTER(Grid), C.POINTER(Medium), C.POINTER(Seis), dp,
                                        C.POINTER(Seis), dp, dp, dp, C.POINTER(Fwi), C.c_int, dp, dp, dp, dp,
                                        dp, dp]
        L.orc_exact_gradient.argtypes = [C.c_int, C.POINTER(Grid), dp, dp, dp, C.POINTER(Seis), dp,
                                         C.POINTER(Seis), dp, dp, dp, dp, dp]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(dp)


def _i(a):
    return a.ctypes.data_as(ip)


def holberg(fdorder, max_rel_err=1):
    hc = np.zeros(7)
    if lib().orc_holberg(fdorder, max_rel_err, _d(hc)) != 0:
        raise ValueError("order/error outside the table")
    return hc


def cpml(npml, dh, fpml, npower, kmax, rcoef, damp, dt):
    n = 2 * (npml + 1)
    arr = [np.zeros(n) for _ in range(6)]
    lib().orc_cpml(npml, dh, fpml, npower, kmax, rcoef, damp, dt, *[_d(a) for a in arr])
    return dict(zip(("a", "b", "K", "a_half", "b_half", "K_half"), arr))


def average(lam, mu, rho):
    nzt, nxt = mu.shape
    out = [np.zeros((nzt - 1, nxt - 1)) for _ in range(3)]
    lib().orc_average(nzt, nxt, _d(np.ascontiguousarray(lam)), _d(np.ascontiguousarray(mu)),
                      _d(np.ascontiguousarray(rho)), *[_d(o) for o in out])
    return out


def wavelet(nt, dt, amp, fc, ts=0.0, shape=1):
    s = np.zeros(nt)
    lib().orc_wavelet(_d(s), nt, dt, amp, fc, ts, shape)
    return s


def total_grid(nx, nz, fdorder, npml, fsurf):
    o = [C.c_int() for _ in range(4)]
    lib().orc_total_grid(nx, nz, fdorder, npml, int(fsurf), *[C.byref(v) for v in o])
    return tuple(v.value for v in o)


class setup_helpers:
    """The five problem-setup functions of the engine library's host code
    (same names and signatures as ``cuda_fwi_gb300._capi``), computed by the
    oracle instead: ``problem.use_setup_helpers(oracle.setup_helpers)`` builds
    problems in a process that never loads the engine library (the bench's
    reference arm).  Bit-identical results (tests/test_capi_host.py)."""

    total_grid = staticmethod(total_grid)

    @staticmethod
    def holberg(fdorder, max_rel_err=1):
        return holberg(fdorder, max_rel_err)

    @staticmethod
    def cpml_profile(npml, dh, fpml, npower, k_max_pml, rcoef, damp_v_pml, dt):
        return cpml(npml, dh, fpml, npower, k_max_pml, rcoef, damp_v_pml, dt)

    @staticmethod
    def wavelet(nt, dt, amp, fc, ts=0.0, shape=1):
        return wavelet(nt, dt, amp, fc, ts, shape)

    @staticmethod
    def average_parameters(mu, rho):
        return average(mu, mu, rho)  # the averages do not read lam


class _Ctx:
    """Keeps the numpy buffers behind the ctypes structs alive."""

    def __init__(self, p, lam=None, mu=None, rho=None, averaged=None):
        self.p = p
        self.cp = {k: np.ascontiguousarray(v, np.float64) for k, v in p.cpml.items()}
        g = Grid()
        for k in ("nt", "nzt", "nxt", "fpad", "ppad", "npml", "fsurf", "fdorder"):
            setattr(g, k, int(getattr(p, k)))
        g.dt, g.dx, g.dz = p.dt, p.dx, p.dz
        for i in range(7):
            g.hc[i] = float(p.hc[i])
        for k in ("a", "b", "K", "a_half", "b_half", "K_half"):
            setattr(g, k, _d(self.cp[k]))
        self.g = g
        lam = p.lam if lam is None else lam
        mu = p.mu if mu is None else mu
        rho = p.rho if rho is None else rho
        avg = average(lam, mu, rho) if averaged is None else [np.ascontiguousarray(a, np.float64) for a in averaged]
        self.mat = [np.ascontiguousarray(x, np.float64) for x in (lam, mu)] + avg
        m = Medium()
        for k, a in zip(("lam", "mu", "mu_zx", "rho_zp", "rho_xp"), self.mat):
            setattr(m, k, _d(a))
        self.m = m
        n, tp = p.nzt * p.nxt, 2 * (p.npml + 1)
        self.wave = {k: np.zeros((p.nzt, p.nxt)) for k in ("vx", "vz", "sxx", "szx", "szz", "We")}
        for k in ("mem_vx_x", "mem_vz_x", "mem_sxx_x", "mem_szx_x"):
            self.wave[k] = np.zeros((p.nzt, tp))
        for k in ("mem_vx_z", "mem_vz_z", "mem_szz_z", "mem_szx_z"):
            self.wave[k] = np.zeros((tp, p.nxt))
        w = Wave()
        for k, a in self.wave.items():
            setattr(w, k, _d(a))
        self.w = w
        del n

    @staticmethod
    def seis(x, z, comp, shot):
        arrs = [np.ascontiguousarray(a, np.int32) for a in (x, z, comp, shot)]
        s = Seis()
        s.n = len(arrs[0])
        s.x, s.z, s.comp, s.shot = (_i(a) for a in arrs)
        return s, arrs

    def fwi(self, fwinv, store=None):
        p = self.p
        f = Fwi()
        f.fwinv, f.fwi_dt, f.fwi_dx, f.fwi_dz = int(fwinv), p.fwi_dt, p.fwi_dx, p.fwi_dz
        f.x1, f.x2, f.z1, f.z2 = p.x1, p.x2, p.z1, p.z2
        if store is None and fwinv:
            store = {k: np.zeros((p.nft, p.nfz, p.nfx)) for k in ("vx", "vz", "sxx", "szx", "szz")}
        if store is not None:
            for k, a in store.items():
                setattr(f, k, _d(a))
        return f, store


def forward(p, shot=0, fwinv=False, lam=None, mu=None, rho=None, averaged=None):
    """orc_forward for one shot.  Returns dict(rec [nrec][nt], wave fields, We,
    CPML memory, store (5 arrays [nft][nfz][nfx]) when fwinv).  `averaged` =
    (mu_zx, rho_zp, rho_xp) replaces the averages of lam/mu/rho."""
    ctx = _Ctx(p, lam, mu, rho, averaged)
    src, keep1 = ctx.seis(p.src_x, p.src_z, p.src_comp, p.src_shot)
    rec, keep2 = ctx.seis(p.rec_x, p.rec_z, p.rec_comp, p.rec_shot)
    sig = np.ascontiguousarray(p.src_signal, np.float64) if p.nsrc else np.zeros((1, p.nt))
    recs = np.zeros((max(p.nrec, 1), p.nt))
    f, store = ctx.fwi(fwinv)
    rc = lib().orc_forward(shot, C.byref(ctx.g), C.byref(ctx.m), C.byref(ctx.w), C.byref(src),
                           _d(sig), C.byref(rec), _d(recs), C.byref(f))
    if rc != 0:
        raise ValueError(f"orc_forward failed ({rc})")
    out = dict(ctx.wave)
    out["rec"] = recs[: p.nrec]
    out["store"] = store
    return out


def adjoint(p, shot, residual, store, lam=None, mu=None, rho=None):
    """orc_adjoint for one shot with the residual [nrec][nt] injected at the
    receivers of `shot`.  Returns dict(grad_lam, grad_mu, grad_rho, fields)."""
    ctx = _Ctx(p, lam, mu, rho)
    adj, keep = ctx.seis(p.rec_x, p.rec_z, p.rec_comp, p.rec_shot)
    res = np.ascontiguousarray(residual, np.float64)
    f, _ = ctx.fwi(1, store)
    g = [np.zeros((p.nfz, p.nfx)) for _ in range(3)]
    rc = lib().orc_adjoint(shot, C.byref(ctx.g), C.byref(ctx.m), C.byref(ctx.w), C.byref(adj),
                           _d(res), C.byref(f), *[_d(x) for x in g])
    if rc != 0:
        raise ValueError(f"orc_adjoint failed ({rc})")
    out = dict(ctx.wave)
    out.update(grad_lam=g[0], grad_mu=g[1], grad_rho=g[2])
    return out


def residual(rec, obs, dt, rows):
    """calculate_l2_adjoint_sources over the given receiver rows."""
    r = np.ascontiguousarray(rec[rows], np.float64).copy()
    o = np.ascontiguousarray(obs[rows], np.float64)
    blow = C.c_int()
    J = lib().orc_l2_adjoint_sources(len(rows), r.shape[1], dt, _d(r), _d(o), C.byref(blow))
    full = np.zeros_like(rec)
    full[rows] = r
    return J, full, bool(blow.value)


def shot_rows(p, shot):
    return np.nonzero((np.asarray(p.rec_shot) == shot) & (np.asarray(p.rec_comp) == 2))[0]


def gradient(p, obs, shot=0, lam=None, mu=None, rho=None):
    """Forward (with storage) -> residual -> adjoint for one shot, the reference's
    CPU FWI sequence (fd_wave_model.cu:791-859).  Returns (J, grads, fwd, adj)."""
    fw = forward(p, shot, True, lam, mu, rho)
    rows = shot_rows(p, shot)
    J, res, _ = residual(fw["rec"], obs, p.dt, rows)
    ad = adjoint(p, shot, res, fw["store"], lam, mu, rho)
    return J, (ad["grad_lam"], ad["grad_mu"], ad["grad_rho"]), fw, ad


def set_threads(n):
    """Threads of the oracle's cell loops (results do not depend on it)."""
    return lib().orc_set_threads(int(n))


def ckpt_interval(p):
    """Steps between the stored states of gradient_ckpt: about sqrt(nt x state
    / window frame), which balances the states against one segment's frames."""
    state = 5 * p.nzt * p.nxt + 8 * p.nxt * (p.npml + 1)
    frame = 5 * p.nfz * p.nfx
    return max(1, min(p.nt, int(round(np.sqrt(p.nt * state / frame)))))


def gradient_ckpt(p, obs, shot=0, interval=None, lam=None, mu=None, rho=None, residual=None):
    """The same result as gradient() bit for bit (forward, residual, adjoint of
    one shot) with the forward wavefield recomputed from a state every
    `interval` steps instead of stored: memory for a full-size shot.
    `residual` ([nrec][nt]) replaces the adjoint source syn - obs (the misfit
    is still computed from obs).
    Returns (J, (grad_lam, grad_mu, grad_rho), rec, We_fwd, We_adj)."""
    ctx = _Ctx(p, lam, mu, rho)
    src, keep1 = ctx.seis(p.src_x, p.src_z, p.src_comp, p.src_shot)
    rec, keep2 = ctx.seis(p.rec_x, p.rec_z, p.rec_comp, p.rec_shot)
    sig = np.ascontiguousarray(p.src_signal, np.float64) if p.nsrc else np.zeros((1, p.nt))
    ob = np.ascontiguousarray(obs, np.float64) if p.nrec else np.zeros((1, p.nt))
    recs = np.zeros((max(p.nrec, 1), p.nt))
    f = Fwi()
    f.fwinv, f.fwi_dt, f.fwi_dx, f.fwi_dz = 1, p.fwi_dt, p.fwi_dx, p.fwi_dz
    f.x1, f.x2, f.z1, f.z2 = p.x1, p.x2, p.z1, p.z2
    g = [np.zeros((p.nfz, p.nfx)) for _ in range(3)]
    wf, wa = np.zeros((p.nzt, p.nxt)), np.zeros((p.nzt, p.nxt))
    J = C.c_double()
    k = int(interval) if interval else ckpt_interval(p)
    res = None if residual is None else np.ascontiguousarray(residual, np.float64)
    if res is not None and res.shape != (p.nrec, p.nt):
        raise ValueError("residual must be [nrec][nt]")
    rc = lib().orc_gradient_ckpt(shot, C.byref(ctx.g), C.byref(ctx.m), C.byref(src), _d(sig), C.byref(rec),
                                 _d(ob), _d(res) if res is not None else None, _d(recs), C.byref(f), k,
                                 C.byref(J), *[_d(x) for x in g], _d(wf), _d(wa))
    if rc < 0:
        raise ValueError(f"orc_gradient_ckpt failed ({rc})")
    return J.value, tuple(g), recs[: p.nrec], wf, wa


def misfit(p, obs, shot=0, lam=None, mu=None, rho=None):
    """J = sum 0.5 dt (rec - obs)^2 over the receivers of `shot`, in FP64."""
    fw = forward(p, shot, False, lam, mu, rho)
    rows = shot_rows(p, shot)
    d = fw["rec"][rows] - np.asarray(obs, np.float64)[rows]
    return float(0.5 * p.dt * np.sum(d * d))


def exact_gradient(p, obs, shot=0, lam=None, mu=None, rho=None):
    """orc_exact_gradient: the discrete adjoint of the oracle's own time
    stepping.  Returns (J, grad_lam, grad_mu, grad_rho), gradients [nzt][nxt]
    with respect to the raw (unaveraged) models."""
    ctx = _Ctx(p, lam, mu, rho)
    lam = ctx.mat[0]
    mu = ctx.mat[1]
    rho = np.ascontiguousarray(p.rho if rho is None else rho, np.float64)
    src, keep1 = ctx.seis(p.src_x, p.src_z, p.src_comp, p.src_shot)
    rec, keep2 = ctx.seis(p.rec_x, p.rec_z, p.rec_comp, p.rec_shot)
    sig = np.ascontiguousarray(p.src_signal, np.float64) if p.nsrc else np.zeros((1, p.nt))
    ob = np.ascontiguousarray(obs, np.float64) if p.nrec else np.zeros((1, p.nt))
    g = [np.zeros((p.nzt, p.nxt)) for _ in range(3)]
    J = C.c_double()
    rc = lib().orc_exact_gradient(shot, C.byref(ctx.g), _d(lam), _d(mu), _d(rho), C.byref(src), _d(sig),
                                  C.byref(rec), _d(ob), C.byref(J), *[_d(x) for x in g])
    if rc != 0:
        raise ValueError(f"orc_exact_gradient failed ({rc})")
    return J.value, g[0], g[1], g[2]


def calc_opt_step(L2, sl):
    a = np.ascontiguousarray(L2[:3], np.float64)
    b = np.ascontiguousarray(sl[:3], np.float64)
    return lib().orc_calc_opt_step(_d(a), _d(b))


def lib_path() -> Path:
    return _build.ORACLE_SO
