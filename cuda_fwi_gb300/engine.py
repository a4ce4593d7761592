"""Pythonic wrapper of the engine C ABI (``include/fwi_psv.h``).

Mirrors the reference's per-shot propagator pair (Mohammad-debug/CUDA_FWI,
CUDA_week2/fd_kernel.cuh:75-173) as a batched forward/backward pair:

    eng = Engine(problem)                 # grid, scheme, CPML, materials, acquisition
    rec, misfit = eng.forward(shots, obs, keep=True)
    g_lam, g_mu, g_rho = eng.backward(sum_shots=True)

All work runs on the GPU; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi
from ._capi import check, pd, pi
from .problem import Problem

STRATEGIES = {"full": _capi.FWI_STORE_FULL, "binomial": _capi.FWI_STORE_BINOMIAL,
              "random": _capi.FWI_STORE_RANDOM}


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class Engine:
    def __init__(self, problem: Problem, device: int = 0, set_model: bool = True):
        self.p = problem
        L = _capi.lib()
        self._cp = {k: _f64(v) for k, v in problem.cpml.items()}
        d = _capi.Desc()
        for k in ("nt", "nzt", "nxt", "fpad", "ppad", "npml", "fsurf", "fdorder"):
            setattr(d, k, int(getattr(problem, k)))
        d.dt, d.dx, d.dz = problem.dt, problem.dx, problem.dz
        for i in range(7):
            d.hc[i] = float(problem.hc[i])
        for k in ("a", "b", "K", "a_half", "b_half", "K_half"):
            setattr(d, k, pd(self._cp[k]))
        h = C.c_void_p()
        check(L.fwi_psv_create(C.byref(d), device, C.byref(h)), "fwi_psv_create")
        self.h = h
        self._last_nshots = 0
        if set_model and problem.lam is not None:
            self.set_model_lmr(problem.lam, problem.mu, problem.rho)
        self.set_sources(problem.src_x, problem.src_z, problem.src_comp, problem.src_shot,
                         problem.src_signal)
        self.set_receivers(problem.rec_x, problem.rec_z, problem.rec_comp, problem.rec_shot)
        self.set_fwi(problem.fwi_dt, problem.fwi_dx, problem.fwi_dz, problem.x1, problem.x2,
                     problem.z1, problem.z2)

    # ---- configuration ---------------------------------------------------------
    def set_model(self, lam, mu, mu_zx, rho_zp, rho_xp):
        a = [_f64(x) for x in (lam, mu, mu_zx, rho_zp, rho_xp)]
        check(_capi.lib().fwi_psv_set_model(self.h, *[pd(x) for x in a]), "set_model")

    def set_model_lmr(self, lam, mu, rho):
        a = [_f64(x) for x in (lam, mu, rho)]
        check(_capi.lib().fwi_psv_set_model_lmr(self.h, *[pd(x) for x in a]), "set_model_lmr")

    def set_sources(self, x, z, comp, shot, signal):
        x, z, comp, shot = map(_i32, (x, z, comp, shot))
        sig = _f64(signal) if len(x) else np.zeros((1, self.p.nt))
        check(_capi.lib().fwi_psv_set_sources(self.h, len(x), pi(x), pi(z), pi(comp), pi(shot),
                                              pd(sig)), "set_sources")

    def set_receivers(self, x, z, comp, shot):
        x, z, comp, shot = map(_i32, (x, z, comp, shot))
        self.nrec = len(x)
        check(_capi.lib().fwi_psv_set_receivers(self.h, len(x), pi(x), pi(z), pi(comp), pi(shot)),
              "set_receivers")

    def set_fwi(self, fwi_dt=1, fwi_dx=1, fwi_dz=1, x1=0, x2=None, z1=0, z2=None):
        x2 = self.p.nxt if x2 is None else x2
        z2 = self.p.nzt if z2 is None else z2
        check(_capi.lib().fwi_psv_set_fwi(self.h, fwi_dt, fwi_dx, fwi_dz, x1, x2, z1, z2), "set_fwi")
        self.nfz = 1 + (z2 - z1) // fwi_dz
        self.nfx = 1 + (x2 - x1) // fwi_dx

    def set_strategy(self, strategy="full", snapshots=0, budget_bytes=0):
        s = STRATEGIES[strategy] if isinstance(strategy, str) else int(strategy)
        check(_capi.lib().fwi_psv_set_strategy(self.h, s, snapshots, budget_bytes), "set_strategy")

    def set_gradient_mode(self, mode="reference"):
        """'reference': the reference's correlation gradient; 'exact': the
        discrete adjoint of the FP32 time stepping (gradient of the misfit the
        forward returns, with respect to the raw lam, mu, rho)."""
        m = {"reference": 0, "exact": 1}[mode] if isinstance(mode, str) else int(mode)
        check(_capi.lib().fwi_psv_set_gradient_mode(self.h, m), "set_gradient_mode")

    def set_exec(self, use_graphs=True, block_x=0, tile_z=0, batch=0):
        check(_capi.lib().fwi_psv_set_exec(self.h, int(use_graphs), block_x, tile_z, batch), "set_exec")

    def set_snapshots(self, interval: int, which: int = 4):
        """Keep field `which` (0 vx .. 4 szz) of every batch slot every `interval` steps
        of the recording sweep (the reference's vz_snap files hold szz: which = 4)."""
        check(_capi.lib().fwi_psv_set_snapshots(self.h, int(interval), int(which)), "set_snapshots")

    def snapshot(self, slot: int, k: int):
        """Snapshot k (step k * interval) of batch slot `slot` of the last forward, [nzt][nxt]."""
        out = np.zeros((self.p.nzt, self.p.nxt))
        check(_capi.lib().fwi_psv_snapshot(self.h, int(slot), int(k), pd(out)), "snapshot")
        return out

    def set_wait_limit(self, seconds: float):
        """Bound of every wait of the kernels on their own copies (default 2 s)."""
        check(_capi.lib().fwi_psv_set_wait_limit(self.h, float(seconds)), "set_wait_limit")

    def debug_stall_next(self):
        """Test hook: the next forward's first TMA-staged step waits for bytes that never arrive."""
        check(_capi.lib().fwi_psv_debug_stall_next(self.h), "debug_stall_next")

    def set_stream(self, stream_handle: int | None):
        check(_capi.lib().fwi_psv_set_stream(self.h, C.c_void_p(stream_handle or 0)), "set_stream")

    # ---- forward / backward -------------------------------------------------
    def forward(self, shots, obs=None, keep=False, want_rec=True, resident=False):
        """Run the shots together.  obs [nrec][nt] (host, FP64) or, with
        resident=True, the observed data left on the device by the previous
        forward of the same batch.  Returns (rec [nrec][nt] or None, misfit [nshots])."""
        shots = _i32(np.atleast_1d(shots))
        rec = np.zeros((max(self.nrec, 1), self.p.nt)) if want_rec else None
        mis = np.zeros(len(shots))
        o = _f64(obs) if (obs is not None and not resident) else None
        flags = (_capi.FWI_FWD_KEEP if keep else 0) | (_capi.FWI_FWD_RESIDENT_OBS if resident else 0)
        check(_capi.lib().fwi_psv_forward(self.h, len(shots), pi(shots), pd(o), pd(rec), pd(mis),
                                          flags), "forward")
        self._last_nshots = len(shots)
        return rec, mis

    def backward(self, sum_shots=False, want=True):
        """Gradients (lam, mu, rho) [nshots][nfz][nfx], or summed over the
        batch; want=False leaves them on the device (returns None)."""
        if not want:
            check(_capi.lib().fwi_psv_backward(self.h, None, None, None, int(sum_shots)), "backward")
            return None
        n = 1 if sum_shots else self._last_nshots
        g = [np.zeros((n, self.nfz, self.nfx)) for _ in range(3)]
        check(_capi.lib().fwi_psv_backward(self.h, *[pd(x) for x in g], int(sum_shots)), "backward")
        if sum_shots:
            g = [x[0] for x in g]
        return tuple(g)

    def gradient(self, shots, obs=None, resident=False, want=True):
        """Summed shot gradients (lam, mu, rho) [nfz][nfx] and per-shot misfits,
        computed in sub-batches on the device (fwi_psv_gradient)."""
        shots = _i32(np.atleast_1d(shots))
        mis = np.zeros(len(shots))
        g = [np.zeros((self.nfz, self.nfx)) for _ in range(3)] if want else [None] * 3
        o = _f64(obs) if (obs is not None and not resident) else None
        flags = _capi.FWI_FWD_RESIDENT_OBS if resident else 0
        check(_capi.lib().fwi_psv_gradient(self.h, len(shots), pi(shots), pd(o), pd(mis),
                                           *[pd(x) for x in g], flags), "gradient")
        return (tuple(g) if want else None), mis

    def misfit(self, shots, obs=None, resident=False):
        """Per-shot misfits from forward-only runs (the step-length trials)."""
        ids = _i32(shots)
        mis = np.zeros(len(ids))
        o = None if resident else _f64(obs)
        check(_capi.lib().fwi_psv_misfit(self.h, len(ids), pi(ids), pd(o), pd(mis),
                                         _capi.FWI_FWD_RESIDENT_OBS if resident else 0), "misfit")
        return mis

    def set_precondition(self, on=True, c=(1.0, 1.0, 1.0)):
        """Energy-weight preconditioning of each shot's gradient with medium
        averages c = (C_lam, C_mu, C_rho)."""
        check(_capi.lib().fwi_psv_set_precondition(self.h, int(on), *[float(x) for x in c]), "set_precondition")

    def set_model_device(self, lam, mu, rho):
        """lam, mu, rho: CUDA float64 tensors [nzt][nxt] on the engine's device."""
        for t in (lam, mu, rho):
            assert t.is_cuda and t.dtype == __import__("torch").float64 and t.is_contiguous()
        check(_capi.lib().fwi_psv_set_model_device(self.h, C.c_void_p(lam.data_ptr()), C.c_void_p(mu.data_ptr()),
                                                   C.c_void_p(rho.data_ptr())), "set_model_device")

    def fwi_run(self, shots, obs, max_iter, step_length=0.01, max_error=0.0, order="summed", trial="sum",
                precondition=True, model=None, true_model=None, restart_step=0.0, resume_file=None):
        """The inversion loop on the device.  model = (lam, mu, rho) start
        (default: the problem's); returns ((lam, mu, rho), log) with one dict
        per update (misfit, step_length, trials, status, model_error, seconds).
        restart_step > 0 retries a failed step search once from that step.
        resume_file: the loop state is saved there after each iteration, and a
        run that finds it continues from it (to max_iter iterations in all)."""
        ids = _i32(shots)
        lam, mu, rho = [np.array(x, np.float64, order="C") for x in (model or (self.p.lam, self.p.mu, self.p.rho))]
        tm = [_f64(x) for x in true_model] if true_model is not None else [None] * 3
        o = _capi.FwiOpts(max_iter, max_error, step_length, {"summed": 0, "per_shot": 1}[order],
                          {"sum": 0, "last": 1}[trial], int(precondition), pd(tm[0]), pd(tm[1]), pd(tm[2]),
                          float(restart_step), None if resume_file is None else str(resume_file).encode())
        n = max_iter * (len(ids) if order == "per_shot" else 1)
        log = (_capi.FwiIter * max(n, 1))()
        done = C.c_int()
        check(_capi.lib().fwi_psv_fwi_run(self.h, C.byref(o), len(ids), pi(ids), pd(_f64(obs)), pd(lam), pd(mu),
                                          pd(rho), log, C.byref(done)), "fwi_run")
        out = [{k: getattr(log[i], k) for k, _ in _capi.FwiIter._fields_} for i in range(done.value)]
        return (lam, mu, rho), out

    def time_kernels(self, reps=20):
        """Average device ms of one launch of: forward stress, forward velocity,
        adjoint stress, adjoint velocity (drops the retained forward)."""
        ms = np.zeros(4)
        check(_capi.lib().fwi_psv_time_kernels(self.h, reps, pd(ms)), "time_kernels")
        return [float(x) for x in ms]

    def energy(self, slot=0):
        ws = np.zeros((self.p.nzt, self.p.nxt))
        wr = np.zeros((self.p.nzt, self.p.nxt))
        check(_capi.lib().fwi_psv_energy(self.h, slot, pd(ws), pd(wr)), "energy")
        return ws, wr

    def wavefield(self, which=0, slot=0):
        f = [np.zeros((self.p.nzt, self.p.nxt)) for _ in range(5)]
        check(_capi.lib().fwi_psv_wavefield(self.h, which, slot, *[pd(x) for x in f]), "wavefield")
        return dict(zip(("vx", "vz", "sxx", "szx", "szz"), f))

    def stats(self) -> dict:
        s = _capi.Stats()
        check(_capi.lib().fwi_psv_get_stats(self.h, C.byref(s)), "get_stats")
        return {k: getattr(s, k) for k, _ in _capi.Stats._fields_}

    def close(self):
        if getattr(self, "h", None):
            _capi.lib().fwi_psv_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
