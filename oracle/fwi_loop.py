"""FP64 restatement of the reference's FWI optimiser loop (checker only).

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of the engine's
fwi_psv_fwi_run / fwi_psv_step_search; the product never imports it.

Restates (Mohammad-debug/CUDA_FWI, CUDA_week2/):
  step_search        fwi_step_length_estimation.cu:16-223 (conditions 1.1, 1.2,
                     2.1, 2.2; est_scale_factor 2, stepmax 6; the process exit of
                     a failed search becomes status 1)
  scale_gradients    fd_wave_model.cu:1004-1052 (energy weights, eps 0.005)
  grad_update        fd_medium.cu:161-240 (max normalisation with the signed
                     grad_max its loop leaves, clamps, negative -> old value)
  fwi_loop           fd_wave_model.cu:736-955 (medium averages, gradients,
                     preconditioning, step search, update)
The window indexing is the natural one: gradient sample (zf, xf) belongs to
cell (z1 + zf*fwi_dz, x1 + xf*fwi_dx); the reference's loops index the
[nfz][nfx] arrays with padded-grid indices, which coincide for the default
window (z1 = x1 = 0, unit intervals).
"""
from __future__ import annotations

from dataclasses import replace

import numpy as np

from . import oracle as O

LIMITS = {"lam": (0.0, 48.0e9), "mu": (0.0, 27.0e9), "rho": (1.5, 3000.0)}  # fd_medium.cu:172-183


def calc_opt_step(L2, sl):
    return O.calc_opt_step(np.asarray(L2[:3], np.float64), np.asarray(sl[:3], np.float64))


def step_search(est, L2_0, trial):
    """Returns (opt, trials, status, steps_tried)."""
    scale, stepmax = 2.0, 6
    L2 = [L2_0, 0.0, 0.0, L2_0]
    sl = [0.0, 0.0, 0.0, 0.0]
    step1 = step2 = 0
    itest, count, calls, status = 1, 0, 0, 0
    tried = []
    while step2 != 1 or step1 != 1:
        L2[itest] = trial(est)
        tried.append(est)
        calls += 1
        sl[itest] = est
        sl[0] = 0.0
        if step1 == 1 and L2[1] < L2[2]:
            sl[2] = est
            step2 = 1
        elif step1 == 1 and L2[1] >= L2[2]:
            sl[2] = est
            est = est + est / scale
            count += 1
        elif step1 == 0 and L2[0] > L2[1]:
            sl[1] = est
            step1 = 1
            itest = 2
            count = 0
            est = est + est / scale
        else:
            est = est / scale
            count += 1
        if step1 == 0 and count > stepmax:
            status = 1
            break
        if step1 == 1 and count > stepmax:
            status = 2
            step1 = step2 = 1
    opt = 0.0 if status == 1 else calc_opt_step(L2, sl)
    return opt, calls, status, tried


def window_cells(p):
    zs = np.arange(p.z1, p.z2, p.fwi_dz)
    xs = np.arange(p.x1, p.x2, p.fwi_dx)
    return zs, xs


def scale_gradients(p, g, ws, wr, c):
    """Energy-weight preconditioning of one shot's [nfz][nfx] gradients."""
    zs, xs = window_cells(p)
    we = np.sqrt(ws[np.ix_(zs, xs)] * wr[np.ix_(zs, xs)])
    we = we + 0.005 * we.max()
    out = []
    for gi, ci in zip(g, c):
        h = np.zeros_like(gi)
        h[: len(zs), : len(xs)] = gi[: len(zs), : len(xs)] / (we * ci * ci)
        out.append(h)
    return out


def grad_norm(p, mat_old, grad):
    """step -> normalised step factor mat_max / grad_max (signed grad_max)."""
    zs, xs = window_cells(p)
    mat_max = max(0.0, float(mat_old[np.ix_(zs, xs)].max()))
    gmax = 0.0
    for v in grad[: len(zs), : len(xs)].ravel():  # row-major, as the reference's loop
        if abs(v) > gmax:
            gmax = float(v)
    return mat_max / gmax if gmax != 0.0 else 0.0


def grad_update(p, mat_old, grad, sn, name):
    lo, hi = LIMITS[name]
    zs, xs = window_cells(p)
    new = mat_old.copy()
    sub = mat_old[np.ix_(zs, xs)] + sn * grad[: len(zs), : len(xs)]
    sub = np.clip(sub, lo, hi)
    sub = np.where(sub < 0.0, mat_old[np.ix_(zs, xs)], sub)
    new[np.ix_(zs, xs)] = sub
    return new


def misfits(p, obs, shots, lam, mu, rho):
    return [O.misfit(p, obs, s, lam, mu, rho) for s in shots]


def fwi_loop(p, obs, shots, iters, step0=0.01, precondition=True, trial="sum", order="summed", restart_step=0.0):
    """The inversion loop.  order "summed": one update per iteration from the
    shot-summed gradient; "per_shot": the reference's order
    (fd_wave_model.cu:777-955), one gradient, step search and update per shot
    inside each iteration.  trial "sum": the search compares misfits summed over
    all shots (with per-shot order its step-0 value is the all-shot sum at the
    current model too); "last": the reference's search, which keeps the last
    shot's trial misfit (fwi_step_length_estimation.cu:136) against the
    gradient's own misfit.  The material constants C (medium_average) are taken
    once per iteration; the staggered averages that each gradient and trial
    forward use come from the model it runs on.  A failed search (status 1)
    stops the loop with the model unchanged, unless restart_step > 0: then the
    search is run once more on the same gradient from restart_step (the
    engine's opt-in continuation; trials add up).  Returns (lam, mu, rho, log) with
    one entry dict(misfit, step_length, trials, status) per update."""
    lam, mu, rho = p.lam.copy(), p.mu.copy(), p.rho.copy()
    step = step0
    log = []
    groups = [list(shots)] if order == "summed" else [[s] for s in shots]
    for _ in range(iters):
        c = [float(np.mean(x)) for x in (lam, mu, rho)]
        for grp in groups:
            g = [np.zeros((p.nfz, p.nfx)) for _ in range(3)]
            L0 = 0.0
            for s in grp:
                J, gs, fw, ad = O.gradient(p, obs, s, lam, mu, rho)
                L0 += J
                if precondition:
                    gs = scale_gradients(p, list(gs), fw["We"], ad["We"], c)
                for i in range(3):
                    g[i] += gs[i]
            if order == "per_shot" and trial == "sum":
                L0 = sum(misfits(p, obs, shots, lam, mu, rho))
            norms = [grad_norm(p, m, gi) for m, gi in zip((lam, mu, rho), g)]

            def model(est, g=g, norms=norms, cur=(lam, mu, rho)):
                f = (est, est, 0.5 * est)
                return [grad_update(p, m, gi, fi * ni, name)
                        for m, gi, fi, ni, name in zip(cur, g, f, norms, ("lam", "mu", "rho"))]

            def trial_fn(est, model=model):
                mis = misfits(p, obs, shots, *model(est))
                return mis[-1] if trial == "last" else sum(mis)

            opt, calls, status, _ = step_search(step, L0, trial_fn)
            if status == 1 and restart_step > 0:
                opt, more, status, _ = step_search(restart_step, L0, trial_fn)
                calls += more
            log.append(dict(misfit=L0, step_length=opt if status != 1 else 0.0, trials=calls, status=status))
            if status == 1:
                return lam, mu, rho, log
            lam, mu, rho = model(opt)
            step = opt
    return lam, mu, rho, log


def with_model(p, lam, mu, rho):
    return replace(p, lam=np.ascontiguousarray(lam), mu=np.ascontiguousarray(mu), rho=np.ascontiguousarray(rho))
