"""torch.autograd wrapper: the L2 waveform misfit of a batch of shots as a
differentiable function of lam, mu, rho.

    J = FWIMisfit.apply(lam, mu, rho, engine, shots, obs)
    J.backward()   # lam.grad, mu.grad, rho.grad

forward returns sum over shots of J_s = sum 0.5 dt (syn - obs)^2 (the
reference's calculate_l2_adjoint_sources, CUDA_week2/fd_wave_model.cu:972-1002);
backward returns the gradient the engine computes -- the reference's
correlation formula (adjoint_kernel_PSV_GPU.cu:830-863) by default, or the
exact discrete adjoint after engine.set_gradient_mode("exact") -- placed on
the FWI window cells of the padded grid (zero elsewhere).  The forward and the
adjoint run together on the GPU in one fwi_psv_gradient call; backward only
scales the stored gradient.

Tensors are CPU float64 [nzt][nxt] (the reference's host layout).
"""
from __future__ import annotations

import numpy as np
import torch


def _to_grid(g, p):
    """[nfz][nfx] window gradient -> [nzt][nxt] grid (zeros outside the window)."""
    out = np.zeros((p.nzt, p.nxt))
    zs = np.arange(p.z1, p.z2, p.fwi_dz)
    xs = np.arange(p.x1, p.x2, p.fwi_dx)
    out[np.ix_(zs, xs)] = g[: len(zs), : len(xs)]
    return out


class FWIMisfit(torch.autograd.Function):
    @staticmethod
    def forward(ctx, lam, mu, rho, engine, shots, obs):
        engine.set_model_lmr(lam.detach().cpu().numpy(), mu.detach().cpu().numpy(),
                             rho.detach().cpu().numpy())
        g, mis = engine.gradient(list(shots), obs)
        p = engine.p
        ctx.grads = [torch.from_numpy(_to_grid(x, p)) for x in g]
        return torch.tensor(float(np.sum(mis)), dtype=torch.float64)

    @staticmethod
    def backward(ctx, gout):
        gl, gm, gr = (gout * x for x in ctx.grads)
        return gl, gm, gr, None, None, None


def misfit(lam, mu, rho, engine, shots, obs):
    return FWIMisfit.apply(lam, mu, rho, engine, shots, obs)
