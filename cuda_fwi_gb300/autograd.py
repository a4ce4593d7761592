"""torch.autograd wrapper: the L2 waveform misfit of a batch of shots as a
differentiable function of lam, mu, rho.

    J = FWIMisfit.apply(lam, mu, rho, engine, shots, obs, "exact")
    J.backward()   # lam.grad, mu.grad, rho.grad

``forward`` is the engine's forward entry point (``fwi_psv_forward``): it runs
the shots' forward sweep, records their seismograms and returns
J = sum over shots of sum 0.5 dt (syn - obs)^2 (the reference's
calculate_l2_adjoint_sources, CUDA_week2/fd_wave_model.cu:972-1002), keeping
what the backward needs (checkpoints or storage, the residual) on the device.
``backward`` is the engine's backward entry point (``fwi_psv_backward``): the
adjoint sweep and the gradient accumulation, summed over the shots and scaled
by the incoming gradient.  A forward whose result never reaches ``backward``
costs one forward sweep only.

The gradient mode is explicit:

* ``"exact"`` (default) -- the discrete adjoint of the FP32 time stepping:
  dJ/d(lam, mu, rho) of the very misfit ``forward`` returns, with respect to
  the raw models (the staggered averages are differentiated too);
* ``"reference"`` -- the reference's correlation formula
  (adjoint_kernel_PSV_GPU.cu:830-863).  It is what the reference's FWI loop
  uses, but it is not the derivative of J; choose it only to reproduce the
  reference.

Gradients are placed on the FWI window cells of the padded grid (zero
elsewhere).  Tensors are CPU float64 [nzt][nxt] (the reference's host layout).
Each forward must be followed by its backward before the engine runs another
forward (the engine keeps one forward's state).
"""
from __future__ import annotations

import numpy as np
import torch

MODES = ("exact", "reference")


def _to_grid(g, p):
    """[nfz][nfx] window gradient -> [nzt][nxt] grid (zeros outside the window)."""
    out = np.zeros((p.nzt, p.nxt))
    zs = np.arange(p.z1, p.z2, p.fwi_dz)
    xs = np.arange(p.x1, p.x2, p.fwi_dx)
    out[np.ix_(zs, xs)] = g[: len(zs), : len(xs)]
    return out


class FWIMisfit(torch.autograd.Function):
    @staticmethod
    def forward(ctx, lam, mu, rho, engine, shots, obs, mode="exact"):
        if mode not in MODES:
            raise ValueError(f"mode must be one of {MODES}, not {mode!r}")
        engine.set_gradient_mode(mode)
        engine.set_model_lmr(lam.detach().cpu().numpy(), mu.detach().cpu().numpy(),
                             rho.detach().cpu().numpy())
        _, mis = engine.forward(list(shots), obs, keep=True, want_rec=False)
        ctx.engine = engine
        return torch.tensor(float(np.sum(mis)), dtype=torch.float64)

    @staticmethod
    def backward(ctx, gout):
        eng = ctx.engine
        g = eng.backward(sum_shots=True)
        gl, gm, gr = (gout * torch.from_numpy(_to_grid(x, eng.p)) for x in g)
        return gl, gm, gr, None, None, None, None


def misfit(lam, mu, rho, engine, shots, obs, mode="exact"):
    return FWIMisfit.apply(lam, mu, rho, engine, shots, obs, mode)
