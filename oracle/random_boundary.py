"""Random-boundary gradient of the FP64 oracle (checker only).

TEST INFRASTRUCTURE ONLY: the checker of the engine's FWI_STORE_RANDOM.

The engine's random-boundary strategy records seismograms, misfit and
residual with the absorbing (CPML) forward, runs a second forward without
CPML in a seeded random-velocity frame (Clapp, "Reverse time migration with
random boundaries", SEG 2009; Shen & Clapp, Geophysics 2015) and rebuilds
that second wavefield backwards in time for the gradient.  In exact
arithmetic this is the reference's gradient computed from the residual of
the CPML forward and the stored wavefield of the frame forward, which the
oracle gives directly: orc_forward with an identity CPML (a = b = 0, K = 1)
on the frame materials for the storage, then orc_adjoint with the real CPML
and medium.

The frame: in the padding, velocities are scaled by f = 1 - alpha (d / ppad) u
with d the depth into the padding and u = (hash(block) >> 8) / 2^24 per block
of GRAIN x GRAIN cells, the same hash the engine uses; lam, mu and mu_zx are
scaled by f^2, densities kept.
"""
from __future__ import annotations

from dataclasses import replace

import numpy as np

from . import oracle as O

SEED = 20090625
ALPHA = np.float32(0.5)
GRAIN = 16
M32 = 0xFFFFFFFF


def _hash_u32(x):
    x = x & M32
    x ^= x >> 16
    x = (x * 0x7FEB352D) & M32
    x ^= x >> 15
    x = (x * 0x846CA68B) & M32
    x ^= x >> 16
    return x


def frame_factor2(p):
    """f^2 per padded cell [nzt][nxt] (float32 arithmetic, as the engine)."""
    iz, ix = np.mgrid[0:p.nzt, 0:p.nxt].astype(np.int64)
    d = np.zeros_like(iz)
    d = np.maximum(d, p.ppad - ix)
    d = np.maximum(d, ix - (p.nxt - 1 - p.ppad))
    if not p.fsurf:
        d = np.maximum(d, p.ppad - iz)
    d = np.maximum(d, iz - (p.nzt - 1 - p.ppad))
    key = ((iz // GRAIN) * 65599 + (ix // GRAIN)).astype(np.uint64) & np.uint64(M32)
    h = _hash_u32((key * np.uint64(2654435761) + np.uint64(SEED)) & np.uint64(M32))
    u = (h >> np.uint64(8)).astype(np.float32) * np.float32(1.0 / 16777216.0)
    q = d.astype(np.float32) / np.float32(max(p.ppad, 1))
    f = np.float32(1.0) - ALPHA * q * u
    f2 = np.where(d > 0, f * f, np.float32(1.0))
    return f2.astype(np.float64)


def gradient(p, obs, shot=0, residual=None):
    """(J, (grad_lam, grad_mu, grad_rho)) of the random-boundary strategy.
    `residual` ([nrec][nt]) replaces the adjoint source syn - obs (J still
    comes from obs)."""
    f2 = frame_factor2(p)
    mzx, rzp, rxp = O.average(p.lam, p.mu, p.rho)
    ident = {k: (np.ones_like(v) if k in ("K", "K_half") else np.zeros_like(v)) for k, v in p.cpml.items()}
    q = replace(p, cpml=ident)
    fw = O.forward(q, shot, True, p.lam * f2, p.mu * f2, p.rho,
                   averaged=(mzx * f2[:-1, :-1], rzp, rxp))
    rows = O.shot_rows(p, shot)
    J, res, _ = O.residual(O.forward(p, shot)["rec"], obs, p.dt, rows)
    if residual is not None:
        res = np.ascontiguousarray(residual, np.float64)
    ad = O.adjoint(p, shot, res, fw["store"])
    return J, (ad["grad_lam"], ad["grad_mu"], ad["grad_rho"])
