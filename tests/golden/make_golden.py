"""Generate the golden fixtures in this directory from the reference itself.

Runs the reference's own CPU functions (compiled from its sources by
oracle/build.py into oracle/_ref/libfwi_ref.so) on small seeded problems and
stores inputs and outputs together, so the fixtures are self-contained:

  ref_o2.npz        fdorder 2, CPML on all sides, 1 shot, FWI storage with
                    sub-sampling (t 2, x 2, z 3): forward seismograms, final
                    wavefield, We, storage; adjoint gradients and We.
  ref_o2_fsurf.npz  same with a free surface (override + mirroring).
  ref_o2_multi.npz  3 shots sharing the acquisition arrays, shot 1 run.
  ricker_kat.npz    the Ricker wavelet known-answer vector shipped by the
                    reference (CUDA_week2/io/receiver/src_signal_1_1.csv, first
                    source: amplitude 1000, f0 15 Hz, dt 0.2 ms, 6 significant
                    digits), read as text.

Usage: python tests/golden/make_golden.py   (needs the reference sources)
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from cuda_fwi_gb300 import problem as P  # noqa: E402
from oracle import build as B  # noqa: E402
from oracle import reference as R  # noqa: E402

SCALARS = ("nx", "nz", "nt", "dx", "dz", "dt", "fdorder", "npml", "fsurf", "fpad", "ppad", "nxt",
           "nzt", "fwi_dt", "fwi_dx", "fwi_dz", "x1", "x2", "z1", "z2")
ARRAYS = ("hc", "lam", "mu", "rho", "src_x", "src_z", "src_comp", "src_shot", "src_signal", "rec_x",
          "rec_z", "rec_comp", "rec_shot")


def pack(p, shot, obs_scale, **extra):
    fw = R.forward(p, shot, True)
    rows = np.nonzero((p.rec_shot == shot) & (p.rec_comp == 2))[0]
    obs = fw["rec"] * obs_scale
    res = np.zeros_like(fw["rec"])
    res[rows] = fw["rec"][rows] - obs[rows]
    misfit = float(np.sum(0.5 * p.dt * res[rows] ** 2))
    ad = R.adjoint(p, shot, res, fw["store"])
    d = {k: np.asarray(getattr(p, k)) for k in SCALARS + ARRAYS}
    for k, v in p.cpml.items():
        d["cpml_" + k] = v
    d["shot"] = np.int32(shot)
    d["obs"] = obs
    d["out_rec"] = fw["rec"]
    d["out_misfit"] = np.float64(misfit)
    for k in ("vx", "vz", "sxx", "szx", "szz", "We"):
        d["out_fwd_" + k] = fw[k]
    for k, v in fw["store"].items():
        d["out_store_" + k] = v
    for k in ("grad_lam", "grad_mu", "grad_rho", "We", "vz"):
        d["out_adj_" + k] = ad[k]
    d.update(extra)
    return d


def main():
    if B.build_ref() is None:
        sys.exit("reference sources not found (set FWI_REFERENCE_DIR)")
    p = P.small(fdorder=2, nx=40, nz=32, nt=160, npml=6, nrec=5, perturb=0.05, fwi=(2, 2, 3))
    np.savez_compressed(HERE / "ref_o2.npz", **pack(p, 0, 0.6))
    p = P.small(fdorder=2, nx=40, nz=30, nt=160, npml=6, fsurf=1, nrec=5, perturb=0.05, fwi=(3, 2, 2))
    np.savez_compressed(HERE / "ref_o2_fsurf.npz", **pack(p, 0, 0.5))
    p = P.small(fdorder=2, nx=44, nz=30, nt=140, npml=6, nshots=3, nrec=4, perturb=0.03, fwi=(4, 2, 2))
    np.savez_compressed(HERE / "ref_o2_multi.npz", **pack(p, 1, 0.8))
    csv = B.reference_root() / "CUDA_week2/io/receiver/src_signal_1_1.csv"
    first = csv.read_text().splitlines()[0]
    vals = np.array([float(v) for v in first.split(",") if v.strip()])
    np.savez_compressed(HERE / "ricker_kat.npz", signal=vals, amp=1000.0, fc=15.0, dt=0.2e-3, ts=0.0)
    print("wrote", sorted(x.name for x in HERE.glob("*.npz")))


if __name__ == "__main__":
    main()
