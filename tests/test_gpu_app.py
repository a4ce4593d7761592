"""The INI-driven host program on the GPU.

Forward modelling of tests/golden/ini/forward_small.ini: io/receiver/
rec_signal.csv and the last szz snapshot against the oracle run on the same
set-up (homogeneous medium with the reference's stiffer circle; CSV values
carry 6 significant digits).  Full waveform inversion from a CSV observed-data
file: two iterations, models written per iteration, the misfit decreasing; and
one iteration in the program's default order (the reference's: a gradient,
step search and update per shot, last-shot trial misfit) against
oracle/fwi_loop.py.
"""
import re
import subprocess
from dataclasses import replace
from pathlib import Path

import numpy as np
import pytest

from conftest import rel_l2
from cuda_fwi_gb300 import build as B
from cuda_fwi_gb300 import problem as P
from oracle import fwi_loop as FL
from oracle import oracle as O

pytestmark = pytest.mark.gpu
INI = Path(__file__).parent / "golden" / "ini"


def _problem(nt=200):
    p = P.Problem(nx=60, nz=50, nt=nt, dx=10.0, dz=10.0, dt=1e-3, fdorder=4, npml=8, fpml=12.0,
                  damp_v_pml=3000.0, name="ini").finalize()
    mu = 1732.0 ** 2 * 2000.0
    lam = 3000.0 ** 2 * 2000.0 - 2.0 * mu
    L = np.full((p.nzt, p.nxt), lam)
    zz, xx = np.mgrid[0:p.nzt, 0:p.nxt]
    L[(zz - p.nzt // 2) ** 2 + (xx - p.nxt // 2) ** 2 < p.nzt * p.nzt // 49] = 1.3 * lam
    p = p.with_model(L, np.full((p.nzt, p.nxt), mu), np.full((p.nzt, p.nxt), 2000.0))
    p.set_sources([20, 40], [5, 5], [0, 1], [15.0, 12.0])
    p.set_receivers([10, 25, 35, 50], [3, 3, 3, 3], [0, 0, 1, 1])
    return p


def _csv(path):
    rows = [[float(v) for v in line.split(",") if v.strip()] for line in Path(path).read_text().splitlines()]
    return np.array(rows)


def test_forward_outputs_match_oracle(tmp_path):
    r = subprocess.run([str(B.APP), str(INI / "forward_small.ini"), "--out", str(tmp_path)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr + r.stdout
    rec = _csv(tmp_path / "io/receiver/rec_signal.csv")
    p = _problem()
    want = np.zeros((p.nrec, p.nt))
    for s in (0, 1):
        rows = O.shot_rows(p, s)
        want[rows] = O.forward(p, s)["rec"][rows]
    assert rec.shape == want.shape
    assert rel_l2(rec, want) <= 1e-5
    snaps = sorted((tmp_path / "io/snap_data").glob("vz_snap*.csv"))
    assert [s.name for s in snaps] == [f"vz_snap{k}.csv" for k in range(4)]  # steps 0, 66, 132, 198
    q = replace(p, nt=199, src_signal=np.ascontiguousarray(p.src_signal[:, :199]))
    szz = O.forward(q, 1)["szz"]  # the last shot's field after step 198
    assert rel_l2(_csv(tmp_path / "io/snap_data/vz_snap3.csv"), szz) <= 1e-5


def test_fwi_mode_two_iterations(tmp_path):
    p = _problem(nt=160)
    obs = np.zeros((p.nrec, p.nt))
    for s in (0, 1):
        rows = O.shot_rows(p, s)
        obs[rows] = O.forward(p, s)["rec"][rows]
    obs_path = tmp_path / "obs.csv"
    obs_path.write_text("".join("".join(f"{v:.17g}, " for v in row) + "\n" for row in obs))
    ini = (INI / "forward_small.ini").read_text()
    ini = ini.replace("time = 0.2;", "nt = 160;").replace("full_waveform_inversion = 0;",
                      "full_waveform_inversion = 1;\nmax_iteration = 2;\nmax_error = 0.0;\n"
                      "fwi_order = summed;\ntrial_misfit = sum;\ncheckpoints = 8;")
    ini = ini.replace("[receiver]\n", f"[receiver]\nmeasurement_records = 1;\nsignal_file = {obs_path}\n")
    cfg = tmp_path / "fwi.ini"
    cfg.write_text(ini)
    r = subprocess.run([str(B.APP), str(cfg), "--out", str(tmp_path)], capture_output=True, text=True,
                       timeout=600)
    # two iterations without reaching max_error: the reference's "not converged" status
    assert r.returncode == 1, r.stderr + r.stdout
    l2 = [float(m) for m in re.findall(r"iteration \d+: L2 = ([0-9.eE+-]+)", r.stdout)]
    assert len(l2) == 2 and l2[1] < l2[0], r.stdout
    for it in (1, 2):
        for name in ("density", "lam", "mu"):
            m = _csv(tmp_path / f"io/density_snap/{name}_snap{it}.csv")
            assert m.shape == (p.nzt, p.nxt)
    lam2 = _csv(tmp_path / "io/density_snap/lam_snap2.csv")
    assert not np.allclose(lam2, lam2[0, 0])  # the homogeneous start was updated


def test_fwi_mode_default_order_matches_restatement(tmp_path):
    """No fwi_order / trial_misfit keys: fwi_run takes the reference's per-shot
    order with the last shot's trial misfit (fd_wave_model.cu:777-955,
    fwi_step_length_estimation.cu:136); one iteration over the two shots gives
    the restatement's misfits and step lengths and its model."""
    p = _problem(nt=160)
    obs = np.zeros((p.nrec, p.nt))
    for s in (0, 1):
        rows = O.shot_rows(p, s)
        obs[rows] = O.forward(p, s)["rec"][rows]
    # a homogeneous starting model (no circle): the program inverts for it
    mu = 1732.0 ** 2 * 2000.0
    start = p.with_model(np.full((p.nzt, p.nxt), 3000.0 ** 2 * 2000.0 - 2.0 * mu), np.full((p.nzt, p.nxt), mu),
                         np.full((p.nzt, p.nxt), 2000.0))
    # the program's default window: [ppad, nxt) x [ppad, nzt) (INI defaults moved onto the padded grid)
    start = replace(start, x1=start.ppad, z1=start.ppad)
    rows = O.shot_rows(p, 1)  # the last shot's data halfway to the start's: the search accepts steps
    obs[rows] = 0.5 * (obs[rows] + O.forward(start, 1)["rec"][rows])
    obs_path = tmp_path / "obs.csv"
    obs_path.write_text("".join("".join(f"{v:.17g}, " for v in row) + "\n" for row in obs))
    ini = (INI / "forward_small.ini").read_text()
    ini = ini.replace("time = 0.2;", "nt = 160;").replace(
        "full_waveform_inversion = 0;", "full_waveform_inversion = 1;\nmax_iteration = 1;\nmax_error = 0.0;\n"
        "checkpoints = 8;")
    ini = ini.replace("[receiver]\n", f"[receiver]\nmeasurement_records = 1;\nsignal_file = {obs_path}\n")
    cfg = tmp_path / "fwi.ini"
    cfg.write_text(ini)
    r = subprocess.run([str(B.APP), str(cfg), "--out", str(tmp_path)], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode in (0, 1), r.stderr + r.stdout
    got = [(float(a), float(b), int(c)) for a, b, c in
           re.findall(r"iteration 1: L2 = ([0-9.eE+-]+), step length = ([0-9.eE+-]+), trials = (\d+)", r.stdout)]
    lam_r, mu_r, rho_r, log_r = FL.fwi_loop(start, obs, [0, 1], iters=1, step0=0.01, order="per_shot",
                                            trial="last")
    assert len(got) == len(log_r) == 2, r.stdout
    for (mis, step, trials), want in zip(got, log_r):
        assert trials == want["trials"]
        assert mis == pytest.approx(want["misfit"], rel=1e-4)
        assert step == pytest.approx(want["step_length"], rel=1e-3)
    lam1 = _csv(tmp_path / "io/density_snap/lam_snap1.csv")
    assert rel_l2(lam1 - start.lam, lam_r - start.lam) <= 1e-3  # CSV values carry 6 significant digits
