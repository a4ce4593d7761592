"""bench.py on the host: the reference arm's JSON line and the roofline arithmetic.

The reference arm times the CPU path (the FP64 restatement of the reference's
CPU propagators) on the host cores; here it runs a 4-step sample so the test
takes seconds.  The algorithmic-byte model is checked against the per-cell
figures of the kernels (stress 32 B per shot + 12 B per launch, velocity 28 + 8,
adjoint stress 92 + 12, adjoint velocity 36 + 8, 16 B per CPML strip cell) and
the bound it puts on any batched path of the benchmark workload.
"""
import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402
from cuda_fwi_gb300 import problem as P  # noqa: E402


def test_reference_arm_prints_one_json_line():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--cpu-nt-sample", "4"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "shot-gradients/s" and d["unit"] == "shot-gradients/s"
    assert d["higher_is_better"] is True and d["value"] > 0
    assert d["steps"] == 1 and d["warmup"] == 0
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert "4 of 3000 time steps" in cb["sample"]
    assert "1000x500" in d["config"]["workload"]
    # the same workload description as the engine's arm
    assert d["config"] == bench.bench_config(bench.parse_args([]), P.config3(False, nshots=64), 1)
    # the arm's process never loaded the engine library (its problem set-up is the oracle's)
    assert d["product_library_mapped"] is False


def test_algorithmic_bytes_per_cell():
    p = P.small(fdorder=8, nx=300, nz=100, nt=10, npml=8, nshots=1, nrec=3)
    fp = p.fpad
    cells = (p.nxt - 2 * fp) * (p.nzt - 2 * fp)
    strip = 2 * p.npml * (p.nzt - 2 * fp) + 2 * p.npml * (p.nxt - 2 * fp)
    for B in (1, 7, 32):
        s, v, a, va = bench.algorithmic_bytes(p, B)
        assert s == B * (32 * cells + 16 * strip) + 12 * cells
        assert v == B * (28 * cells + 16 * strip) + 8 * cells
        assert a == B * (92 * cells + 16 * strip) + 12 * cells
        assert va == B * (36 * cells + 16 * strip) + 8 * cells


def test_roofline_bound_of_the_benchmark_workload():
    """580 GB of algorithmic traffic per shot-gradient at 32 shots per launch:
    at 6,787.6 GB/s no batched path exceeds ~11.7 shot-gradients/s."""
    syn = P.config3(False, nshots=64)
    sub, recompute = 32, 5374
    fb = [x / sub for x in bench.algorithmic_bytes(syn, sub)]
    per_grad = (syn.nt + recompute) * (fb[0] + fb[1]) + syn.nt * (fb[2] + fb[3]) + \
        syn.nt * (syn.nxt - 2 * syn.fpad) * (syn.nzt - 2 * syn.fpad) * 8
    assert per_grad / 1e9 == pytest.approx(580.0, rel=0.01)
    assert 6787.6e9 / per_grad == pytest.approx(11.70, rel=0.01)
