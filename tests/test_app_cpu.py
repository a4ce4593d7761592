"""The INI-driven host program (cuda_fwi_gb300/_lib/fwi_run) without a GPU:
its configuration reading and grid set-up (--dry-run) against the reference's
rules restated here (fd_grid.cu:52-71 padding, fd_seismogram.cu:153-163
positions, fd_fwi.cu:26-51 window, holbergcoeff, cpml_pro)."""
import json
import subprocess
from pathlib import Path

import numpy as np
import pytest

from cuda_fwi_gb300 import build as B
from oracle import oracle as O

INI = Path(__file__).parent / "golden" / "ini"


def _dry(path, tmp_path=None):
    r = subprocess.run([str(B.APP), str(path), "--dry-run"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout)


def test_dry_run_matches_reference_rules():
    c = _dry(INI / "forward_small.ini")
    fpad, ppad, nxt, nzt = O.total_grid(60, 50, 4, 8, 0)
    assert (c["fpad"], c["ppad"], c["nxt"], c["nzt"]) == (fpad, ppad, nxt, nzt)
    assert c["nt"] == 200 and c["nshots"] == 2 and c["snap_interval"] == 66 and c["fwinv"] == 0
    assert c["src"] == [[20 + ppad, 5 + ppad, 2, 0], [40 + ppad, 5 + ppad, 2, 1]]
    assert c["rec"] == [[x + ppad, 3 + ppad, 2, s] for x, s in zip((10, 25, 35, 50), (0, 0, 1, 1))]
    assert c["hc1"] == O.holberg(4)[1]
    cp = O.cpml(8, 10.0, 12.0, 2.0, 1.0, 1e-3, 3000.0, 1e-3)
    assert c["cpml_b0"] == cp["b"][0]
    # window defaults (fd_fwi.cu:36-51), clipped to the padded grid
    assert c["window"] == [1, 1, 1, ppad, min(nxt - 1 + ppad, nxt), ppad, min(nzt - 1 + ppad, nzt)]


def test_ini_syntax_and_fallbacks(tmp_path):
    p = tmp_path / "c.ini"
    p.write_text("[GRID]\nNX = 0x20 ; hex like strtol\nnz=16\nnt = 50\nfree_surface = 1\n"
                 "[fdm]\nfdorder=2\n[PML_boundary]\nnpml = 0\n"
                 "[source]\nnseis = 3\nx_seis = { 4 ,5};\nz_seis={1}\nshot_to_fire = {0};\n"
                 "[receiver]\nnseis = 2\nx_seis = {7, 8}\nz_seis = {2, 2}\n"
                 "[full_waveform_inversion]\ngrid_interval_z = 5\ngrid_interval_y = 2\n")
    c = _dry(p)
    assert c["nx"] == 32 and c["nz"] == 16 and c["nt"] == 50 and c["fsurf"] == 1
    fpad, ppad = 1, 1
    # short vectors repeat their last entry; z offsets use fpad with a free surface
    assert [s[0] for s in c["src"]] == [4 + ppad, 5 + ppad, 5 + ppad]
    assert [s[1] for s in c["src"]] == [1 + fpad] * 3
    # the window's z interval is read from grid_interval_y, as the reference does
    assert c["window"][2] == 2


def test_missing_file_fails():
    r = subprocess.run([str(B.APP), "/nonexistent.ini", "--dry-run"], capture_output=True, text=True)
    assert r.returncode == 2 and "can't load" in r.stderr
