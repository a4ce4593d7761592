"""The exact-signature drop-in, executed by a reference-style C++ caller.

``cuda_fwi_gb300/_lib/ref_driver`` (app/ref_driver.cpp) calls
forward_kernel_PSV_GPU and adjoint_kernel_PSV_GPU the way the reference's FWI
driver does (CUDA_week2/fd_wave_model.cu:498-591): row-pointer host tables,
``std::vector<int>`` arguments by value and cudaMalloc'd FP64 ``d_*`` buffers.
Its outputs -- host results and the device buffers copied back -- are
compared with the golden fixtures made by the reference's own compiled CPU
path (tests/golden/make_golden.py), at the tolerances of the other parity
tests.
"""
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

from cuda_fwi_gb300 import build as B
from oracle import oracle as O

from _fixtures import load

pytestmark = pytest.mark.gpu

SEIS_TOL, GRAD_TOL = 1e-5, 1e-4
INTS = ("nt", "nzt", "nxt", "fpad", "ppad", "npml", "fdorder", "fsurf", "fwi_dt", "fwi_dx", "fwi_dz",
        "x1", "x2", "z1", "z2")


def rel_l2(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def write_blobs(path, f64, i32):
    with open(path, "wb") as fp:
        for name, arr in list(f64.items()) + list(i32.items()):
            kind = 0 if name in f64 else 1
            a = np.ascontiguousarray(arr, np.float64 if kind == 0 else np.int32).ravel()
            nb = name.encode()
            fp.write(struct.pack("<I", len(nb)) + nb + struct.pack("<IQ", kind, a.size) + a.tobytes())


def read_blobs(path):
    out, buf, o = {}, Path(path).read_bytes(), 0
    while o < len(buf):
        (nl,) = struct.unpack_from("<I", buf, o)
        o += 4
        name = buf[o:o + nl].decode()
        o += nl
        kind, n = struct.unpack_from("<IQ", buf, o)
        o += 12
        dt = np.float64 if kind == 0 else np.int32
        out[name] = np.frombuffer(buf, dt, n, o).copy()
        o += n * np.dtype(dt).itemsize
    return out


@pytest.mark.parametrize("name", ["ref_o2.npz", "ref_o2_fsurf.npz", "ref_o2_multi.npz"])
def test_reference_style_caller_matches_golden(name, tmp_path):
    drv = B.REF_DRIVER
    assert drv.exists(), "build() makes the reference-style driver"
    p, d = load(name)
    mu_zx, rho_zp, rho_xp = O.average(p.lam, p.mu, p.rho)
    f64 = {"dt": [p.dt], "dx": [p.dx], "dz": [p.dz], "hc": p.hc, "lam": p.lam, "mu": p.mu, "mu_zx": mu_zx,
           "rho_zp": rho_zp, "rho_xp": rho_xp, "src_signal": p.src_signal, "obs": d["obs"]}
    for k, v in p.cpml.items():
        f64["cpml_" + k] = v
    i32 = {k: [int(getattr(p, k))] for k in INTS}
    i32["shot"] = [int(d["shot"])]
    for k in ("src_x", "src_z", "src_comp", "src_shot", "rec_x", "rec_z", "rec_comp", "rec_shot"):
        i32[k] = getattr(p, k)
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    write_blobs(fin, f64, i32)
    r = subprocess.run([str(drv), str(fin), str(fout)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    o = read_blobs(fout)
    rows = O.shot_rows(p, int(d["shot"]))
    shape = (p.nzt, p.nxt)
    rec = o["fwd_rec"].reshape(p.nrec, p.nt)
    assert rel_l2(rec[rows], d["out_rec"][rows]) <= SEIS_TOL
    assert rel_l2(o["fwd_vz"].reshape(shape), d["out_fwd_vz"]) <= SEIS_TOL
    assert rel_l2(o["fwd_szz"].reshape(shape), d["out_fwd_szz"]) <= SEIS_TOL
    # the caller's device buffers received the final wavefield, We and the storage
    assert rel_l2(o["fwd_d_We"].reshape(shape), d["out_fwd_We"]) <= SEIS_TOL
    assert rel_l2(o["fwd_d_vz"].reshape(shape), d["out_fwd_vz"]) <= SEIS_TOL
    assert rel_l2(o["fwd_d_sxx"].reshape(shape), d["out_fwd_sxx"]) <= SEIS_TOL
    st = d["out_store_szz"].shape
    assert rel_l2(o["fwd_d_store_szz"].reshape(st), d["out_store_szz"]) <= SEIS_TOL
    assert rel_l2(o["fwd_d_store_vx"].reshape(st), d["out_store_vx"]) <= SEIS_TOL
    assert rel_l2(o["fwd_store_sxx"].reshape(st), d["out_store_sxx"]) <= SEIS_TOL
    assert float(o["misfit"][0]) == pytest.approx(float(d["out_misfit"]), rel=1e-4)
    gshape = d["out_adj_grad_lam"].shape
    for k in ("grad_lam", "grad_mu", "grad_rho"):
        host = o["adj_" + k].reshape(gshape)
        assert rel_l2(host, d["out_adj_" + k]) <= GRAD_TOL, k
        assert np.array_equal(o["adj_d_" + k].reshape(gshape), host), k
    assert rel_l2(o["adj_d_We"].reshape(shape), d["out_adj_We"]) <= GRAD_TOL
    assert rel_l2(o["adj_vz"].reshape(shape), d["out_adj_vz"]) <= GRAD_TOL
