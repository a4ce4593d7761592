"""Build recipe for the parity checker (test infrastructure only).

* ``build_oracle()`` compiles the C restatement ``oracle/fwi_oracle.c`` into
  ``oracle/_lib/libfwi_oracle.so`` with gcc (``-ffp-contract=off`` so x86-64
  and aarch64 round identically; ``-fopenmp`` where the compiler has it).
* ``build_ref()`` compiles the reference's own CPU path from its sources where
  they lie (``$FWI_REFERENCE_DIR``, default: a ``reference`` checkout beside
  this repository) together with
  ``oracle/ref_harness.cpp`` into ``oracle/_ref/libfwi_ref.so``.  Nothing is
  copied out of the reference tree; every output goes to ``oracle/_ref/``.
  ``CUDA_week2/fd_medium.cu`` holds a Latin-1 byte in a string literal that
  nvcc's front end rejects, so that one file (it has no device code) goes
  through g++ with ``-finput-charset=ISO-8859-1``.  When the reference tree is
  absent (e.g. on the GPU host) ``build_ref()`` does nothing and returns None.

Run ``python oracle/build.py`` to build both.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB_DIR = HERE / "_lib"
REF_DIR = HERE / "_ref"
ORACLE_SO = LIB_DIR / "libfwi_oracle.so"
REF_SO = REF_DIR / "libfwi_ref.so"

CFLAGS = ["-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-std=c11"]


def _run(cmd, cwd=None):
    res = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed ({res.returncode}): {' '.join(map(str, cmd))}\n"
                           f"{res.stdout}\n{res.stderr}")
    return res


def _stale(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build_oracle(force: bool = False) -> Path:
    src = HERE / "fwi_oracle.c"
    deps = [src, HERE / "fwi_oracle.h", Path(__file__)]
    if force or _stale(ORACLE_SO, deps):
        LIB_DIR.mkdir(exist_ok=True)
        cc = os.environ.get("CC", "gcc")
        tmp = ORACLE_SO.with_suffix(".so.tmp")
        try:  # OpenMP cell loops (results do not depend on the thread count)
            _run([cc, *CFLAGS, "-fopenmp", "-shared", "-o", str(tmp), str(src), "-lm"])
        except RuntimeError:
            _run([cc, *CFLAGS, "-shared", "-o", str(tmp), str(src), "-lm"])
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def reference_root() -> Path:
    """The reference checkout: $FWI_REFERENCE_DIR, else ``../reference`` beside this repository."""
    env = os.environ.get("FWI_REFERENCE_DIR")
    return Path(env) if env else HERE.parent.parent / "reference"


def reference_dir() -> Path:
    return reference_root() / "CUDA_week2"


def build_ref(force: bool = False) -> Path | None:
    ref = reference_dir()
    if not (ref / "forward_kernel_PSV_GPU.cu").exists():
        return None
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cuda_inc = Path(nvcc).resolve().parent.parent / "include"
    harness = HERE / "ref_harness.cpp"
    nv_units = ["forward_kernel_PSV_GPU", "adjoint_kernel_PSV_GPU", "fd_cpml", "holbergcoeff",
                "fd_seismogram"]
    deps = [harness, Path(__file__)] + [ref / f"{u}.cu" for u in nv_units] + [ref / "fd_medium.cu"]
    if not force and not _stale(REF_SO, deps):
        return REF_SO
    REF_DIR.mkdir(exist_ok=True)
    obj = REF_DIR / "obj"
    obj.mkdir(exist_ok=True)
    # The reference's device kernels are compiled (they share files with the CPU
    # path) but never launched: the harness calls only the CPU functions.
    nvflags = ["-c", "-O2", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
               "-gencode", "arch=compute_103a,code=sm_103a", "-w", f"-I{ref}"]
    jobs = [[nvcc, *nvflags, str(ref / f"{u}.cu"), "-o", str(obj / f"{u}.o")] for u in nv_units]
    jobs.append(["g++", "-c", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-w",
                 "-finput-charset=ISO-8859-1", "-x", "c++", f"-I{ref}", f"-I{cuda_inc}",
                 str(ref / "fd_medium.cu"), "-o", str(obj / "fd_medium.o")])
    jobs.append(["g++", "-c", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-w",
                 f"-I{ref}", f"-I{cuda_inc}", str(harness), "-o", str(obj / "ref_harness.o")])
    with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    objs = [str(obj / f"{u}.o") for u in nv_units] + [str(obj / "fd_medium.o"),
                                                       str(obj / "ref_harness.o")]
    tmp = REF_SO.with_suffix(".so.tmp")
    _run([nvcc, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", str(tmp), *objs])
    os.replace(tmp, REF_SO)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
