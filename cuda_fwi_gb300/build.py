"""Build ``libfwi_psv.so`` (the sm_103a engine + C ABI) in-tree with nvcc.

Output: ``cuda_fwi_gb300/_lib/libfwi_psv.so``, the INI-driven host program
``cuda_fwi_gb300/_lib/fwi_run`` (app/, plain C++ against the C ABI) and
``cuda_fwi_gb300/_lib/ref_driver``, a reference-style caller of the drop-in
propagator symbols (app/ref_driver.cpp).
Translation units are compiled in parallel and only when a source is newer
than its object.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_lib"
OBJ_DIR = OUT_DIR / "obj"
LIB = OUT_DIR / "libfwi_psv.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
           "--expt-relaxed-constexpr", f"-I{ROOT / 'include'}", f"-I{CSRC}"]
UNITS = ["fwi_engine.cu", "fwi_host.cpp", "fwi_refshim.cpp", "fwi_noalloc.cu", "fwi_optim.cu"]
HEADERS = ["fwi_kernels.cuh", "fwi_exact.cuh", "fwi_tma.cuh", "fwi_fused.cuh", "fwi_multi.cuh", "fwi_host.h",
           "fwi_alloc.hpp"]
APP_DIR = PKG / "app"
APP = OUT_DIR / "fwi_run"
REF_DRIVER = OUT_DIR / "ref_driver"


def nvcc() -> str:
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def build(force: bool = False, verbose_ptxas: bool = False, defines=(), out: Path | None = None) -> Path:
    """Compile the library; `defines` (e.g. ["FWI_MIN_BLOCKS=4"]) and `out`
    build a variant into another directory."""
    if defines or out:
        return _build_variant(list(defines), Path(out) if out else OUT_DIR / "variant.so")
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    deps = [CSRC / h for h in HEADERS] + [ROOT / "include" / "fwi_psv.h", Path(__file__)]
    newest_dep = max(p.stat().st_mtime for p in deps if p.exists())
    jobs, objs = [], []
    for u in UNITS:
        src = CSRC / u
        obj = OBJ_DIR / (u + ".o")
        objs.append(obj)
        if force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, newest_dep):
            extra = ["-Xptxas", "-v"] if (verbose_ptxas and u.endswith(".cu")) else []
            jobs.append([nvcc(), "-c", *ARCH, *NVFLAGS, *extra, str(src), "-o", str(obj)])
    logs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            logs = list(ex.map(_run, jobs))
    if jobs or not LIB.exists():
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc(), "-shared", *ARCH, "-o", str(tmp), *map(str, objs)])
        os.replace(tmp, LIB)
    app_deps = [APP_DIR / "fwi_main.cpp", APP_DIR / "ini.hpp", ROOT / "include" / "fwi_psv.h", LIB]
    if force or not APP.exists() or APP.stat().st_mtime < max(p.stat().st_mtime for p in app_deps):
        build_app()
    drv_deps = [APP_DIR / "ref_driver.cpp", ROOT / "include" / "fwi_psv_ref.hpp", ROOT / "include" / "fwi_psv.h", LIB]
    if force or not REF_DRIVER.exists() or REF_DRIVER.stat().st_mtime < max(p.stat().st_mtime for p in drv_deps):
        build_ref_driver()
    if verbose_ptxas:
        print("\n".join(logs))
    return LIB


def build_app() -> Path:
    """The host driver: g++ against the C ABI, libfwi_psv.so found next to it."""
    cxx = os.environ.get("CXX", "g++")
    tmp = APP.with_suffix(".tmp")
    _run([cxx, "-O2", "-std=c++17", f"-I{ROOT / 'include'}", f"-I{APP_DIR}", str(APP_DIR / "fwi_main.cpp"),
          "-o", str(tmp), f"-L{OUT_DIR}", "-lfwi_psv", "-Wl,-rpath,$ORIGIN"])
    os.replace(tmp, APP)
    return APP


def build_ref_driver() -> Path:
    """A reference-style caller of the drop-in propagators (app/ref_driver.cpp):
    host code compiled by nvcc (for the CUDA runtime it allocates with),
    linked against libfwi_psv.so found next to it."""
    tmp = REF_DRIVER.with_suffix(".tmp")
    _run([nvcc(), "-O2", "-std=c++17", f"-I{ROOT / 'include'}", str(APP_DIR / "ref_driver.cpp"), "-o", str(tmp),
          f"-L{OUT_DIR}", "-lfwi_psv", "-Xlinker", "-rpath,$ORIGIN"])
    os.replace(tmp, REF_DRIVER)
    return REF_DRIVER


def _build_variant(defines, out: Path) -> Path:
    out.parent.mkdir(parents=True, exist_ok=True)
    objdir = out.parent / (out.stem + "_obj")
    objdir.mkdir(exist_ok=True)
    dflags = [f"-D{d}" for d in defines]
    jobs = [[nvcc(), "-c", *ARCH, *NVFLAGS, *dflags, str(CSRC / u), "-o", str(objdir / (u + ".o"))]
            for u in UNITS]
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(_run, jobs))
    _run([nvcc(), "-shared", *ARCH, "-o", str(out), *[str(objdir / (u + ".o")) for u in UNITS]])
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
