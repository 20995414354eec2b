"""Builds libbsglmm_gb300.so in-tree with nvcc for sm_103a.

Each translation unit is compiled in parallel; the shared library lands in
``bsglmm_gb300/lib/``.  Usage: ``python -m bsglmm_gb300.build [--force]``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "lib"
BUILD = PKG / "_build"
LIBNAME = "libbsglmm_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-O2", "--expt-relaxed-constexpr"]

SOURCES = [
    "bsg_fused_l1.cu",
    "bsg_fused_l2.cu",
    "bsg_fused_l4.cu",
    "bsg_fused_l8.cu",
    "bsg_fused_mix.cu",
    "bsg_fused_wm.cu",
    "bsg_fp64.cu",
    "bsg_fused_tc.cu",
    "bsg_fused_wide.cu",
    "bsg_kernels.cu",
    "bsg_peak.cu",
    "bsg_noalloc.cu",
    "bsg_predict.cu",
    "bsg_api.cpp",
]
HEADERS = ["bsg_device.cuh", "bsg_fused.cuh", "bsg_internal.h", "bsg_math.cuh",
           "bsg_wishart.cuh", "bsg_mma.cuh"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"),
                 "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def lib_path() -> Path:
    return OUT / LIBNAME


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    deps = [src] + [CSRC / h for h in HEADERS] + [PKG.parent / "include" / "bsglmm_gb300.h"]
    t = obj.stat().st_mtime
    return any(d.exists() and d.stat().st_mtime > t for d in deps)


def _compile(src: str, force: bool, extra: list[str]) -> Path:
    s = CSRC / src
    obj = BUILD / (src + ".o")
    if force or _stale(obj, s):
        cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", str(s), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        if r.stderr.strip():
            sys.stderr.write(r.stderr)
    return obj


DRIVER_SRC = CSRC / "driver" / "bsglmm_main.cpp"
DRIVER = OUT / "bsglmm"


def build_driver(force: bool = False) -> Path:
    """The `bsglmm` command (C++ driver over the C ABI), linked against the
    in-tree library with an $ORIGIN run path."""
    lib = lib_path()
    hdr = PKG.parent / "include" / "bsglmm_gb300.h"
    if (force or not DRIVER.exists()
            or any(p.stat().st_mtime > DRIVER.stat().st_mtime for p in (DRIVER_SRC, hdr, lib))):
        cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
        cmd = [cxx, "-O2", "-std=c++17", "-o", str(DRIVER), str(DRIVER_SRC), f"-L{OUT}",
               "-lbsglmm_gb300", "-Wl,-rpath,$ORIGIN", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"driver build failed:\n{r.stderr}")
    return DRIVER


def build(force: bool = False, verbose_ptxas: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    OUT.mkdir(exist_ok=True)
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, force, extra), SOURCES))
    lib = lib_path()
    if force or not lib.exists() or any(o.stat().st_mtime > lib.stat().st_mtime for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(lib), *map(str, objs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    build_driver(force)
    return lib


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose_ptxas="--ptxas-v" in sys.argv)
    print(p)
