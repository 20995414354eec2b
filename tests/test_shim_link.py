"""CPU check that the drop-in shim links in place of the reference's
covarGPU.cu: every symbol that the reference's mcmc.cpp and main.cu take
from covarGPU.cu is defined by covarGPU_shim.cu with the same (mangled)
name.  Needs the reference tree, so it only runs where that is mounted."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

import oracle

ROOT = Path(__file__).resolve().parents[1]
REF = oracle.reference_tree()


def _nm(obj: Path, flag: str) -> set[str]:
    out = subprocess.run(["nm", flag, str(obj)], capture_output=True, text=True,
                         check=True).stdout
    syms = set()
    for line in out.splitlines():
        parts = line.split()
        if flag == "-u" and parts:
            syms.add(parts[-1])
        elif flag == "--defined-only" and len(parts) >= 3 and parts[1] in "TtWwBbDd":
            syms.add(parts[2])
    return syms


def test_shim_defines_what_the_reference_loop_needs(tmp_path):
    if not REF.exists():
        pytest.skip("reference tree not mounted")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    arch = ["-gencode", "arch=compute_100,code=sm_100"]

    def cc(src: Path, name: str, extra=()) -> Path:
        obj = tmp_path / name
        cmd = [nvcc, *arch, "-w", "-x", "cu", "-c", str(src), "-o", str(obj),
               "-I", str(REF), *extra]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-2000:]
        return obj

    mcmc = cc(REF / "mcmc.cpp", "mcmc.o")
    main = cc(REF / "main.cu", "main.o")
    gpu = cc(REF / "covarGPU.cu", "covarGPU.o")
    shim = cc(ROOT / "bsglmm_gb300" / "csrc" / "shim" / "covarGPU_shim.cu", "shim.o")
    needed = (_nm(mcmc, "-u") | _nm(main, "-u")) & _nm(gpu, "--defined-only")
    assert needed, "expected the reference loop to use covarGPU.cu symbols"
    missing = sorted(needed - _nm(shim, "--defined-only"))
    assert not missing, missing
