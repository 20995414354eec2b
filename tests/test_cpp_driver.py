"""The C++ `bsglmm` command (bsglmm_gb300/csrc/driver/bsglmm_main.cpp, built
into bsglmm_gb300/lib/bsglmm): the reference program's command line over the
C ABI.  It must write what the Python driver writes.

- CPU: usage and input errors; the empirical maps (written before the
  sampler starts) equal the Python driver's, and without a GPU the run stops
  at the sampler with exit status 3.
- GPU: a whole run equals the Python driver's run file for file: every map
  (decompressed), Qhat.dat, Qhat2.dat, DIC.dat and the advanced seed.dat.
"""
from __future__ import annotations

import subprocess
from pathlib import Path

import numpy as np
import pytest

from bsglmm_gb300 import build, driver, nifti
from test_driver import write_study

EXE = build.DRIVER


@pytest.fixture(scope="module")
def exe():
    if not EXE.exists():
        build.build()
    return str(EXE)


def _run(exe, args, cwd):
    return subprocess.run([exe, *args], cwd=cwd, capture_output=True, text=True, timeout=600)


def test_usage_and_input_errors(exe, tmp_path):
    r = _run(exe, [], tmp_path)
    assert r.returncode == 1 and "Usage" in r.stdout
    assert _run(exe, ["1", "2", "1", "d.txt", "1"], tmp_path).returncode == 1
    assert _run(exe, ["x", "2", "1", "d.txt", "1", "0"], tmp_path).returncode == 1
    r = _run(exe, ["1", "2", "0", "d.txt", "1", "0"], tmp_path)
    assert r.returncode == 2 and "GPU = 0" in r.stderr
    r = _run(exe, ["1", "2", "1", "d.txt", "1", "1"], tmp_path)
    assert r.returncode == 2 and "mask.nii.gz: no such file" in r.stderr
    r = _run(exe, ["1", "2", "1", "d.txt", "1", "0", "10", "20"], tmp_path)
    assert r.returncode == 2
    assert "Silly-small" in r.stdout and "Burn-in exceeds" in r.stdout


def test_design_errors(exe, tmp_path):
    write_study(tmp_path)
    (tmp_path / "bad.txt").write_text("ID G0 G1 Cov0 Image\nS0 1 0 0.5\n")
    r = _run(exe, ["2", "3", "1", "bad.txt", "1", "0", "10", "0"], tmp_path)
    assert r.returncode == 2 and "multiple of NCov+2" in r.stderr
    r = _run(exe, ["4", "3", "1", "design.txt", "1", "0", "10", "0"], tmp_path)
    assert r.returncode == 2 and "NTypes cannot exceed NCov" in r.stderr


def _same_images(a: Path, b: Path, names):
    for nm in names:
        x = nifti.read_nifti(a / f"{nm}.nii.gz")
        y = nifti.read_nifti(b / f"{nm}.nii.gz")
        assert x.dims == y.dims and x.datatype == y.datatype == nifti.FLOAT64
        assert np.array_equal(x.data, y.data, equal_nan=True), nm
        assert x.pixdim == y.pixdim


def test_empirical_maps_equal_python_driver(exe, tmp_path, monkeypatch):
    a, b = tmp_path / "cpp", tmp_path / "py"
    for d in (a, b):
        st = write_study(d, seed=7)
        (d / "seed.dat").write_text("4 5 6\n")
    args = [str(st["ntypes"]), str(st["P"]), "1", "design.txt", "1", "0", "1000", "10"]
    r = _run(exe, args, a)
    if r.returncode == 0:
        pytest.skip("a GPU is present: the whole run is compared in the GPU test")
    assert r.returncode == 3, r.stderr  # stops at the sampler without a GPU
    monkeypatch.chdir(b)
    try:
        driver.main(args)
    except Exception:  # noqa: BLE001 -- no GPU for the sampler here either
        pass
    names = [f"empir_prb_{st['names'][g]}" for g in range(st["ntypes"])]
    _same_images(a, b, names + ["total_lesion_cnt", "total_empir_prb"])


@pytest.mark.gpu
@pytest.mark.parametrize("wm", [False, True])
def test_cpp_run_equals_python_driver(exe, tmp_path, monkeypatch, capsys, wm):
    a, b = tmp_path / "cpp", tmp_path / "py"
    for d in (a, b):
        st = write_study(d, seed=11, N=29, shape=(11, 10, 9))
        (d / "seed.dat").write_text("21 22 23\n")
        if wm:
            rng = np.random.default_rng(3)
            vol = rng.integers(0, 256, (9, 10, 11)).astype(np.float64)
            nifti.write_nifti(d / "images" / "wm.nii", vol, (11, 10, 9), datatype=nifti.UINT8)
    args = [str(st["ntypes"]), str(st["P"]), "1", "design.txt", "1",
            "wm.nii" if wm else "0", "1500", "500"]
    r = _run(exe, args, a)
    assert r.returncode == 0, r.stderr
    monkeypatch.chdir(b)
    assert driver.main(args) == 0
    py_out = capsys.readouterr().out
    assert r.stdout.splitlines()[-2:] == py_out.splitlines()[-2:]  # TOTSAV, DIC
    assert "iter = 1500" in r.stdout
    names = ([f"empir_prb_{g}" for g in st["names"][:st["ntypes"]]]
             + ["total_lesion_cnt", "total_empir_prb"]
             + [f"spatCoef_{n}" for n in st["names"]]
             + [f"spatCoef_{n}.Var" for n in st["names"]]
             + [f"standCoef_{n}" for n in st["names"]]
             + [f"prb_{g}" for g in st["names"][:st["ntypes"]]]
             + (["bWM"] if wm else []))
    _same_images(a, b, names)
    for f in ("Qhat.dat", "Qhat2.dat", "DIC.dat", "seed.dat"):
        assert (a / f).read_text() == (b / f).read_text(), f
