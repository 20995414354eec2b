"""The NIfTI readers on the images the reference ships (bsglmm/images:
mask.nii.gz, FLOAT64, 91x109x91, 2 mm; avg152T1_white.nii.gz, UINT8), read
in place where the reference tree is mounted (CPU only; skipped elsewhere).

- Both the Python reader and the C++ `bsglmm` command read the gzipped
  FLOAT64 mask: 274,596 in-mask voxels, the count of the reference's own
  data; the WM image reads as UINT8 on the same grid.
- A study on that mask (synthetic lesion maps, two groups) gives the same
  empirical maps from the C++ command (which stops at the sampler without a
  GPU) and from the Python driver's readers.
"""
from __future__ import annotations

import shutil
import subprocess

import numpy as np
import pytest

import oracle
from bsglmm_gb300 import build, driver, nifti

IMAGES = oracle.reference_tree() / "images"


@pytest.fixture(scope="module")
def ref_images():
    if not (IMAGES / "mask.nii.gz").exists():
        pytest.skip("the reference's images are not mounted here")
    return IMAGES


def test_reference_mask_and_wm(ref_images):
    mask = driver.read_mask(ref_images / "mask.nii.gz")
    assert mask.shape == (91, 109, 91)
    assert int(mask.sum()) == 274596
    img = nifti.read_nifti(ref_images / "avg152T1_white.nii.gz")
    assert img.datatype == nifti.UINT8 and img.dims == (91, 109, 91)
    assert img.pixdim == pytest.approx((2.0, 2.0, 2.0))
    wm = driver.read_wm(ref_images / "avg152T1_white.nii.gz", mask)
    assert wm.shape == (274596,) and 0.0 <= wm.min() and wm.max() <= 1.0


def test_cpp_command_reads_the_reference_mask(ref_images, tmp_path):
    exe = build.DRIVER
    if not exe.exists():
        build.build()
    img = tmp_path / "images"
    img.mkdir()
    shutil.copy(ref_images / "mask.nii.gz", img / "mask.nii.gz")
    mask = driver.read_mask(img / "mask.nii.gz")
    m = mask.astype(bool)
    rng = np.random.default_rng(3)
    N = 6
    lines = ["ID G0 G1 Image"]
    for i in range(N):
        vol = np.zeros(mask.shape)
        vol[m] = rng.random(int(m.sum())) < 0.05
        nifti.write_nifti(img / f"s{i}.nii.gz", vol, (91, 109, 91), datatype=nifti.FLOAT32)
        lines.append(f"S{i} {int(i % 2 == 0)} {int(i % 2 == 1)} s{i}.nii.gz")
    (tmp_path / "design.txt").write_text("\n".join(lines) + "\n")
    r = subprocess.run([str(exe), "2", "2", "1", "design.txt", "1", "0", "10", "0"],
                       cwd=tmp_path, capture_output=True, text=True, timeout=600)
    if r.returncode == 0:
        pytest.skip("a GPU is present: the whole run is compared in the GPU driver tests")
    assert r.returncode == 3, r.stderr
    # the empirical maps from the same inputs, through the Python readers
    data = np.stack([driver._as_byte(nifti.read_nifti(img / f"s{i}.nii.gz").data[m])
                     for i in range(N)])
    covar = np.array([[float(i % 2 == 0) for i in range(N)],
                      [float(i % 2 == 1) for i in range(N)]], np.float32)
    groups, total, total_p = driver.empirical_maps(mask, covar, data, 2)
    for g, nm in enumerate(["G0", "G1"]):
        got = nifti.read_nifti(tmp_path / f"empir_prb_{nm}.nii.gz").data.ravel()
        assert np.array_equal(got, groups[g])
    assert np.array_equal(nifti.read_nifti(tmp_path / "total_lesion_cnt.nii.gz").data.ravel(),
                          total)
    assert np.array_equal(nifti.read_nifti(tmp_path / "total_empir_prb.nii.gz").data.ravel(),
                          total_p)
