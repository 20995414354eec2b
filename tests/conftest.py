"""Shared test set-up: the `gpu` marker, import paths, golden fixtures."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
for p in (ROOT, ROOT / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")


def golden_cases():
    return sorted(p.stem for p in GOLDEN.glob("sweep_*.npz"))


def load_golden(name: str) -> dict:
    with np.load(GOLDEN / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build_oracle()
    return oracle


def omega_rel_err(om, ref, tiny: float = 1e-2) -> float:
    """Worst elementwise relative error of a precision matrix against its
    reference over the entries that are not tiny (|ref| >= tiny * max|ref|);
    the tiny ones are measured against tiny * max|ref| instead.  (The
    reference forms Omega from FP32 pair sums and stores it in FP32, so its
    near-zero off-diagonal entries carry an absolute rounding of about
    1e-8 max|Omega|: an exact FP64 restatement differs from it by 7e-5
    relative on an entry of 2e-4 max|Omega|.)"""
    om = np.asarray(om, np.float64)
    ref = np.asarray(ref, np.float64)
    scale = np.maximum(np.abs(ref), tiny * np.abs(ref).max())
    return float((np.abs(om - ref) / scale).max())
