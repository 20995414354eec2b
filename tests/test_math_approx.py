"""CPU check of the FP32 normal-tail and inverse-normal approximations used
by the latent draws (bsglmm_gb300/csrc/bsg_math.cuh): the coefficients are
read from the header and both functions are evaluated in float32."""
from __future__ import annotations

import re
from pathlib import Path

import numpy as np
from scipy import special

HDR = Path(__file__).resolve().parents[1] / "bsglmm_gb300" / "csrc" / "bsg_math.cuh"


def coeffs():
    text = HDR.read_text()
    block = text[text.index("BEGIN-COEFFICIENTS"):text.index("END-COEFFICIENTS")]
    return {k: np.float32(float(v)) for k, v in
            re.findall(r"(k\w+)\s*=\s*([-+0-9.eE]+)f", block)}


C = coeffs()
f32 = np.float32


def fma(a, b, c):
    return (a.astype(np.float64) * b + c).astype(np.float32)


def phi_tail32(x):
    x = x.astype(np.float32)
    h = (x * (x * f32(-0.72134752044448170))).astype(np.float32)
    e = np.exp2(h.astype(np.float64)).astype(np.float32)
    n = fma(fma(fma(C["kMillsN3"], x, C["kMillsN2"]), x, C["kMillsN1"]), x, C["kMillsN0"])
    d = fma(fma(fma(fma(C["kMillsD4"], x, C["kMillsD3"]), x, C["kMillsD2"]), x,
                C["kMillsD1"]), x, f32(1))
    return (e * n * (f32(1) / d)).astype(np.float32)


def ndtri_lower32(p):
    p = p.astype(np.float32)
    l = (-np.log2(p.astype(np.float64))).astype(np.float32)
    rho = (l * (1 / np.sqrt(l.astype(np.float64))).astype(np.float32)).astype(np.float32)
    n = fma(fma(fma(fma(fma(C["kNdtN5"], rho, C["kNdtN4"]), rho, C["kNdtN3"]), rho,
                    C["kNdtN2"]), rho, C["kNdtN1"]), rho, C["kNdtN0"])
    d = fma(fma(fma(fma(C["kNdtD4"], rho, C["kNdtD3"]), rho, C["kNdtD2"]), rho,
                C["kNdtD1"]), rho, f32(1))
    return (n * (f32(1) / d)).astype(np.float32)


def test_all_coefficients_parsed():
    assert len(C) == 8 + 10


def test_phi_tail_relative_error():
    x = np.linspace(0, 5, 40001).astype(np.float32)  # the range the sampler uses
    err = np.abs(phi_tail32(x) / special.ndtr(-x.astype(np.float64)) - 1)
    assert err.max() < 2e-6


def test_phi_tail_beyond_fit_range_decays():
    x = np.array([9.5, 12.0, 20.0, 40.0], np.float32)
    t = phi_tail32(x)
    assert np.all(np.isfinite(t)) and np.all(np.diff(t) <= 0)
    assert np.allclose(t[:2], special.ndtr(-x[:2]), rtol=1e-5)


def test_ndtri_lower_relative_error():
    p = np.concatenate([np.logspace(-37, -1.2, 4000),
                        np.linspace(0.06, 0.5, 4000)]).astype(np.float32)
    ref = special.ndtri(p.astype(np.float64))
    got = ndtri_lower32(p)
    assert np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1.0)) < 1e-6
