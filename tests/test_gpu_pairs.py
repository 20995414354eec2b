"""The paired (f32x2) forms of the latent-draw helpers equal their scalar
forms bit for bit: the truncated-normal inversion, the normal map, the first
Marsaglia-Tsang attempt (value and acceptance) and the A&S / logistic
log-likelihoods of the predictive pass, on 4M seeded random inputs each."""
from __future__ import annotations

import ctypes as C

import pytest

pytestmark = pytest.mark.gpu


def test_paired_helpers_equal_scalar_forms():
    from bsglmm_gb300 import _lib
    L = _lib.lib()
    bad = C.c_int64(-1)
    assert L.bsg_selftest_pairs(0, 1 << 22, 0x5EED_0001_2345_6789, C.byref(bad)) == 0
    assert bad.value == 0
