"""CPU tests of host-side logic: synthetic study shapes and the reference's
thinning rule."""
from __future__ import annotations

import numpy as np

from bsglmm_gb300 import save_iter_rule, synth


def test_save_iter_rule_matches_mcmc_cpp():
    # mcmc.cpp:303-308
    assert save_iter_rule(3000, 1000) == 2000
    assert save_iter_rule(100000, 50000) == 5
    assert save_iter_rule(20000, 10000) == 1


def test_config0_shape():
    st = synth.config0()
    assert st.mask.shape == (20, 20, 20)
    assert st.V == 3112  # sphere r = 9 about (10.5, 10.5, 10.5)
    assert st.covar.shape == (3, 50) and st.data.shape == (50, 3112)
    assert set(np.unique(st.data)) <= {0, 1}
    assert np.all(st.covar[0] == 1) and set(np.unique(st.covar[1])) == {-0.5, 0.5}


def test_brain_mask_size():
    m = synth.ellipsoid_mask(synth.BRAIN_SHAPE, synth.BRAIN_AXES)
    assert 220_000 < int(m.sum()) < 240_000


def test_small_study_edge_cases():
    st = synth.small_study(3)
    assert st.mask[0, 0, 0] == 1 and st.mask[0, 0, 1] == 0  # isolated corner
    assert st.N % 32 != 0
