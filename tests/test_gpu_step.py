"""The probit colour kernel's two whole-word steps (bsg_set_step_subjects):
16 subjects from four Philox calls at two resident blocks, or 8 from two at
three.  Both draw the same variates with the same arithmetic in the same
order, so chains agree bit for bit: coefficients, Omega and the posterior
sums, for P = 1..8, ragged subject counts, the beta_WM update, graph
segments and batched chains; the per-group choice (0) equals both, and an
unsupported step is refused.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _wm(st, seed):
    return np.random.default_rng(seed).random(st.V).astype(np.float32)


def _run(studies, step, sweeps=5, wm=False, lpv=0):
    import bsglmm_gb300 as bsg
    out = []
    with bsg.Sampler() as s:
        chains = []
        for k, st in enumerate(studies):
            ds = s.add_dataset(st.mask, st.covar, st.data, st.nsubtypes,
                               wm=_wm(st, k) if wm else None)
            c = s.add_chain(ds, seed=40 + k, beta_wm=0.3 if wm else 0.0)
            if wm:
                s.set_wm_update(c, True)
            chains.append(c)
        if lpv:
            s.set_tuning(lpv, 0)
        s.set_step_subjects(step)
        s.run(sweeps)
        used = s.step_subjects()
        for c in chains:
            m, v, prb, n = s.posterior(c)
            out.append((s.beta(c), s.omega(c), m, v, prb))
    return out, used


def _same(a, b):
    for x, y in zip(a, b):
        for u, w in zip(x, y):
            assert np.array_equal(u, w)


@pytest.mark.parametrize("P,N", [(1, 45), (2, 64), (3, 50), (4, 77), (5, 130), (6, 33),
                                 (7, 96), (8, 41)])
def test_steps_agree_bit_for_bit(P, N):
    from bsglmm_gb300 import synth
    st = synth.small_study(90 + P, shape=(11, 10, 9), N=N, P=P, S=1)
    a, ua = _run([st], 8)
    b, ub = _run([st], 16)
    c, _ = _run([st], 0)
    assert (ua, ub) == (8, 16)
    _same(a, b)
    _same(a, c)


def test_steps_agree_with_beta_wm_update_and_batched_chains():
    from bsglmm_gb300 import synth
    sts = [synth.small_study(5, shape=(12, 11, 10), N=70, P=3, S=1),
           synth.small_study(6, shape=(9, 12, 10), N=300, P=3, S=1)]
    a, _ = _run(sts, 8, wm=True)
    b, _ = _run(sts, 16, wm=True)
    _same(a, b)
    a, _ = _run(sts, 8, sweeps=70)  # a 64-sweep graph segment and more
    b, _ = _run(sts, 16, sweeps=70)
    _same(a, b)


def test_auto_choice_and_refusal():
    import bsglmm_gb300 as bsg
    from bsglmm_gb300 import synth
    st = synth.small_study(7, shape=(10, 10, 10), N=40, P=3, S=1)
    # a grid of a few blocks leaves the SMs room: 16 subjects
    _, used = _run([st], 0)
    assert used == 16
    # lanes per voxel > 1 keep the 8-subject step
    _, used = _run([st], 16, lpv=2)
    assert used == 8
    with bsg.Sampler() as s:
        ds = s.add_dataset(st.mask, st.covar, st.data, st.nsubtypes)
        s.add_chain(ds, seed=1)
        with pytest.raises(RuntimeError):
            s.set_step_subjects(12)


def test_per_group_choice_on_the_benchmark_studies():
    """16 subjects for one chain of the brain-sized study (N = 1000); 8 for
    64 chains of the 20^3 study (N = 50), whose grid fills the GPU."""
    import bsglmm_gb300 as bsg
    from bsglmm_gb300 import synth
    brain = synth.config1(seed=1)
    with bsg.Sampler() as s:
        s.add_chain(s.add_dataset(brain.mask, brain.covar, brain.data, brain.nsubtypes),
                    seed=1)
        assert s.step_subjects() == 16
    small = synth.config0(0)
    with bsg.Sampler() as s:
        ds = s.add_dataset(small.mask, small.covar, small.data, small.nsubtypes)
        for c in range(64):
            s.add_chain(ds, seed=1 + c)
        assert s.step_subjects() == 8
        s.set_step_subjects(16)
        assert s.step_subjects() == 16
