"""The white-matter coefficient update (updateBetaGPU, covarGPU.cu:585-724;
mcmc.cpp:344-345): beta_WM | Z, beta drawn after both colours' coefficient
updates.  GPU chain against the FP64 oracle chain on the same counters,
recovery of a known beta_WM, determinism across graph segments, checkpoint
continuity, and the design requirement."""
from __future__ import annotations

import numpy as np
import pytest

from bsglmm_gb300 import synth


def _wm_study(seed, shape=(12, 11, 10), N=40, P=3, beta_wm=1.5):
    """Intercept + covariates, a voxelwise-random WM map in [0, 1] (so that
    beta_WM is identified apart from the smooth intercept field) and
    outcomes drawn with eta = -0.6 + beta_WM WM_v + noise."""
    rng = np.random.default_rng(seed)
    X, Y, Z = shape
    mask = (rng.random((Z, Y, X)) < 0.7).astype(np.uint8)
    V = int(mask.sum())
    covar = np.ones((P, N), np.float32)
    covar[1:] = rng.standard_normal((P - 1, N)).astype(np.float32)
    wm = rng.random(V).astype(np.float32)
    beta = np.zeros((P, V), np.float32)
    beta[0] = -0.6 + 0.1 * rng.standard_normal(V)
    beta[1:] = 0.2 * rng.standard_normal((P - 1, V))
    eta = covar.T @ beta + beta_wm * wm[None, :]
    data = (rng.standard_normal((N, V)) < eta).astype(np.uint8)
    return mask, covar, data, wm


@pytest.mark.gpu
def test_gpu_wm_chain_matches_oracle_chain(oracle_mod):
    import bsglmm_gb300 as bsg
    mask, covar, data, wm = _wm_study(1, shape=(9, 8, 7), N=33)
    pb = oracle_mod.Problem(mask, covar, data, 1, wm)
    seed = 0xBEEF_1234
    with bsg.Sampler() as s:
        ds = s.add_dataset(mask, covar, data, 1, wm)
        ch = s.add_chain(ds, seed=seed, beta_wm=0.3)
        s.set_wm_update(ch, True)
        s.run(1)
        o = pb.chain(seed, 1, beta_wm=0.3, wm_update=True)
        assert np.allclose(s.beta(ch), o["beta"], rtol=1e-4, atol=1e-4)
        b1, _ = s.beta_wm(ch)
        assert b1 == pytest.approx(o["beta_wm"], rel=1e-4, abs=1e-5)
        assert b1 != 0.3
        s.run(3)
        o = pb.chain(seed, 3, s0=1, spatcoef=o["beta"], omega=o["omega"],
                     beta_wm=o["beta_wm"], wm_update=True)
        assert np.allclose(s.beta(ch), o["beta"], rtol=2e-3, atol=2e-3)
        assert s.beta_wm(ch)[0] == pytest.approx(o["beta_wm"], rel=2e-3, abs=1e-4)


@pytest.mark.gpu
def test_gpu_wm_posterior_recovers_known_coefficient():
    import bsglmm_gb300 as bsg
    mask, covar, data, wm = _wm_study(2, N=60, beta_wm=1.5)
    with bsg.Sampler() as s:
        ds = s.add_dataset(mask, covar, data, 1, wm)
        ch = s.add_chain(ds, seed=11, burnin=300, thin=1)
        s.set_wm_update(ch, True)
        trace = []
        for _ in range(900):
            s.run(1)
            trace.append(s.beta_wm(ch)[0])
        cur, mean = s.beta_wm(ch)
        nkept = s.sweep_count(ch)[1]
    tr = np.array(trace[301:])
    assert nkept == 599
    assert mean == pytest.approx(tr.mean(), rel=1e-5)
    assert abs(mean - 1.5) < 0.15, mean
    assert 0.0 < tr.std() < 0.2


@pytest.mark.gpu
def test_gpu_wm_graph_segments_equal_single_sweeps_and_checkpoint():
    """Colour-0 launches do not start early when beta_WM is drawn (their
    latent phase reads it): an 8-sweep graph equals 8 single sweeps bit for
    bit, and a checkpoint taken halfway continues to the same state."""
    import bsglmm_gb300 as bsg
    mask, covar, data, wm = _wm_study(3, shape=(10, 9, 8), N=36)
    states = []
    for mode in ("graph", "single"):
        with bsg.Sampler() as s:
            ds = s.add_dataset(mask, covar, data, 1, wm)
            ch = s.add_chain(ds, seed=5, beta_wm=-0.2)
            s.set_wm_update(ch, True)
            if mode == "graph":
                s.run(4)
                ck = s.checkpoint(ch)
                s.run(4)
            else:
                for _ in range(8):
                    s.run(1)
            states.append((s.beta(ch), s.omega(ch), s.beta_wm(ch)))
    with bsg.Sampler() as s:
        ds = s.add_dataset(mask, covar, data, 1, wm)
        ch = s.add_chain(ds, seed=1)
        s.restore(ch, ck)
        s.run(4)
        states.append((s.beta(ch), s.omega(ch), s.beta_wm(ch)))
    for other in states[1:]:
        assert np.array_equal(states[0][0], other[0])
        assert np.array_equal(states[0][1], other[1])
        assert states[0][2] == other[2]


@pytest.mark.gpu
def test_gpu_wm_update_needs_constant_in_design():
    import bsglmm_gb300 as bsg
    st = synth.small_study(5, P=3, S=1)
    covar = st.covar.copy()
    covar[0] = np.random.default_rng(6).standard_normal(st.N)  # no intercept
    wm = np.ones(st.V, np.float32)
    with bsg.Sampler() as s:
        ds = s.add_dataset(st.mask, covar, st.data, 1, wm)
        ch = s.add_chain(ds, seed=1)
        with pytest.raises(bsg.BsgError, match="sum to 1"):
            s.set_wm_update(ch, True)
        ds2 = s.add_dataset(st.mask, st.covar, st.data, 1, np.zeros(st.V, np.float32))
        ch2 = s.add_chain(ds2, seed=1)
        with pytest.raises(bsg.BsgError, match="nonzero WM"):
            s.set_wm_update(ch2, True)
