"""The sampler at the benchmark's full size: the brain-sized study of the
bench (91x109x91 grid, ellipsoid mask of 230,261 voxels, N = 1000, P = 5).

- One sweep from the same seed equals the FP64 oracle chain (the oracle takes
  about half a minute for it): every voxel's coefficients and the Omega draw.
- Size-independent properties over several sweeps: an 8-sweep graph segment
  equals 8 single sweeps bit for bit, a checkpoint taken halfway continues
  to the same state in a new context, the posterior sums equal the mean and
  variance of the recorded coefficient maps, and the column means equal the
  mean of the coefficients over the mask."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def brain():
    from bsglmm_gb300 import synth
    return synth.config1(seed=1)


def _cols(s, ds):
    lat = s.lattice(ds)
    inmask = lat["idx"] >= 0
    return lat["idxsc"][inmask][np.argsort(lat["idx"][inmask])]


def test_brain_sweep_matches_fp64_oracle(brain, oracle_mod):
    import bsglmm_gb300 as bsg
    seed = 0xB5A1
    pb = oracle_mod.Problem(brain.mask, brain.covar, brain.data, brain.nsubtypes)
    o = pb.chain(seed, 1)
    with bsg.Sampler() as s:
        ds = s.add_dataset(brain.mask, brain.covar, brain.data, brain.nsubtypes)
        ch = s.add_chain(ds, seed=seed)
        s.run(1)
        beta, omega = s.beta(ch), s.omega(ch)
    err = np.abs(beta - o["beta"]) / (1e-4 + 1e-4 * np.abs(o["beta"]))
    print(f"beta: max {err.max():.3g} of tolerance, median {np.median(err):.3g}")
    assert np.isfinite(beta).all()
    assert np.allclose(beta, o["beta"], rtol=1e-4, atol=1e-4)
    assert np.allclose(omega, o["omega"], rtol=1e-4, atol=1e-4 * np.abs(o["omega"]).max())


def test_brain_graph_segment_single_sweeps_and_checkpoint(brain):
    import bsglmm_gb300 as bsg
    states = []
    for mode in ("graph", "single"):
        with bsg.Sampler() as s:
            ds = s.add_dataset(brain.mask, brain.covar, brain.data, brain.nsubtypes)
            ch = s.add_chain(ds, seed=17, burnin=2, thin=1)
            if mode == "graph":
                s.run(4)
                ck = s.checkpoint(ch)
                s.run(4)
            else:
                for _ in range(8):
                    s.run(1)
            states.append((s.beta(ch), s.omega(ch), s.posterior(ch)[0]))
    with bsg.Sampler() as s:
        ds = s.add_dataset(brain.mask, brain.covar, brain.data, brain.nsubtypes)
        ch = s.add_chain(ds, seed=1)
        s.restore(ch, ck)
        s.run(4)
        states.append((s.beta(ch), s.omega(ch), s.posterior(ch)[0]))
    for other in states[1:]:
        for a, b in zip(states[0], other):
            assert np.array_equal(a, b)


def test_brain_posterior_sums_and_column_means(brain):
    import bsglmm_gb300 as bsg
    with bsg.Sampler() as s:
        ds = s.add_dataset(brain.mask, brain.covar, brain.data, brain.nsubtypes)
        ch = s.add_chain(ds, seed=23, burnin=2, thin=1)  # sweeps 3.. kept
        cols = _cols(s, ds)
        s.run(3)
        trace = []
        for _ in range(5):
            s.run(1)
            b = s.beta(ch)[:, cols].astype(np.float64)
            trace.append(b)
            cm = s.colmeans(ch)
            assert np.allclose(cm, b.mean(axis=1), rtol=1e-5, atol=1e-6)
        mean, var, _, nk = s.posterior(ch)
    tr = np.stack(trace)
    assert nk == 5
    assert np.allclose(mean, tr.mean(0), rtol=1e-12, atol=1e-12)
    assert np.allclose(var, tr.var(0, ddof=1), rtol=1e-6, atol=1e-9)
    assert var.min() > -1e-9


def test_largest_study_batched_chain_equals_lone_chain():
    """The 182x218x182 study (1.5M voxels, N = 500, P = 6): a chain that shares
    its launches with a second chain equals the same chain run alone, bit
    for bit, over a 3-sweep graph segment against 3 single sweeps."""
    import bsglmm_gb300 as bsg
    from bsglmm_gb300 import synth
    big = synth.config4()
    with bsg.Sampler() as s:
        ds = s.add_dataset(big.mask, big.covar, big.data, big.nsubtypes)
        c0 = s.add_chain(ds, seed=3)
        c1 = s.add_chain(ds, seed=4)
        s.run(3)
        b0, o0 = s.beta(c0), s.omega(c0)
        b1 = s.beta(c1)
    with bsg.Sampler() as s:
        ds = s.add_dataset(big.mask, big.covar, big.data, big.nsubtypes)
        ch = s.add_chain(ds, seed=3)
        for _ in range(3):
            s.run(1)
        b, o = s.beta(ch), s.omega(ch)
    assert np.isfinite(b0).all() and not np.array_equal(b0, b1)
    assert np.array_equal(b0, b)
    assert np.array_equal(o0, o)


def test_precision_form_graph_segment_and_posterior_sums():
    """The N = 2000, P = 8 study on the brain mask (two 1024-subject chunks,
    the two-block P = 8 kernel): a 4-sweep graph segment equals 4 single
    sweeps, and the posterior sums equal the recorded maps of the kept
    sweeps 1-3."""
    import bsglmm_gb300 as bsg
    from bsglmm_gb300 import synth
    st = synth.config2()
    out = []
    for mode in ("graph", "single"):
        with bsg.Sampler() as s:
            ds = s.add_dataset(st.mask, st.covar, st.data, st.nsubtypes)
            ch = s.add_chain(ds, seed=29, burnin=0, thin=1)
            cols = _cols(s, ds)
            trace = []
            if mode == "graph":
                s.run(4)
            else:
                for _ in range(4):
                    s.run(1)
                    trace.append(s.beta(ch)[:, cols].astype(np.float64))
            out.append((s.beta(ch), s.omega(ch)))
            mean, var, _, nk = s.posterior(ch)
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    tr = np.stack(trace[1:])  # sweep 0 is not kept (kept: sweep > burnin)
    assert nk == 3
    assert np.allclose(mean, tr.mean(0), rtol=1e-12, atol=1e-12)
    assert np.allclose(var, tr.var(0, ddof=1), rtol=1e-6, atol=1e-9)
