"""FP64 chains (bsg_set_precision(..., 64)): the whole sweep in double
precision on the sampler's Philox counters.

- Against the CPU FP64 oracle chain on the same counters: the 20^3 sphere
  study (r = 9, N = 50, P = 3) and a ragged study with two group columns;
  coefficients, Omega and the posterior sums agree to 1e-9 after 30 sweeps
  (both sides are FP64; they differ only in the last bits of the CDF and
  its inverse, CUDA's normcdf/normcdfinv against the oracle's
  erfc / Newton-refined AS 241).
- A graph segment equals single sweeps, and a checkpoint taken mid-way
  continues bit for bit in a new context.
- The FP32 sampler on the same seed tracks it to FP32 rounding.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL64 = 1e-9


def _studies():
    from bsglmm_gb300 import synth
    return [("c0", synth.config0(0)),
            ("ragged", synth.small_study(13, shape=(11, 9, 10), N=37, P=4, S=2))]


@pytest.mark.parametrize("which", [0, 1])
def test_fp64_chain_matches_cpu_fp64_oracle(oracle_mod, which):
    import bsglmm_gb300 as bsg
    name, st = _studies()[which]
    seed, T, burn = 0xF64 + which, 30, 10
    pb = oracle_mod.Problem(st.mask, st.covar, st.data, st.nsubtypes)
    o = pb.chain(seed, T, burnin=burn)
    assert o["err"] == 0
    with bsg.Sampler() as s:
        ds = s.add_dataset(st.mask, st.covar, st.data, st.nsubtypes)
        ch = s.add_chain(ds, seed=seed, burnin=burn)
        s.set_precision(ch, 64)
        s.run(T)
        b64, om = s.beta64(ch), s.omega(ch)
        mean, var, prb, nk = s.posterior(ch)
        b32 = s.beta(ch)
    err = np.abs(b64 - o["beta"]).max()
    print(f"{name}: FP64 GPU vs CPU oracle after {T} sweeps: beta {err:.3g}, "
          f"Omega {np.abs(om - o['omega']).max():.3g}")
    assert nk == o["nkept"] == T - 1 - burn
    assert np.allclose(b64, o["beta"], rtol=TOL64, atol=TOL64)
    assert np.allclose(om, o["omega"], rtol=TOL64, atol=TOL64)
    assert np.allclose(mean, o["mean"], rtol=TOL64, atol=TOL64)
    assert np.allclose(var, o["var"], rtol=1e-7, atol=1e-9)
    assert np.allclose(prb, o["prb"], rtol=TOL64, atol=TOL64)
    assert np.array_equal(b32, b64.astype(np.float32))


def test_fp64_graph_single_sweeps_and_checkpoint():
    import bsglmm_gb300 as bsg
    name, st = _studies()[1]
    out = []
    for mode in ("graph", "single"):
        with bsg.Sampler() as s:
            ds = s.add_dataset(st.mask, st.covar, st.data, st.nsubtypes)
            ch = s.add_chain(ds, seed=77, burnin=3)
            s.set_precision(ch, 64)
            if mode == "graph":
                s.run(6)
                ck = s.checkpoint(ch)
                s.run(6)
            else:
                for _ in range(12):
                    s.run(1)
            out.append((s.beta64(ch), s.omega(ch), s.posterior(ch)[0]))
    with bsg.Sampler() as s:
        ds = s.add_dataset(st.mask, st.covar, st.data, st.nsubtypes)
        ch = s.add_chain(ds, seed=1)
        s.restore(ch, ck)  # carries the FP64 mode and coefficients
        s.run(6)
        out.append((s.beta64(ch), s.omega(ch), s.posterior(ch)[0]))
    for other in out[1:]:
        for a, b in zip(out[0], other):
            assert np.array_equal(a, b)


def test_fp32_chain_tracks_fp64_chain_on_the_same_counters():
    """Common random numbers: the FP32 sampler and the FP64 chain of the
    same seed, run side by side in one context, stay within FP32 rounding
    of each other (the maps after 40 sweeps, 20 kept)."""
    import bsglmm_gb300 as bsg
    name, st = _studies()[0]
    with bsg.Sampler() as s:
        ds = s.add_dataset(st.mask, st.covar, st.data, st.nsubtypes)
        c32 = s.add_chain(ds, seed=5, burnin=20)
        # same key: the counters differ only by the chain id, so give the
        # FP64 chain its own context instead
        s.run(40)
        m32, _, p32, _ = s.posterior(c32)
    with bsg.Sampler() as s:
        ds = s.add_dataset(st.mask, st.covar, st.data, st.nsubtypes)
        c64 = s.add_chain(ds, seed=5, burnin=20)
        s.set_precision(c64, 64)
        s.run(40)
        m64, v64, p64, _ = s.posterior(c64)
    d = np.abs(m32 - m64)
    print(f"FP32 vs FP64 posterior mean: max {d.max():.3g}, sd scale {np.sqrt(v64).mean():.3g}")
    assert np.allclose(m32, m64, rtol=1e-3, atol=1e-3)
    assert np.allclose(p32, p64, atol=1e-3)


def test_fp64_mode_rejects_other_links_and_supplied_sweeps():
    import bsglmm_gb300 as bsg
    name, st = _studies()[1]
    with bsg.Sampler() as s:
        ds = s.add_dataset(st.mask, st.covar, st.data, st.nsubtypes)
        ch = s.add_chain(ds, seed=3)
        s.set_precision(ch, 64)
        with pytest.raises(bsg.BsgError):
            s.set_model(ch, "logistic")
        with pytest.raises(bsg.BsgError):
            s.set_wm_update(ch, True)
        info = s.info(ds)
        N, V, P = info["N"], info["V"], info["P"]
        with pytest.raises(bsg.BsgError):
            s.sweep_supplied(ch, np.zeros((N, V), np.uint32), np.zeros((V, P), np.float32),
                             np.full(P, 10.0), np.zeros(P * (P - 1) // 2), form=1)
        s.set_precision(ch, 32)
        s.run(1)


def test_fp64_chain_matches_cpu_oracle_on_the_brain_study(oracle_mod):
    """The brain-sized study (230,261 voxels, N = 1000, P = 5), two sweeps
    (the second with the first's Omega): the FP64 GPU chain equals the CPU
    FP64 oracle chain to 1e-9."""
    import bsglmm_gb300 as bsg
    from bsglmm_gb300 import synth
    st = synth.config1(seed=1)
    pb = oracle_mod.Problem(st.mask, st.covar, st.data, st.nsubtypes)
    o = pb.chain(0xB64, 2)
    assert o["err"] == 0
    with bsg.Sampler() as s:
        ds = s.add_dataset(st.mask, st.covar, st.data, st.nsubtypes)
        ch = s.add_chain(ds, seed=0xB64)
        s.set_precision(ch, 64)
        s.run(2)
        b64, om = s.beta64(ch), s.omega(ch)
    print(f"brain study, FP64 GPU vs CPU oracle: beta {np.abs(b64 - o['beta']).max():.3g}, "
          f"Omega {np.abs(om - o['omega']).max():.3g}")
    assert np.allclose(b64, o["beta"], rtol=TOL64, atol=TOL64)
    assert np.allclose(om, o["omega"], rtol=TOL64, atol=TOL64)


def test_map_error_study_on_a_small_study():
    """bsglmm_gb300.precision.map_error_vs_fp64 end to end on a small study:
    the FP32 chain on the FP64 chain's counters stays far inside 0.5 MCSE,
    and the independent chain's z-scores look like Monte-Carlo noise."""
    from bsglmm_gb300 import precision
    name, st = _studies()[1]
    r = precision.map_error_vs_fp64(st, seed=4, burnin=50, batches=10, batch=20)
    print(r["beta"], r["prb"])
    assert r["sweeps"] == 250 and r["P"] == st.P
    for what in ("beta", "prb"):
        assert r[what]["same_counters"]["max"] < 0.01
        assert r[what]["same_counters"]["frac_le_0.5"] == 1.0
        z = r[what]["independent_chain_z"]
        assert 0.2 < z["median"] < 2.0 and z["frac_within_4"] > 0.97
