"""The CUDA sampler against the FP64 oracle chain (the C restatement of
covar.cpp:121-325 driven by the same Philox counters) at the benchmark's
larger study sizes, where the other GPU tests only compare the sampler with
itself:

- the precision study: the brain mask (230,261 voxels) with N = 2000 and
  P = 8, two sweeps (the second one draws with the Omega of the first);
- the largest study: 182x218x182 grid, 1.5M voxels, N = 500, P = 6, one
  sweep of the second of two chains batched in one context;
- a batch of replicate studies of uneven size, N and P (cube side 32-64,
  N 40-400, P 2-6) in one context, two sweeps, each chain against its own
  oracle chain.

Common random numbers make an FP32 sweep and the FP64 chain agree to FP32
rounding: coefficients within 1e-4 (absolute and relative), Omega within
1e-4 elementwise (entries below 1% of max|Omega| against that floor).  The
oracle splits each colour over the host's cores."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import omega_rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-4


def _check(name, beta, omega, o):
    err = np.abs(beta - o["beta"]) / (TOL + TOL * np.abs(o["beta"]))
    worst = omega_rel_err(omega, o["omega"])
    print(f"{name}: beta max {err.max():.3g} of tolerance (median "
          f"{np.median(err):.3g}); Omega worst relative {worst:.3g}")
    assert np.isfinite(beta).all()
    assert np.allclose(beta, o["beta"], rtol=TOL, atol=TOL), name
    assert worst <= TOL, (name, worst)


def test_precision_study_two_sweeps_match_fp64_oracle(oracle_mod):
    import bsglmm_gb300 as bsg
    from bsglmm_gb300 import synth
    st = synth.config2()
    seed = 0xC2C2
    pb = oracle_mod.Problem(st.mask, st.covar, st.data, st.nsubtypes)
    o = pb.chain(seed, 2)
    assert o["err"] == 0
    with bsg.Sampler() as s:
        ds = s.add_dataset(st.mask, st.covar, st.data, st.nsubtypes)
        ch = s.add_chain(ds, seed=seed)
        s.run(2)
        _check("N=2000 P=8", s.beta(ch), s.omega(ch), o)


def test_largest_study_batched_chain_matches_fp64_oracle(oracle_mod):
    import bsglmm_gb300 as bsg
    from bsglmm_gb300 import synth
    st = synth.config4()
    seed = 0xC4
    pb = oracle_mod.Problem(st.mask, st.covar, st.data, st.nsubtypes)
    o = pb.chain(seed + 1, 1, chain_id=1)  # the second chain of the context
    assert o["err"] == 0
    with bsg.Sampler() as s:
        ds = s.add_dataset(st.mask, st.covar, st.data, st.nsubtypes)
        s.add_chain(ds, seed=seed)
        ch = s.add_chain(ds, seed=seed + 1)
        assert ch == 1
        s.run(1)
        _check("1.5M voxels N=500 P=6", s.beta(ch), s.omega(ch), o)


def test_uneven_replicate_batch_each_chain_matches_its_oracle(oracle_mod):
    import bsglmm_gb300 as bsg
    from bsglmm_gb300 import synth
    studies = synth.config3()
    # one study of every P, the largest and the smallest
    pick = {}
    for k, st in enumerate(studies):
        pick.setdefault(st.P, k)
    sizes = [st.V * st.N for st in studies]
    pick = sorted(set(pick.values()) | {int(np.argmax(sizes)), int(np.argmin(sizes))})
    with bsg.Sampler() as s:
        chains = []
        for k in pick:
            st = studies[k]
            ds = s.add_dataset(st.mask, st.covar, st.data, st.nsubtypes)
            chains.append((k, s.add_chain(ds, seed=700 + k)))
        s.run(2)
        for k, ch in chains:
            st = studies[k]
            pb = oracle_mod.Problem(st.mask, st.covar, st.data, st.nsubtypes)
            o = pb.chain(700 + k, 2, chain_id=ch)
            assert o["err"] == 0
            _check(f"study {k} (side {st.mask.shape[0]}, N={st.N}, P={st.P})",
                   s.beta(ch), s.omega(ch), o)
