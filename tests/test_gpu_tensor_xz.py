"""The probit colour kernel with X'(Z - b_WM WM) on the tensor cores
(bsg_set_tensor_xz: BF16x3 split product, m16n8k16 MMAs, FP32 accumulation).

The latent and coefficient draws are the SIMT kernel's; only the
contraction's rounding differs (about 2^-16 relative per product), so:
- a sweep equals the FP64 oracle chain within the same 1e-4 tolerance as
  the SIMT kernel, on the N = 2000, P = 8 study and on small studies with a
  ragged subject count (a partial outcome word), partly filled warps and
  P = 1, 3, 4, 8;
- it stays within 1e-4 of the SIMT kernel's sweep;
- graph segments equal single sweeps bit for bit, and a chain batched with
  others equals the same chain alone.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-4


def _sweeps(st, seed, n, tc, extra_chains=0, single=False):
    import bsglmm_gb300 as bsg
    with bsg.Sampler() as s:
        ds = s.add_dataset(st.mask, st.covar, st.data, st.nsubtypes)
        ch = s.add_chain(ds, seed=seed)
        for e in range(extra_chains):
            s.add_chain(ds, seed=seed + 100 + e)
        s.set_tensor_xz(tc)
        if single:
            for _ in range(n):
                s.run(1)
        else:
            s.run(n)
        return s.beta(ch), s.omega(ch)


@pytest.mark.parametrize("shape,N,P,S", [((10, 9, 8), 37, 4, 2), ((12, 12, 12), 130, 3, 1),
                                         ((9, 10, 11), 64, 8, 3), ((8, 7, 9), 45, 1, 1)])
def test_small_studies_match_fp64_oracle(oracle_mod, shape, N, P, S):
    from bsglmm_gb300 import synth
    st = synth.small_study(31, shape=shape, N=N, P=P, S=S)
    pb = oracle_mod.Problem(st.mask, st.covar, st.data, st.nsubtypes)
    o = pb.chain(71, 2)
    b, om = _sweeps(st, 71, 2, True)
    err = np.abs(b - o["beta"]).max()
    print(f"P={P} N={N}: max |beta - oracle| {err:.3g}")
    assert np.allclose(b, o["beta"], rtol=TOL, atol=TOL)
    assert np.allclose(om, o["omega"], rtol=TOL, atol=TOL * np.abs(o["omega"]).max())


def test_precision_study_matches_fp64_oracle_and_simt(oracle_mod):
    from bsglmm_gb300 import synth
    st = synth.config2()
    pb = oracle_mod.Problem(st.mask, st.covar, st.data, st.nsubtypes)
    o = pb.chain(0xC2, 1)
    b_tc, om_tc = _sweeps(st, 0xC2, 1, True)
    b_simt, _ = _sweeps(st, 0xC2, 1, False)
    e_tc = np.abs(b_tc - o["beta"]) / (TOL + TOL * np.abs(o["beta"]))
    e_simt = np.abs(b_simt - o["beta"]) / (TOL + TOL * np.abs(o["beta"]))
    print(f"N=2000 P=8: tensor-core X'Z max {e_tc.max():.3g} of tolerance "
          f"(SIMT {e_simt.max():.3g}); |tc - simt| max {np.abs(b_tc - b_simt).max():.3g}")
    assert np.allclose(b_tc, o["beta"], rtol=TOL, atol=TOL)
    assert np.allclose(b_tc, b_simt, rtol=TOL, atol=TOL)
    assert np.allclose(om_tc, o["omega"], rtol=TOL, atol=TOL * np.abs(o["omega"]).max())


def test_graph_equals_single_sweeps_and_batched_equals_alone():
    from bsglmm_gb300 import synth
    st = synth.small_study(41, shape=(13, 12, 11), N=77, P=5, S=1)
    g = _sweeps(st, 9, 6, True)
    one = _sweeps(st, 9, 6, True, single=True)
    batched = _sweeps(st, 9, 6, True, extra_chains=2)
    for other in (one, batched):
        assert np.array_equal(g[0], other[0]) and np.array_equal(g[1], other[1])
