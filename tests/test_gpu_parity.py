"""GPU parity tests through the C ABI (libbsglmm_gb300.so).

* Supplied variates: one sweep equals the reference's own CPU update
  (golden fixtures from covar.cpp/cholesky.cpp) bit-exactly in lattice and
  colouring, and within 1e-5 (rtol and atol) in floating state.
* Philox variates: sweeps equal the FP64 oracle chain driven by the same
  counters (common random numbers) within FP32 rounding.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_cases, load_golden, omega_rel_err

pytestmark = pytest.mark.gpu

RTOL = 1e-5   # floating state vs the reference / FP64 oracle
ATOL = 1e-5


@pytest.fixture(scope="module")
def bsg():
    import bsglmm_gb300
    return bsglmm_gb300


def _sampler_for(bsg, g, df_offset=None):
    s = bsg.Sampler()
    wm = g["wm"] if g["wm"].size else None
    ds = s.add_dataset(g["mask"], g["covar"], g["data"], int(g["nsubtypes"]), wm)
    P = g["covar"].shape[0]
    ch = s.add_chain(ds, seed=1234, df_offset=P if df_offset is None else df_offset,
                     beta_wm=float(g["beta_wm"]))
    return s, ds, ch


@pytest.mark.parametrize("name", golden_cases())
def test_lattice_bit_exact(bsg, name):
    g = load_golden(name)
    s, ds, ch = _sampler_for(bsg, g)
    lat = s.lattice(ds)
    assert np.array_equal(lat["idx"], g["idx"])
    assert np.array_equal(lat["idxsc"], g["idxsc"])
    for c in range(2):
        assert np.array_equal(lat["vox"][c], g[f"vox{c}"])
        assert np.array_equal(lat["nbrs"][c], g[f"nbrs{c}"])
    s.close()


@pytest.mark.parametrize("name", golden_cases())
def test_supplied_sweep_matches_reference(bsg, name):
    g = load_golden(name)
    s, ds, ch = _sampler_for(bsg, g)
    s.set_beta(ch, g["beta0"])
    s.set_omega(ch, g["omega0"].astype(np.float64))
    s.sweep_supplied(ch, g["ubits"], g["normals"], g["chi2"], g["wnorm"], form=0)
    b1 = s.beta(ch)
    om1 = s.omega(ch)
    assert np.allclose(b1, g["ref_beta1"], rtol=RTOL, atol=ATOL), \
        np.abs(b1 - g["ref_beta1"]).max()
    ref_om = g["ref_omega1"].astype(np.float64)
    # elementwise relative, entries below 1e-2 max|Omega| against that floor
    worst = omega_rel_err(om1, ref_om)
    print(f"{name}: worst Omega relative error {worst:.3g}")
    assert worst <= RTOL, worst
    prb = s.compute_prb(ch)
    assert np.allclose(prb, g["ref_prb1"], atol=2e-6)
    assert s.sweep_count(ch) == (1, 0)
    s.close()


@pytest.mark.parametrize("name", golden_cases())
def test_supplied_sweep_production_form(bsg, oracle_mod, name):
    """Form 1 (beta = m + G^-T e) against the FP64 oracle's form 1; column
    means against the oracle's."""
    g = load_golden(name)
    s, ds, ch = _sampler_for(bsg, g)
    s.set_beta(ch, g["beta0"])
    s.set_omega(ch, g["omega0"].astype(np.float64))
    s.sweep_supplied(ch, g["ubits"], g["normals"], g["chi2"], g["wnorm"], form=1)
    wm = g["wm"] if g["wm"].size else None
    pb = oracle_mod.Problem(g["mask"], g["covar"], g["data"], int(g["nsubtypes"]), wm)
    ob, oom, _, _, fails, ok = pb.sweep_supplied(
        g["beta0"].astype(np.float64), g["omega0"].astype(np.float64), g["ubits"],
        g["normals"], g["chi2"], g["wnorm"], form=1, beta_wm=float(g["beta_wm"]))
    assert fails == 0 and ok
    b1 = s.beta(ch)
    assert np.allclose(b1, ob, rtol=RTOL, atol=ATOL), np.abs(b1 - ob).max()
    worst = omega_rel_err(s.omega(ch), oom)
    print(f"{name}: worst Omega relative error {worst:.3g}")
    assert worst <= RTOL, worst
    assert np.allclose(s.colmeans(ch), pb.col_means(b1.astype(np.float64)),
                       rtol=RTOL, atol=ATOL)
    s.close()


def _study(seed=0, **kw):
    from bsglmm_gb300 import synth
    return synth.small_study(seed, **kw)


@pytest.mark.parametrize("shape,N,P,S", [((10, 9, 8), 37, 4, 2),
                                         ((12, 12, 12), 130, 3, 1),
                                         ((9, 10, 11), 64, 8, 3)])
def test_philox_sweep_matches_oracle_chain(bsg, oracle_mod, shape, N, P, S):
    """Production sweeps (Philox counters, inversion + tail rejection) equal
    the FP64 oracle chain on the same counters."""
    st = _study(41, shape=shape, N=N, P=P, S=S)
    pb = oracle_mod.Problem(st.mask, st.covar, st.data, S)
    seed = 0x1234_5678_9ABC
    with bsg.Sampler() as s:
        ds = s.add_dataset(st.mask, st.covar, st.data, S)
        ch = s.add_chain(ds, seed=seed)
        s.run(1)
        o = pb.chain(seed, 1)
        assert np.allclose(s.beta(ch), o["beta"], rtol=RTOL, atol=ATOL)
        assert np.allclose(s.omega(ch), o["omega"], rtol=RTOL,
                           atol=ATOL * np.abs(o["omega"]).max())
        s.run(2)
        o = pb.chain(seed, 2, s0=1, spatcoef=o["beta"], omega=o["omega"])
        assert np.allclose(s.beta(ch), o["beta"], rtol=1e-4, atol=1e-4)


def test_extreme_linear_predictor_uses_tail_sampler(bsg, oracle_mod):
    """Voxels whose outcome contradicts |eta| > 5 go through the bounded
    rejection tail; values still equal the oracle's."""
    st = _study(43, shape=(8, 8, 8), N=40, P=2, S=1)
    pb = oracle_mod.Problem(st.mask, st.covar, st.data, 1)
    lat = pb.lattice()
    b0 = np.zeros((2, pb.Vp), np.float32)
    sc = lat["idxsc"][lat["idx"] >= 0]
    b0[0, sc] = np.where(np.arange(pb.V) % 2 == 0, 6.5, -6.5)
    seed = 99
    with bsg.Sampler() as s:
        ds = s.add_dataset(st.mask, st.covar, st.data, 1)
        ch = s.add_chain(ds, seed=seed)
        s.set_beta(ch, b0)
        s.run(1)
        o = pb.chain(seed, 1, spatcoef=b0.astype(np.float64))
        assert o["err"] == 0
        assert np.allclose(s.beta(ch), o["beta"], rtol=1e-4, atol=1e-4)


def test_accumulators_match_oracle(bsg, oracle_mod):
    st = _study(45, shape=(9, 9, 9), N=50, P=3, S=2)
    pb = oracle_mod.Problem(st.mask, st.covar, st.data, 2)
    seed = 777
    with bsg.Sampler() as s:
        ds = s.add_dataset(st.mask, st.covar, st.data, 2)
        ch = s.add_chain(ds, seed=seed, burnin=2, thin=2)
        s.run(9)
        mean, var, prb, nk = s.posterior(ch)
        o = pb.chain(seed, 9, burnin=2, thin=2)
        assert nk == o["nkept"] == 3  # sweeps 4, 6, 8
        assert np.allclose(mean, o["mean"], rtol=1e-4, atol=1e-4)
        assert np.allclose(var, o["var"], rtol=1e-3, atol=1e-4)
        assert np.allclose(prb, o["prb"], atol=1e-4)
        maps = s.maps(ch)
        m = st.mask.astype(bool)
        assert np.allclose(maps["spatCoef"][:, m], mean)
        assert np.all(maps["spatCoef"][:, ~m] == 0)
        assert np.allclose(maps["prb"][:, m], prb)
        st_map = maps["standCoef"][:, m]
        assert np.allclose(st_map, mean / np.sqrt(var))


def test_deterministic_and_graph_equals_plain(bsg):
    st = _study(47, shape=(12, 11, 10), N=70, P=4, S=1)
    outs = []
    for mode in ["graph", "graph", "plain"]:
        with bsg.Sampler() as s:
            ds = s.add_dataset(st.mask, st.covar, st.data, 1)
            ch = s.add_chain(ds, seed=5)
            if mode == "graph":
                s.run(7)
            else:
                s.profile(7)
                s.sync()
            outs.append((s.beta(ch), s.omega(ch)))
    for b, o in outs[1:]:
        assert np.array_equal(b, outs[0][0]) and np.array_equal(o, outs[0][1])


@pytest.mark.parametrize("lpv,threads", [(2, 128), (4, 256), (8, 64), (1, 256)])
def test_tile_shapes_agree(bsg, lpv, threads):
    st = _study(49, shape=(10, 10, 10), N=300, P=5, S=1)
    res = []
    for tune in [(1, 128), (lpv, threads)]:
        with bsg.Sampler() as s:
            ds = s.add_dataset(st.mask, st.covar, st.data, 1)
            ch = s.add_chain(ds, seed=11)
            s.set_tuning(*tune)
            s.run(2)
            res.append(s.beta(ch))
    assert np.allclose(res[0], res[1], rtol=1e-4, atol=1e-4)


def test_batched_chains_equal_single(bsg):
    """Chains of different P and size in one batched launch give the same
    state as each chain run alone."""
    studies = [_study(51, shape=(8, 9, 10), N=40, P=2, S=1),
               _study(52, shape=(11, 9, 7), N=90, P=5, S=2),
               _study(53, shape=(9, 9, 9), N=33, P=3, S=1)]
    with bsg.Sampler() as s:
        ids = []
        for k, st in enumerate(studies):
            ds = s.add_dataset(st.mask, st.covar, st.data, st.nsubtypes)
            ids.append(s.add_chain(ds, seed=100))
        s.run(3)
        batched = [(s.beta(c), s.omega(c)) for c in ids]
    for k, st in enumerate(studies):
        with bsg.Sampler() as s:
            for j in range(k):  # keep chain ids equal: they are Philox inputs
                d = s.add_dataset(studies[j].mask, studies[j].covar,
                                  studies[j].data, studies[j].nsubtypes)
                s.add_chain(d, seed=100)
            ds = s.add_dataset(st.mask, st.covar, st.data, st.nsubtypes)
            c = s.add_chain(ds, seed=100)
            s.run(3)
            assert np.allclose(s.beta(c), batched[k][0], rtol=1e-6, atol=1e-6)


# ------------------------------------------------------------ error paths --
def test_rejects_non_binary_outcomes(bsg):
    st = _study(55)
    data = st.data.copy()
    data[3, 5] = 2
    with bsg.Sampler() as s:
        with pytest.raises(bsg.BsgError) as e:
            s.add_dataset(st.mask, st.covar, data, 1)
        assert e.value.status == 1


def test_rejects_unsupported_sizes(bsg):
    st = _study(56)
    with bsg.Sampler() as s:
        with pytest.raises(bsg.BsgError) as e:
            s.add_dataset(np.zeros_like(st.mask), st.covar, st.data, 1)
        assert e.value.status == 1  # empty mask
        cov9 = np.ones((9, st.N), np.float32)
        with pytest.raises(bsg.BsgError) as e:
            s.add_dataset(st.mask, cov9, st.data, 1)
        assert e.value.status == 8
        with pytest.raises(bsg.BsgError):
            s.run(1)  # no chain yet


def test_nan_state_reported(bsg):
    st = _study(57, shape=(8, 8, 8), N=40, P=2, S=1)
    with bsg.Sampler() as s:
        ds = s.add_dataset(st.mask, st.covar, st.data, 1)
        ch = s.add_chain(ds, seed=1)
        b = s.beta(ch)
        lat = s.lattice(ds)
        b[0, lat["idxsc"][lat["vox"][0][3]]] = np.nan
        s.set_beta(ch, b)
        with pytest.raises(bsg.BsgError) as e:
            s.run(1)
        assert e.value.status == 5  # BSG_ERR_NAN


def test_non_spd_precision_reported(bsg):
    st = _study(58, shape=(8, 8, 8), N=40, P=2, S=1)
    with bsg.Sampler() as s:
        ds = s.add_dataset(st.mask, st.covar, st.data, 1)
        ch = s.add_chain(ds, seed=1)
        s.set_omega(ch, -50.0 * np.eye(2))
        with pytest.raises(bsg.BsgError) as e:
            s.run(1)
        assert e.value.status == 3  # BSG_ERR_NOT_SPD


# ------------------------------------------------- checkpoint / autotune --
def test_checkpoint_resume_is_bit_exact(bsg):
    st = _study(81, shape=(10, 9, 11), N=70, P=4, S=2)
    with bsg.Sampler() as s:
        ds = s.add_dataset(st.mask, st.covar, st.data, 2)
        ch = s.add_chain(ds, seed=4242, burnin=3)
        s.run(6)
        ck = s.checkpoint(ch)
        s.run(5)
        ref = (s.beta(ch), s.omega(ch), s.posterior(ch))
    with bsg.Sampler() as s:  # another context, the chain at another index
        ds0 = s.add_dataset(st.mask, st.covar, st.data, 2)
        s.add_chain(ds0, seed=1)
        ch = s.add_chain(ds0, seed=999)
        s.restore(ch, ck)
        s.run(5)
        assert np.array_equal(s.beta(ch), ref[0])
        assert np.array_equal(s.omega(ch), ref[1])
        m, v, p, nk = s.posterior(ch)
        assert nk == ref[2][3] and np.array_equal(m, ref[2][0])
        assert np.array_equal(p, ref[2][2])


def test_restore_rejects_other_shapes(bsg):
    a = _study(82, shape=(8, 8, 8), N=40, P=3, S=1)
    b = _study(83, shape=(9, 8, 8), N=40, P=3, S=1)
    with bsg.Sampler() as s:
        ca = s.add_chain(s.add_dataset(a.mask, a.covar, a.data, 1), seed=1)
        cb = s.add_chain(s.add_dataset(b.mask, b.covar, b.data, 1), seed=1)
        ck = s.checkpoint(ca)
        with pytest.raises(bsg.BsgError):
            s.restore(cb, ck)
        with pytest.raises(bsg.BsgError):
            s.restore(ca, b"not a checkpoint" * 8)


def test_autotune_restores_state(bsg):
    st = _study(84, shape=(12, 12, 12), N=200, P=5, S=1)
    with bsg.Sampler() as s:
        ch = s.add_chain(s.add_dataset(st.mask, st.covar, st.data, 1), seed=77)
        s.run(2)
        b0, o0, sw0 = s.beta(ch), s.omega(ch), s.sweep_count(ch)
        lpv, thr = s.autotune(2)
        assert (lpv, thr) == s.tuning()
        assert s.step_subjects() in (8, 16)
        assert np.array_equal(s.beta(ch), b0) and np.array_equal(s.omega(ch), o0)
        assert s.sweep_count(ch) == sw0
