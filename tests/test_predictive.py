"""DIC / Qhat predictive pass (compute_predictGPU, covarGPU.cu:1783-1957;
compute_prb_DIC, covar.cpp:442-486; mcmc.cpp:717-786, 966-975).

CPU: the oracle's restatement pinned against the reference's own
compute_prb_DIC and a loop restatement of the GPU pass.  GPU: the kernel
against the oracle on the same coefficients, and the in-graph ED / Qhat
accumulation against the oracle replaying the chain's kept sweeps."""
from __future__ import annotations

import numpy as np
import pytest

from bsglmm_gb300 import synth


def _ref_kiss_available(O):
    return O.REF_KISS.exists()


def _indicator_study(seed, shape=(9, 8, 7), N=29, S=2, extra=2, wm=False):
    """Group indicator columns (every subject in one group) + covariates."""
    rng = np.random.default_rng(seed)
    X, Y, Z = shape
    mask = (rng.random((Z, Y, X)) < 0.55).astype(np.uint8)
    V = int(mask.sum())
    grp = rng.integers(0, S, N)
    P = S + extra
    covar = np.zeros((P, N), np.float32)
    for g in range(S):
        covar[g] = grp == g
    covar[S:] = rng.standard_normal((extra, N)).astype(np.float32)
    beta = rng.normal(0, 0.6, (P, V)).astype(np.float32)
    beta[:S] -= 1.0
    eta = covar.T @ beta
    data = (rng.random((N, V)) < 0.5 * (1 + np.tanh(eta))).astype(np.uint8)
    w = rng.random(V).astype(np.float32) if wm else None
    return mask, covar, data, S, w


def _beta_grid(pb, rng, scale=0.7):
    b = np.zeros((pb.P, pb.Vp))
    lat = pb.lattice()
    sc = lat["idxsc"][lat["idx"] >= 0]
    b[:, sc] = rng.normal(-0.5, scale, (pb.P, sc.size))
    return b


def _compact(pb, spatcoef):
    lat = pb.lattice()
    q = np.nonzero(lat["idx"] >= 0)[0]
    out = np.zeros((pb.P, pb.V))
    out[:, lat["idx"][q]] = np.asarray(spatcoef)[:, lat["idxsc"][q]]
    return out


# ------------------------------------------------------------------ CPU --
def test_loglik_is_log_of_as_probability(oracle_mod):
    L = oracle_mod.lib()
    for eta in np.linspace(-6, 6, 97):
        p = L.orc_prob_sdnorm(eta)
        assert L.orc_loglik_as(eta, 1) == pytest.approx(np.log(p), rel=1e-12, abs=1e-14)
        assert L.orc_loglik_as(eta, 0) == pytest.approx(np.log1p(-p), rel=1e-9, abs=1e-14)
    # deep tail: the observed side's probability stays finite and exact
    assert L.orc_loglik_as(-30.0, 1) == pytest.approx(-30.0 ** 2 / 2 + np.log(
        0.39894228 / (1 + 0.2316419 * 30)), rel=0.05)


def test_predict_matches_loop_restatement(oracle_mod):
    mask, covar, data, S, wm = _indicator_study(3, wm=True)
    pb = oracle_mod.Problem(mask, covar, data, S, wm)
    rng = np.random.default_rng(4)
    b = _beta_grid(pb, rng)
    got = pb.predict(b, beta_wm=0.3)
    L = oracle_mod.lib()
    bc = _compact(pb, b)
    want = np.zeros((pb.N, S))
    for i in range(pb.N):
        rest = 0.3 * wm.astype(np.float64) + (bc[S:] * covar[S:, i:i + 1].astype(np.float64)).sum(0)
        for g in range(S):
            eta = bc[g] + rest
            want[i, g] = sum(L.orc_loglik_as(float(e), int(y)) for e, y in zip(eta, data[i]))
    assert np.allclose(got, want, rtol=1e-12, atol=1e-9)


def test_predict_own_group_sums_to_de(oracle_mod):
    """With indicator groups, the own-group prediction at beta is the
    deviance term of compute_prb_DIC at mean = beta (up to its float eta)."""
    mask, covar, data, S, _ = _indicator_study(5)
    pb = oracle_mod.Problem(mask, covar, data, S)
    b = _beta_grid(pb, np.random.default_rng(6), scale=0.3)
    # the reference's 1 - x loses digits beyond |eta| = 5 (and gives log(DBL_MIN)
    # beyond 8.3); the two forms agree where it does not
    assert np.abs(covar.T.astype(np.float64) @ _compact(pb, b)).max() < 6
    mp = pb.predict(b)
    sub = np.argmax(covar[:S] != 0, axis=0)
    ed_like = mp[np.arange(pb.N), sub].sum()
    de = pb.dic_de(_compact(pb, b))
    assert -2 * ed_like == pytest.approx(de, rel=1e-6)


@pytest.mark.parametrize("wm", [False, True])
def test_dic_de_matches_reference(oracle_mod, wm):
    """orc_dic_de against the reference's own compute_prb_DIC
    (covar.cpp:442-486) compiled from its source."""
    O = oracle_mod
    if not _ref_kiss_available(O):
        pytest.skip("reference build (oracle/_ref) not present")
    st = synth.small_study(11, P=4, S=2)
    pb = O.Problem(st.mask, st.covar, st.data, 2)
    rng = np.random.default_rng(12)
    mean = rng.normal(-0.6, 0.5, (pb.P, pb.V))
    mwm = rng.normal(0, 0.2, pb.V) if wm else None
    ref = O.RefKiss(pb)
    want = ref.compute_prb_dic(mean, mwm)
    got = pb.dic_de(mean, mwm)
    assert got == pytest.approx(want, rel=1e-10)


def test_qhat_update_restatement():
    """The host logic of compute_predictGPU (covarGPU.cu:1921-1953): the
    first kept sweep sets column 0 and log-adds the others onto 0."""
    from oracle import qhat_update
    q = np.zeros((2, 3))
    m1 = np.array([[-5.0, -7.0, -4.0], [-3.0, -2.0, -9.0]])
    sub = np.array([0, 1])
    qhat_update(q, m1, sub, first=True)
    d = m1 - m1[np.arange(2), sub][:, None]
    assert q[0, 0] == d[0, 0] and q[1, 0] == d[1, 0]
    assert np.allclose(q[:, 1:], np.logaddexp(0.0, d[:, 1:]))
    q0 = q.copy()
    qhat_update(q, m1, sub, first=False)
    assert np.allclose(q, np.logaddexp(q0, d))


# ------------------------------------------------------------------ GPU --
@pytest.mark.gpu
@pytest.mark.parametrize("P,S,wm", [(4, 2, True), (3, 1, False), (8, 3, False), (1, 1, False), (6, 6, True)])
def test_gpu_predict_matches_oracle(oracle_mod, P, S, wm):
    import bsglmm_gb300 as bsg
    mask, covar, data, S, w = _indicator_study(20 + P, N=45, S=S, extra=P - S, wm=wm)
    pb = oracle_mod.Problem(mask, covar, data, S, w)
    with bsg.Sampler() as s:
        ds = s.add_dataset(mask, covar, data, S, w)
        ch = s.add_chain(ds, seed=77, beta_wm=0.25 if wm else 0.0)
        s.run(3)
        b = s.beta(ch)
        got = s.predict(ch)
    want = pb.predict(b.astype(np.float64), beta_wm=0.25 if wm else 0.0)
    assert got.shape == (pb.N, S)
    assert np.allclose(got, want, rtol=1e-5, atol=1e-3)


@pytest.mark.gpu
def test_gpu_predictive_accumulation_matches_oracle_replay(oracle_mod):
    """ED and Qhat accumulated inside the sweep graph over the kept sweeps
    equal the oracle replaying the same chain sweep by sweep; DE and DIC
    from the posterior means equal the oracle's."""
    import bsglmm_gb300 as bsg
    from oracle import qhat_update
    mask, covar, data, S, _ = _indicator_study(31, N=40, S=3, extra=1)
    pb = oracle_mod.Problem(mask, covar, data, S)
    sub = np.argmax(covar[:S] != 0, axis=0)
    burnin, thin, nsw = 3, 2, 12
    with bsg.Sampler() as s:
        ds = s.add_dataset(mask, covar, data, S)
        ch = s.add_chain(ds, seed=2024, burnin=burnin, thin=thin)
        s.set_predictive(ch, True)
        q = np.zeros((pb.N, S))
        ed = 0.0
        nk = 0
        for sweep in range(nsw):
            s.run(1)
            if sweep > burnin and sweep % thin == 0:
                mp = pb.predict(s.beta(ch).astype(np.float64))
                ed += mp[np.arange(pb.N), sub].sum()
                qhat_update(q, mp, sub, first=nk == 0)
                nk += 1
        gq, ged, gn = s.predictive(ch)
        mean, var, prb, nkept = s.posterior(ch)
        dic = s.dic(ch)
    # the same chain as one graph segment
    with bsg.Sampler() as s:
        ds = s.add_dataset(mask, covar, data, S)
        ch = s.add_chain(ds, seed=2024, burnin=burnin, thin=thin)
        s.set_predictive(ch, True)
        s.run(nsw)
        gq2, ged2, gn2 = s.predictive(ch)
    assert gn == nk == nkept and gn2 == nk
    assert ged == pytest.approx(ed, rel=1e-5)
    assert np.allclose(gq, q, rtol=1e-5, atol=1e-3)
    assert np.array_equal(gq2, gq) and ged2 == ged
    de = pb.dic_de(mean)
    ED = -2.0 * ged / gn
    assert dic["DE"] == pytest.approx(de, rel=1e-5)
    assert dic["ED"] == pytest.approx(ED, rel=1e-12)
    assert dic["PD"] == pytest.approx(dic["ED"] - dic["DE"], rel=1e-12)
    assert dic["DIC"] == pytest.approx(dic["DE"] + 2 * dic["PD"], rel=1e-12)


@pytest.mark.gpu
def test_gpu_predictive_off_costs_nothing_and_resets(oracle_mod):
    import bsglmm_gb300 as bsg
    mask, covar, data, S, _ = _indicator_study(41, N=33, S=2, extra=1)
    with bsg.Sampler() as s:
        ds = s.add_dataset(mask, covar, data, S)
        ch = s.add_chain(ds, seed=5)
        base = s.launches_per_sweep()
        s.set_predictive(ch, True)
        assert s.launches_per_sweep() == base + 2
        s.run(4)
        assert s.predictive(ch)[2] == 3  # sweeps 1..3 (kept iff sweep > burnin)
        s.reset_accumulators(ch)
        q, ed, n = s.predictive(ch)
        assert n == 0 and ed == 0.0 and not q.any()
        s.set_predictive(ch, False)
        assert s.launches_per_sweep() == base
        s.run(2)
        assert s.predictive(ch)[2] == 0


@pytest.mark.gpu
def test_gpu_predictive_state_in_checkpoint():
    """Qhat, the ED sum and the pass's on/off switch travel in checkpoints:
    a restored chain continues to the same values bit-exactly."""
    import bsglmm_gb300 as bsg
    mask, covar, data, S, _ = _indicator_study(43, N=30, S=2, extra=1)
    with bsg.Sampler() as s:
        ds = s.add_dataset(mask, covar, data, S)
        ch = s.add_chain(ds, seed=9)
        s.set_predictive(ch, True)
        s.run(5)
        ck = s.checkpoint(ch)
        s.run(4)
        want = s.predictive(ch)
    with bsg.Sampler() as s:
        ds = s.add_dataset(mask, covar, data, S)
        ch = s.add_chain(ds, seed=1)
        s.restore(ch, ck)
        s.run(4)
        got = s.predictive(ch)
    assert want[2] == 8 and got[2] == 8
    assert np.array_equal(got[0], want[0]) and got[1] == want[1]
