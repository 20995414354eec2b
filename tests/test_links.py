"""The t/logit links (the reference's MODEL 0 and 2: Z_GPU2 / Phi_GPU /
Spat_Coef, covarGPU.cu:398-513,1430-1563; ProbLogitGPU and its prediction,
covarGPU.cu:1695-1781; the logistic branch of compute_prb_DIC,
covar.cpp:457-465).  CPU: the oracle's pieces against scipy and the
reference's own compute_prb_DIC.  GPU: the scale-mixture chain against the
FP64 oracle chain on the same counters, recovery of a logistic model, the
lesion probabilities and DIC, determinism and checkpoints."""
from __future__ import annotations

import numpy as np
import pytest
from scipy import stats

from bsglmm_gb300 import synth


def _logit_study(seed, shape=(11, 10, 9), N=60, b0=-1.0, b1=0.8):
    """Intercept + one N(0,1) covariate; Y ~ Bernoulli(logistic(b0 + b1 x))
    at every voxel."""
    rng = np.random.default_rng(seed)
    X, Y, Z = shape
    mask = (rng.random((Z, Y, X)) < 0.7).astype(np.uint8)
    V = int(mask.sum())
    covar = np.ones((2, N), np.float32)
    covar[1] = rng.standard_normal(N).astype(np.float32)
    eta = (b0 + b1 * covar[1].astype(np.float64))[:, None] + np.zeros((N, V))
    data = (rng.random((N, V)) < 1.0 / (1.0 + np.exp(-eta))).astype(np.uint8)
    return mask, covar, data


# ------------------------------------------------------------------ CPU --
@pytest.mark.parametrize("alpha", [4.5, 2.0])
def test_mixture_gamma_law(oracle_mod, alpha):
    """Marsaglia-Tsang on the sampler's counters has the Gamma(alpha) law."""
    L = oracle_mod.lib()
    g = np.array([L.orc_mix_gamma(alpha, i, 7, 3, 11, 12, 0) for i in range(6000)])
    assert stats.kstest(g, stats.gamma(alpha).cdf).pvalue > 1e-3


def test_dic_de_logistic_matches_reference(oracle_mod):
    O = oracle_mod
    if not O.REF_KISS.exists():
        pytest.skip("reference build (oracle/_ref) not present")
    st = synth.small_study(21, P=3, S=1)
    pb = O.Problem(st.mask, st.covar, st.data, 1)
    rng = np.random.default_rng(22)
    mean = rng.normal(-0.5, 0.6, (pb.P, pb.V))
    mwm = rng.normal(0, 0.2, pb.V)
    ref = O.RefKiss(pb)
    want = ref.compute_prb_dic(mean, mwm, model=0)
    ref.compute_prb_dic(mean, mwm, model=1)  # leave the reference on probit
    assert pb.dic_de(mean, mwm, model=0) == pytest.approx(want, rel=1e-10)


def test_oracle_mixture_chain_runs(oracle_mod):
    mask, covar, data = _logit_study(23, shape=(6, 5, 5), N=24)
    pb = oracle_mod.Problem(mask, covar, data, 1)
    o = pb.chain(5, 3, model=2)
    assert o["err"] == 0 and np.all(o["phi"] > 0) and np.all(np.isfinite(o["beta"]))
    assert not np.allclose(o["phi"], 1.0)


# ------------------------------------------------------------------ GPU --
@pytest.mark.gpu
@pytest.mark.parametrize("model", [0, 2])
def test_gpu_mixture_chain_matches_oracle(oracle_mod, model):
    import bsglmm_gb300 as bsg
    mask, covar, data = _logit_study(24 + model, shape=(9, 8, 7), N=36)
    pb = oracle_mod.Problem(mask, covar, data, 1)
    seed = 0x5EED_0000 + model
    with bsg.Sampler() as s:
        ds = s.add_dataset(mask, covar, data, 1)
        ch = s.add_chain(ds, seed=seed)
        s.set_model(ch, model)
        s.run(1)
        o = pb.chain(seed, 1, model=model)
        b = s.beta(ch)
        close = np.isclose(b, o["beta"], rtol=1e-4, atol=1e-4).all(axis=0)
        # an FP32 Marsaglia-Tsang decision can fall the other way than the
        # FP64 one: at most a handful of voxels may differ
        assert close.mean() > 0.99
        s.run(2)
        o = pb.chain(seed, 2, s0=1, spatcoef=o["beta"], omega=o["omega"],
                     model=model, phi=o["phi"])
        close = np.isclose(s.beta(ch), o["beta"], rtol=2e-3, atol=2e-3).all(axis=0)
        assert close.mean() > 0.95


@pytest.mark.gpu
def test_gpu_logistic_recovers_coefficients(oracle_mod):
    """Data from logistic(-1 + 0.8 x): with the t_8 scale mixture and
    logit_factor 0.634 the coefficients are 0.634 times the logistic ones,
    and the lesion probability map is logistic(beta_0 / 0.634)."""
    import bsglmm_gb300 as bsg
    mask, covar, data = _logit_study(30, N=120)
    with bsg.Sampler() as s:
        ds = s.add_dataset(mask, covar, data, 1)
        ch = s.add_chain(ds, seed=3, burnin=200)
        s.set_model(ch, "logistic")
        s.run(600)
        s.sync()
        mean, var, prb, nk = s.posterior(ch)
        assert nk == 399
        b = s.beta(ch)
        cp = s.compute_prb(ch)
        pb = oracle_mod.Problem(mask, covar, data, 1)
        lat = pb.lattice()
        q = np.nonzero(lat["idx"] >= 0)[0]
        bc = np.zeros(pb.V)
        bc[lat["idx"][q]] = b[0, lat["idxsc"][q]]
        assert np.allclose(cp[0], 1 / (1 + np.exp(-bc / 0.634)), rtol=1e-5, atol=1e-6)
    assert abs(mean[0].mean() - 0.634 * -1.0) < 0.08, mean[0].mean()
    assert abs(mean[1].mean() - 0.634 * 0.8) < 0.08, mean[1].mean()
    p_true = 1 / (1 + np.exp(1.0))
    assert abs(prb[0].mean() - p_true) < 0.05


@pytest.mark.gpu
def test_gpu_logistic_predictive_and_dic_match_oracle(oracle_mod):
    import bsglmm_gb300 as bsg
    mask, covar, data = _logit_study(31, shape=(9, 8, 7), N=40)
    pb = oracle_mod.Problem(mask, covar, data, 1)
    with bsg.Sampler() as s:
        ds = s.add_dataset(mask, covar, data, 1)
        ch = s.add_chain(ds, seed=8, burnin=2)
        s.set_model(ch, 0)
        s.set_predictive(ch, True)
        s.run(6)
        got = s.predict(ch)
        want = pb.predict(s.beta(ch).astype(np.float64), model=0)
        assert np.allclose(got, want, rtol=1e-5, atol=1e-3)
        mean, _, _, _ = s.posterior(ch)
        dic = s.dic(ch)
    assert dic["DE"] == pytest.approx(pb.dic_de(mean, model=0), rel=1e-5)


@pytest.mark.gpu
def test_gpu_mixture_deterministic_and_checkpointed():
    import bsglmm_gb300 as bsg
    mask, covar, data = _logit_study(32, shape=(9, 8, 7), N=30)
    out = []
    for mode in ("graph", "single", "restored"):
        with bsg.Sampler() as s:
            ds = s.add_dataset(mask, covar, data, 1)
            ch = s.add_chain(ds, seed=9)
            if mode == "restored":
                s.restore(ch, ck)
                s.run(3)
            else:
                s.set_model(ch, "t")
                if mode == "graph":
                    s.run(3)
                    ck = s.checkpoint(ch)
                    s.run(3)
                else:
                    for _ in range(6):
                        s.run(1)
            out.append((s.beta(ch), s.omega(ch)))
    for b, om in out[1:]:
        assert np.array_equal(b, out[0][0]) and np.array_equal(om, out[0][1])


@pytest.mark.gpu
def test_gpu_mixture_combinations_rejected():
    import bsglmm_gb300 as bsg
    st = synth.small_study(33, P=3, S=1)
    wm = np.random.default_rng(34).random(st.V).astype(np.float32)
    with bsg.Sampler() as s:
        ds = s.add_dataset(st.mask, st.covar, st.data, 1, wm)
        ch = s.add_chain(ds, seed=1)
        s.set_model(ch, 0)
        with pytest.raises(bsg.BsgError, match="probit only"):
            s.set_wm_update(ch, True)
        ch2 = s.add_chain(ds, seed=2)
        s.set_wm_update(ch2, True)
        with pytest.raises(bsg.BsgError, match="probit only"):
            s.set_model(ch2, 2)
        with pytest.raises(bsg.BsgError):
            s.set_model(ch, 5)
