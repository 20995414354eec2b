"""Edge shapes of the colour kernels against the FP64 oracle chain on the
same counters: more subjects than one shared-memory chunk (1024) with a
partial last outcome word, a single subject, single-voxel masks (one colour
empty), and several P at once in one context."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = ATOL = 1e-4


def _study(seed, shape, N, P, S=1, fill=0.6, mask=None):
    rng = np.random.default_rng(seed)
    X, Y, Z = shape
    if mask is None:
        mask = (rng.random((Z, Y, X)) < fill).astype(np.uint8)
    V = int(mask.sum())
    covar = np.ones((P, N), np.float32)
    if P > 1:
        covar[1:] = rng.standard_normal((P - 1, N)).astype(np.float32)
    eta = rng.normal(-0.5, 0.7, (N, V))
    data = (rng.standard_normal((N, V)) < eta).astype(np.uint8)
    return mask, covar, data, S


def _compare(oracle_mod, mask, covar, data, S, seed, sweeps=2):
    import bsglmm_gb300 as bsg
    pb = oracle_mod.Problem(mask, covar, data, S)
    with bsg.Sampler() as s:
        ds = s.add_dataset(mask, covar, data, S)
        ch = s.add_chain(ds, seed=seed)
        s.run(1)
        o = pb.chain(seed, 1)
        assert np.allclose(s.beta(ch), o["beta"], rtol=RTOL, atol=ATOL)
        assert np.allclose(s.omega(ch), o["omega"], rtol=RTOL,
                           atol=ATOL * np.abs(o["omega"]).max())
        if sweeps > 1:
            s.run(sweeps - 1)
            o = pb.chain(seed, sweeps - 1, s0=1, spatcoef=o["beta"], omega=o["omega"])
            assert np.allclose(s.beta(ch), o["beta"], rtol=1e-3, atol=1e-3)
        s.sync()


@pytest.mark.parametrize("N", [600, 1025, 2100])
def test_subjects_across_chunks_and_partial_word(oracle_mod, N):
    """600 (one chunk, the last word 24 subjects), 1025 = 1024 + 1 and
    2100 = 2 x 1024 + 52: one to three shared-memory chunks, partial last
    outcome words."""
    mask, covar, data, S = _study(3, (6, 6, 5), N, 3)
    _compare(oracle_mod, mask, covar, data, S, seed=0xC0FFEE)


def test_single_subject(oracle_mod):
    mask, covar, data, S = _study(4, (7, 6, 5), 1, 1)
    _compare(oracle_mod, mask, covar, data, S, seed=77)


@pytest.mark.parametrize("pos", [(0, 0, 0), (0, 0, 1)])
def test_single_voxel_mask(oracle_mod, pos):
    """One in-mask voxel: only one colour has voxels (the other colour's
    kernel has no work; the colour-1 kernel still draws Omega)."""
    mask = np.zeros((4, 4, 4), np.uint8)
    mask[pos] = 1
    _, covar, data, S = _study(5, (4, 4, 4), 20, 2, mask=mask)
    _compare(oracle_mod, mask, covar, data, S, seed=91, sweeps=3)


def test_mixed_p_in_one_context(oracle_mod):
    """Chains of P = 1, 4 and 8 in one context run as three launch groups on
    parallel graph branches; each equals its own oracle chain."""
    import bsglmm_gb300 as bsg
    studies = [_study(10 + P, (6, 5, 5), 40 + P, P) for P in (1, 4, 8)]
    seeds = [5, 6, 7]
    with bsg.Sampler() as s:
        chs = []
        for (mask, covar, data, S), seed in zip(studies, seeds):
            ds = s.add_dataset(mask, covar, data, S)
            chs.append(s.add_chain(ds, seed=seed))
        s.run(1)
        for ch, (mask, covar, data, S), seed in zip(chs, studies, seeds):
            o = oracle_mod.Problem(mask, covar, data, S).chain(seed, 1, chain_id=ch)
            assert np.allclose(s.beta(ch), o["beta"], rtol=RTOL, atol=ATOL)


def test_mcmc_convenience_equals_sampler():
    """bsglmm_gb300.mcmc() with the WM update and the DIC pass equals the
    same chain driven through Sampler."""
    import bsglmm_gb300 as bsg
    mask, covar, data, S = _study(21, (7, 6, 6), 30, 3)
    V = int(mask.sum())
    wm = np.random.default_rng(22).random(V).astype(np.float32)
    out = bsg.mcmc(mask, covar, data, ntypes=1, maxiter=40, burnin=10, seed=9, wm=wm,
                   wm_update=True, predictive=True)
    with bsg.Sampler() as s:
        ds = s.add_dataset(mask, covar, data, 1, wm)
        ch = s.add_chain(ds, seed=9, burnin=10, thin=bsg.save_iter_rule(40, 10))
        s.set_wm_update(ch, True)
        s.set_predictive(ch, True)
        s.run(41)
        maps = s.maps(ch)
        dic = s.dic(ch)
        cur, mean = s.beta_wm(ch)
    assert out["TOTSAV"] == 1
    assert np.array_equal(out["spatCoef"], maps["spatCoef"])
    assert out["DIC"] == dic and out["beta_WM"] == cur
    assert np.array_equal(out["bWM"][mask.astype(bool)], mean * wm.astype(np.float64))


def test_reset_accumulators_is_ordered_with_the_sweeps():
    """bsg_reset_accumulators clears the running sums on the context stream:
    with four chains of a mid-sized study, the posterior after a reset and
    six single sweeps is exactly the mean and sample variance of the six
    recorded coefficient maps (a clear that raced the following sweeps would
    leave stale sums and negative variances)."""
    import bsglmm_gb300 as bsg
    mask, covar, data, S = _study(31, (48, 44, 40), 128, 3)
    with bsg.Sampler() as s:
        ds = s.add_dataset(mask, covar, data, S)
        chs = [s.add_chain(ds, seed=100 + k, burnin=0, thin=1) for k in range(4)]
        lat = s.lattice(ds)
        inmask = lat["idx"] >= 0
        cols = lat["idxsc"][inmask][np.argsort(lat["idx"][inmask])]
        s.run(5)
        for ch in chs:
            s.reset_accumulators(ch)
        trace = {ch: [] for ch in chs}
        for _ in range(6):
            s.run(1)
            for ch in chs:
                trace[ch].append(s.beta(ch)[:, cols].astype(np.float64))
        for ch in chs:
            mean, var, _, nk = s.posterior(ch)
            tr = np.stack(trace[ch])
            assert nk == 6
            assert np.allclose(mean, tr.mean(0), rtol=1e-12, atol=1e-12)
            assert np.allclose(var, tr.var(0, ddof=1), rtol=1e-6, atol=1e-9)
            assert var.min() > -1e-9


def test_page_locked_host_buffers():
    """The accessors take page-locked host buffers as well as pageable ones:
    an upload from a page-locked buffer that the caller overwrites right
    after the call, and a download into one, read the values of the call."""
    torch = pytest.importorskip("torch")
    import bsglmm_gb300 as bsg
    from bsglmm_gb300.sampler import _ptr
    mask, covar, data, S = _study(41, (8, 7, 6), 40, 3)
    with bsg.Sampler() as s:
        ds = s.add_dataset(mask, covar, data, S)
        ch = s.add_chain(ds, seed=3)
        P = 3
        pin_in = torch.empty(P * P, dtype=torch.float64, pin_memory=True).numpy()
        pin_out = torch.empty(P * P, dtype=torch.float64, pin_memory=True).numpy()
        target = np.array([[2.0, 0.3, 0.1], [0.3, 1.5, 0.2], [0.1, 0.2, 1.2]])
        pin_in[:] = target.ravel()
        assert s._L.bsg_set_omega(s._h, ch, _ptr(pin_in)) == 0
        pin_in[:] = -7.0  # the caller reuses its buffer at once
        assert s._L.bsg_get_omega(s._h, ch, _ptr(pin_out)) == 0
        assert np.array_equal(pin_out.reshape(P, P), target)
        s.run(2, sync=False)
        assert s._L.bsg_get_omega(s._h, ch, _ptr(pin_out)) == 0
        assert np.array_equal(pin_out.reshape(P, P), s.omega(ch))
        assert not np.array_equal(pin_out.reshape(P, P), target)
