"""CPU tests of the oracle: Philox known answers, the variate maps, and the
FP64 restatement pinned against the reference's own update code (golden
fixtures from oracle/_ref, and the live reference build where present)."""
from __future__ import annotations

import numpy as np
import pytest
from scipy import special, stats

from conftest import golden_cases, load_golden, omega_rel_err

# Published Philox-4x32-10 known-answer vectors (Random123 KAT set).
PHILOX_KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2,
     (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,out", PHILOX_KAT)
def test_philox_kat(oracle_mod, ctr, key, out):
    assert tuple(int(x) for x in oracle_mod.philox(ctr, key)) == out


def test_ndtri_matches_scipy(oracle_mod):
    L = oracle_mod.lib()
    ps = np.concatenate([np.logspace(-300, -1, 300), np.linspace(0.01, 0.99, 300),
                         1 - np.logspace(-15, -1, 60)])
    got = np.array([L.orc_ndtri(p) for p in ps])
    ref = special.ndtri(ps)
    assert np.max(np.abs(got - ref) / np.maximum(1, np.abs(ref))) < 1e-13


def test_normal_from_bits_symmetric_and_exact_tails(oracle_mod):
    L = oracle_mod.lib()
    for k in [0, 1, 12345, 2**31 - 1]:
        a = L.orc_normal_from_bits(k)
        b = L.orc_normal_from_bits(0xFFFFFFFF - k)
        assert a == -b
    assert L.orc_normal_from_bits(0) == pytest.approx(special.ndtri(0.5 / 2**32), rel=1e-14)


@pytest.mark.parametrize("a", [-3.0, -0.5, 0.0, 0.7, 2.5, 4.9])
def test_tn_inverse_distribution(oracle_mod, a):
    """The canonical inversion draw is exactly N(0,1) truncated to (a, inf)."""
    L = oracle_mod.lib()
    ks = oracle_mod.philox_block(7, 0, 1, 11, 22, 2500)
    x = np.array([L.orc_tn_lower_inv(a, int(k)) for k in ks])
    assert np.all(x > a)
    d = stats.truncnorm(a, np.inf)
    assert stats.kstest(x, d.cdf).pvalue > 1e-3


@pytest.mark.parametrize("a", [5.0, 7.5, 12.0])
def test_tn_tail_rejection_distribution(oracle_mod, a):
    import ctypes as C
    L = oracle_mod.lib()
    ks = oracle_mod.philox_block(9, 0, 2, 5, 6, 4 * 4000)
    out = []
    for t in range(4000):
        kp = np.ascontiguousarray(ks[8 * t % len(ks): 8 * t % len(ks) + 32], dtype=np.uint32)
        if kp.size < 32:
            continue
        x = C.c_double()
        n = L.orc_tn_lower_tail(a, kp.ctypes.data_as(C.c_void_p), 16, C.byref(x))
        assert n > 0
        out.append(x.value)
    out = np.array(out)
    assert np.all(out > a)
    assert stats.kstest(out, stats.truncnorm(a, np.inf).cdf).pvalue > 1e-3


def test_wishart_mean(oracle_mod):
    """Bartlett draw: E[Omega] = df (S + I)^-1."""
    rng = np.random.default_rng(0)
    P, df = 3, 40
    A = rng.standard_normal((P, P))
    S = A @ A.T
    pb = _tiny_problem(oracle_mod, P)
    acc = np.zeros((P, P))
    n = 4000
    for _ in range(n):
        chi2 = np.array([rng.chisquare(df - i) for i in range(P)])
        wn = rng.standard_normal(P * (P - 1) // 2)
        om, ok = pb.wishart(S, chi2, wn)
        assert ok
        acc += om
    target = df * np.linalg.inv(S + np.eye(P))
    assert np.allclose(acc / n, target, rtol=0.05, atol=0.05 * np.abs(target).max())


def _tiny_problem(O, P):
    mask = np.ones((3, 3, 3), np.uint8)
    covar = np.ones((P, 5), np.float32)
    data = np.zeros((5, 27), np.uint8)
    return O.Problem(mask, covar, data, 1)


# ---------------------------------------------- pinned by the reference --
@pytest.mark.parametrize("name", golden_cases())
def test_oracle_matches_reference_golden(oracle_mod, name):
    """One sweep of the FP64 restatement equals the reference's own
    covar.cpp/cholesky.cpp (run on the same supplied variates) within the
    FP32 rounding of the reference."""
    g = load_golden(name)
    wm = g["wm"] if g["wm"].size else None
    bwm = float(g["beta_wm"])
    pb = oracle_mod.Problem(g["mask"], g["covar"], g["data"], int(g["nsubtypes"]), wm)
    lat = pb.lattice()
    for k in ["idx", "idxsc"]:
        assert np.array_equal(lat[k], g[k])
    for c in range(2):
        assert np.array_equal(lat["vox"][c], g[f"vox{c}"])
        assert np.array_equal(lat["nbrs"][c], g[f"nbrs{c}"])
    b, om, Z, S, fails, ok = pb.sweep_supplied(
        g["beta0"].astype(np.float64), g["omega0"].astype(np.float64), g["ubits"],
        g["normals"], g["chi2"], g["wnorm"], form=0, beta_wm=bwm)
    assert fails == 0 and ok
    if g["ref_Z"].size:  # (left out of the largest fixture)
        assert np.allclose(Z, g["ref_Z"], rtol=1e-5, atol=1e-5)
    assert np.allclose(b, g["ref_beta1"], rtol=1e-5, atol=1e-5)
    assert omega_rel_err(om, g["ref_omega1"]) <= 1e-5
    prb = pb.compute_prb(g["ref_beta1"].astype(np.float64), bwm)
    assert np.allclose(prb, g["ref_prb1"], atol=1e-6)


def test_lattice_properties(oracle_mod):
    """Colouring is a proper 2-colouring of the 6-neighbour lattice, and the
    neighbour counts and compact maps are consistent."""
    from bsglmm_gb300 import synth
    st = synth.small_study(21, shape=(11, 7, 9))
    pb = oracle_mod.Problem(st.mask, st.covar, st.data, 1)
    lat = pb.lattice()
    X, Y = pb.X, pb.Y
    offs = [1, -1, X + 2, -(X + 2), (X + 2) * (Y + 2), -(X + 2) * (Y + 2)]
    colour = np.full(pb.nsize, -1)
    for c in range(2):
        colour[lat["vox"][c]] = c
    for c in range(2):
        for j, v in enumerate(lat["vox"][c]):
            nb = [v + o for o in offs]
            assert all(colour[n] != c for n in nb)
            assert lat["nbrs"][c][j] == sum(lat["idx"][n] >= 0 for n in nb)
            assert all(lat["idxsc"][n] >= 0 for n in nb)
    assert pb.n0 + pb.n1 == pb.V == int(st.mask.sum())
    assert np.array_equal(np.sort(lat["idx"][lat["idx"] >= 0]), np.arange(pb.V))


# ------------------------------------- live reference (container only) --
def _ref_available(O):
    return O.REF_SUPPLIED.exists() and O.REF_KISS.exists()


def test_oracle_matches_live_reference_random(oracle_mod):
    O = oracle_mod
    if not _ref_available(O):
        pytest.skip("reference build (oracle/_ref) not present")
    from bsglmm_gb300 import synth
    st = synth.small_study(31, shape=(12, 10, 9), N=61, P=5, S=2)
    pb = O.Problem(st.mask, st.covar, st.data, st.nsubtypes)
    lat = pb.lattice()
    rng = np.random.default_rng(5)
    b0 = np.zeros((pb.P, pb.Vp), np.float32)
    b0[:, lat["idxsc"][lat["idx"] >= 0]] = st.beta_true
    om0 = (np.eye(pb.P) * 2).astype(np.float32)
    ub = rng.integers(0, 2**32, (pb.N, pb.V), dtype=np.uint64).astype(np.uint32)
    nm = rng.standard_normal((pb.V, pb.P)).astype(np.float32)
    df = pb.V + pb.P
    c2 = np.array([rng.chisquare(df - i) for i in range(pb.P)])
    wn = rng.standard_normal(pb.P * (pb.P - 1) // 2)
    ref = O.RefSupplied(pb)
    ref.set_supplied(ub, nm, c2, wn)
    rb, rom, rZ = ref.sweep(b0, om0)
    b, om, Z, S, fails, ok = pb.sweep_supplied(b0, om0, ub, nm, c2, wn, form=0)
    assert np.allclose(b, rb, rtol=1e-5, atol=1e-5)
    assert np.allclose(om, rom, rtol=1e-5, atol=1e-5 * np.abs(om).max())


@pytest.mark.parametrize("mu,lo,hi", [(-1.8, 0.0, 500.0), (0.4, 0.0, 500.0),
                                      (1.2, -500.0, -0.0), (-2.5, -500.0, -0.0)])
def test_reference_truncnorm_same_law(oracle_mod, mu, lo, hi):
    """The reference's Robert-1995 rejection sampler (randgen.cpp:726-814,
    KISS stream) and the oracle's inversion draw have the same law."""
    O = oracle_mod
    if not _ref_available(O):
        pytest.skip("reference build (oracle/_ref) not present")
    from bsglmm_gb300 import synth
    st = synth.small_study(1)
    ref = O.RefKiss(O.Problem(st.mask, st.covar, st.data, 1), seed=(7, 8, 9))
    xr = ref.truncnorm(mu, lo, hi, 4000)
    L = O.lib()
    ks = O.philox_block(3, 1, 4, 9, 10, 1000)
    if hi >= 500:
        xo = np.array([mu + L.orc_tn_lower_inv(-mu, int(k)) for k in ks])
    else:
        xo = np.array([mu - L.orc_tn_lower_inv(mu, int(k)) for k in ks])
    assert stats.ks_2samp(xr, xo).pvalue > 1e-3
