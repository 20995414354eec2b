"""Generates the golden fixtures in this directory from the reference's own
CPU update code (nicholst/BSGLMM bsglmm/covar.cpp + cholesky.cpp, compiled
from the reference tree into oracle/_ref/ by `make -C oracle ref`) driven by
supplied variates.

Each fixture holds the inputs (study, initial state, variates) and the
reference's outputs of one sweep in the reference's order
(updateZ -> updateSpatCoef -> updateSpatCoefPrec, mcmc.cpp:400-428) plus
compute_prb (covar.cpp:350-364) of the new state.

The "c0" fixture is the benchmark's CPU-runnable study at full size (20^3
grid, sphere r = 9 about (10.5, 10.5, 10.5), N = 50, P = 3); its latent Z
(N V values) is left out to keep the file small.

Run from the repository root:  python tests/golden/make_golden.py [name ...]
(no names: every fixture).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import oracle as O  # noqa: E402
from bsglmm_gb300 import synth  # noqa: E402

OUT = Path(__file__).resolve().parent


def cases():
    yield "ragged_p4_s2", synth.small_study(3), None, 0.0
    yield "sphere_p3", _sphere(), None, 0.0
    yield "p8_n70", synth.small_study(5, shape=(8, 8, 8), N=70, P=8, S=1), None, 0.0
    yield "p1_n33", synth.small_study(7, shape=(9, 7, 6), N=33, P=1, S=1), None, 0.0
    st = synth.small_study(9, shape=(7, 8, 9), N=45, P=3, S=2)
    wm = np.random.default_rng(9).uniform(0.05, 1.0, st.V).astype(np.float32)
    yield "wm_p3", st, wm, 0.4
    yield "c0", synth.config0(0), None, 0.0


def _sphere():
    rng = np.random.default_rng(11)
    mask = synth.sphere_mask(10, 4.5)
    N, P = 50, 3
    X = synth.design(rng, N, P, "c0")
    V = int(mask.sum())
    beta = np.stack([rng.normal(-1.6, 0.5, V), rng.normal(0, 0.3, V),
                     rng.normal(0, 0.3, V)]).astype(np.float32)
    data = synth.draw_outcomes(rng, X, beta)
    return synth.Study("sphere", mask, X, data, beta, 1)


def make(name, st, wm, beta_wm, seed):
    pb = O.Problem(st.mask, st.covar, st.data, st.nsubtypes, wm)
    lat = pb.lattice()
    rng = np.random.default_rng(seed)
    inmask = lat["idx"] >= 0
    sc_of_v = lat["idxsc"][inmask]  # compact order == padded scan order
    beta0 = np.zeros((pb.P, pb.Vp), np.float32)
    beta0[:, sc_of_v] = st.beta_true
    A = rng.standard_normal((pb.P, pb.P))
    omega0 = (np.eye(pb.P) * 1.5 + 0.1 * (A @ A.T)).astype(np.float32)
    ubits = rng.integers(0, 2 ** 32, size=(pb.N, pb.V), dtype=np.uint64).astype(np.uint32)
    normals = rng.standard_normal((pb.V, pb.P)).astype(np.float32)
    df = pb.V + pb.P
    chi2 = np.array([rng.chisquare(df - i) for i in range(pb.P)])
    wnorm = rng.standard_normal(pb.P * (pb.P - 1) // 2)
    ref = O.RefSupplied(pb)
    ref.set_supplied(ubits, normals, chi2, wnorm)
    b1, om1, Z = ref.sweep(beta0, omega0, beta_wm)
    assert not ref.underrun()
    shapes = ref.gamma_shapes()
    assert np.allclose(shapes, [0.5 * (df - i) for i in range(pb.P)])
    prb1 = ref.compute_prb(b1, beta_wm)
    arrays = dict(
        mask=st.mask, covar=st.covar, data=st.data, nsubtypes=st.nsubtypes,
        wm=wm if wm is not None else np.zeros(0, np.float32),
        beta_wm=np.float32(beta_wm), beta0=beta0, omega0=omega0, ubits=ubits,
        normals=normals, chi2=chi2, wnorm=wnorm, df_offset=np.int32(pb.P),
        ref_Z=np.zeros(0) if name == "c0" else Z, ref_beta1=b1, ref_omega1=om1, ref_prb1=prb1,
        idx=lat["idx"], idxsc=lat["idxsc"], vox0=lat["vox"][0],
        vox1=lat["vox"][1], nbrs0=lat["nbrs"][0], nbrs1=lat["nbrs"][1])
    np.savez_compressed(OUT / f"sweep_{name}.npz", **arrays)
    print(f"sweep_{name}.npz  V={pb.V} Vp={pb.Vp} N={pb.N} P={pb.P}")


def main(names):
    O.build_oracle(ref=True)
    for k, (name, st, wm, bwm) in enumerate(cases()):
        if not names or name in names:
            make(name, st, wm, bwm, 100 + k)


if __name__ == "__main__":
    main(sys.argv[1:])
