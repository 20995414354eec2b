"""Chain-level accuracy of the GPU sampler against the FP64 oracle chain
(tests/golden/chain_c0.npz: 20^3 sphere study, N = 50, P = 3, 1000 burn-in
+ 20 x 100 kept sweeps, batch-means Monte-Carlo standard errors).

* Same seed: the GPU chain consumes the oracle chain's random numbers, so
  the map difference is FP32-versus-FP64 error; it must stay within 0.5 MCSE
  everywhere (the ≤ 0.5 MCSE accuracy target).
* Independent seed: the maps of two independent chains agree within 4
  combined MCSE for 99.5 % of the entries (a check that the sampler targets
  the same posterior)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _fixture():
    with np.load(GOLDEN / "chain_c0.npz") as z:
        g = {k: z[k] for k in z.files}
    N, V = (int(x) for x in g["data_shape"])
    g["data"] = np.unpackbits(g["data_bits"])[: N * V].reshape(N, V)
    return g


def _gpu_batches(g, seed):
    import bsglmm_gb300 as bsg
    burnin, nbatch, batch = int(g["burnin"]), int(g["nbatch"]), int(g["batch"])
    with bsg.Sampler() as s:
        ds = s.add_dataset(g["mask"], g["covar"], g["data"], 1)
        ch = s.add_chain(ds, seed=seed, df_offset=int(g["df_offset"]),
                         burnin=burnin - 1)
        s.run(burnin)
        bm, pm = [], []
        for _ in range(nbatch):
            s.reset_accumulators(ch)
            s.run(batch)
            mean, _, prb, nk = s.posterior(ch)
            assert nk == batch
            bm.append(mean)
            pm.append(prb)
    bm, pm = np.array(bm), np.array(pm)
    return (bm.mean(0), bm.std(0, ddof=1) / np.sqrt(nbatch),
            pm.mean(0), pm.std(0, ddof=1) / np.sqrt(nbatch))


def test_maps_within_half_mcse_of_fp64_chain():
    g = _fixture()
    mb, _, mp, _ = _gpu_batches(g, int(g["seed"]))
    zb = np.abs(mb - g["mean_beta"]) / g["mcse_beta"]
    zp = np.abs(mp - g["mean_prb"]) / g["mcse_prb"]
    print(f"beta: max {zb.max():.3g} median {np.median(zb):.3g} MCSE; "
          f"prb: max {zp.max():.3g} median {np.median(zp):.3g} MCSE")
    assert zb.max() <= 0.5 and zp.max() <= 0.5


def test_independent_chain_agrees_within_mcse():
    g = _fixture()
    mb, sb, mp, sp = _gpu_batches(g, 987654321)
    zb = np.abs(mb - g["mean_beta"]) / np.sqrt(sb**2 + g["mcse_beta"] ** 2)
    zp = np.abs(mp - g["mean_prb"]) / np.sqrt(sp**2 + g["mcse_prb"] ** 2)
    z = np.concatenate([zb.ravel(), zp.ravel()])
    print(f"independent chains: frac within 4 MCSE {np.mean(z < 4):.4f}, max {z.max():.3g}")
    assert np.mean(z < 4) >= 0.995 and z.max() < 8
