"""Error of the FP32 sampler's posterior maps against an FP64 chain.

The FP32 sampler keeps FP64 only for Omega and the posterior sums.  Its maps
are measured against the FP64 chain (``Sampler.set_precision(chain, 64)``):
the same study, seed and chain id, so both chains consume the same Philox
variates (common random numbers).  The Monte-Carlo standard error (MCSE) of
every map entry comes from batch means of the FP64 chain, and the error is
reported as |mean_FP32 - mean_FP64| / MCSE for the coefficient maps
(spatCoef_*) and the lesion-probability maps (prb_*), the metric of
mcmc.cpp:871-964's outputs.  An independent FP32 chain (another seed) is run
beside them: its z = |mean - mean_FP64| / sqrt(MCSE_1^2 + MCSE_64^2) shows the
Monte-Carlo agreement of two independent chains.
"""
from __future__ import annotations

import time

import numpy as np

from .sampler import Sampler


class _BatchMeans:
    """Running sum and sum of squares of batch means (constant memory)."""

    def __init__(self):
        self.n = 0
        self.s = None
        self.s2 = None

    def add(self, m):
        m = np.asarray(m, np.float64)
        if self.s is None:
            self.s = np.zeros_like(m)
            self.s2 = np.zeros_like(m)
        self.s += m
        self.s2 += m * m
        self.n += 1

    def mean(self):
        return self.s / self.n

    def mcse(self):
        n = self.n
        var = np.maximum(self.s2 - self.s * self.s / n, 0.0) / (n - 1)
        return np.sqrt(var / n)


def _summary(err):
    e = np.asarray(err, np.float64).ravel()
    e = e[np.isfinite(e)]
    return {"max": float(e.max()), "median": float(np.median(e)),
            "p99": float(np.percentile(e, 99)),
            "frac_le_0.5": float(np.mean(e <= 0.5)), "entries": int(e.size)}


def map_error_vs_fp64(study, seed: int = 1, burnin: int = 1000, batches: int = 20,
                      batch: int = 100, independent: bool = True, device: int = 0,
                      df_offset: int | None = None) -> dict:
    """Runs the FP64 chain, the FP32 chain on the same counters and (if
    `independent`) an FP32 chain of seed + 1 for `burnin` sweeps and then
    `batches` batches of `batch` kept sweeps; returns the error summaries.
    Entries whose MCSE is zero (a map that does not move) are left out."""
    t0 = time.perf_counter()
    kinds = [("fp64", seed, 64), ("fp32", seed, 32)]
    if independent:
        kinds.append(("fp32_indep", seed + 1, 32))
    ctxs = {}
    for name, sd, bits in kinds:
        s = Sampler(device)
        ds = s.add_dataset(study.mask, study.covar, study.data, study.nsubtypes)
        ch = s.add_chain(ds, seed=sd, df_offset=df_offset)
        if bits == 64:
            s.set_precision(ch, 64)
        ctxs[name] = (s, ch)
    try:
        for s, ch in ctxs.values():
            s.run(burnin, sync=False)
        bm = {k: (_BatchMeans(), _BatchMeans()) for k in ctxs}
        for _ in range(batches):
            for s, ch in ctxs.values():
                s.reset_accumulators(ch)
                s.run(batch, sync=False)
            for k, (s, ch) in ctxs.items():
                mean, _, prb, nk = s.posterior(ch)
                assert nk == batch
                bm[k][0].add(mean)
                bm[k][1].add(prb)
        out = {"sweeps": burnin + batches * batch, "burnin": burnin,
               "batches": batches, "batch": batch, "seed": seed,
               "V": int(study.V), "N": int(study.N), "P": int(study.P)}
        for j, what in enumerate(("beta", "prb")):
            m64, se64 = bm["fp64"][j].mean(), bm["fp64"][j].mcse()
            ok = se64 > 0
            m32 = bm["fp32"][j].mean()
            err = np.where(ok, np.abs(m32 - m64) / np.where(ok, se64, 1.0), np.nan)
            res = {"same_counters": _summary(err),
                   "mcse_median": float(np.median(se64[ok]))}
            if independent:
                mi, sei = bm["fp32_indep"][j].mean(), bm["fp32_indep"][j].mcse()
                sc = np.sqrt(se64 ** 2 + sei ** 2)
                okz = sc > 0
                z = np.where(okz, np.abs(mi - m64) / np.where(okz, sc, 1.0), np.nan)
                zz = z[np.isfinite(z)]
                res["independent_chain_z"] = {
                    "max": float(zz.max()), "median": float(np.median(zz)),
                    "frac_within_4": float(np.mean(zz < 4.0)), "entries": int(zz.size)}
            out[what] = res
        out["seconds"] = time.perf_counter() - t0
        return out
    finally:
        for s, _ in ctxs.values():
            s.close()
