"""Generates tests/golden/chain_c0.npz: an FP64 oracle chain on the 20^3
sphere study (r = 9, N = 50, P = 3, Wishart prior df P + 2), 1000 burn-in
sweeps then 20 batches of 100 kept sweeps, with the posterior-mean maps of
beta and of the lesion probability and their batch-means Monte-Carlo
standard errors.  The chain uses the sampler's Philox counters, so a GPU
chain with the same seed sees the same random numbers and the difference of
the maps measures FP32-versus-FP64 error alone.

Run from the repository root:  python tests/golden/make_chain_golden.py
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

SEED = 2025
BURNIN = 1000
NBATCH = 20
BATCH = 100


def main():
    O.build_oracle()
    st = synth.config0(seed=0)
    pb = O.Problem(st.mask, st.covar, st.data, 1)
    df_offset = pb.P + 2
    o = pb.chain(SEED, BURNIN, df_offset=df_offset, burnin=10**9)
    state = (o["beta"], o["omega"])
    bm, pm = [], []
    s0 = BURNIN
    for b in range(NBATCH):
        o = pb.chain(SEED, BATCH, df_offset=df_offset, burnin=-1, s0=s0,
                     spatcoef=state[0], omega=state[1])
        assert o["err"] == 0 and o["nkept"] == BATCH
        bm.append(o["mean"])
        pm.append(o["prb"])
        state = (o["beta"], o["omega"])
        s0 += BATCH
    bm, pm = np.array(bm), np.array(pm)
    np.savez_compressed(
        Path(__file__).resolve().parent / "chain_c0.npz",
        mask=st.mask, covar=st.covar, data_bits=np.packbits(st.data, axis=None),
        data_shape=np.array(st.data.shape), seed=np.uint64(SEED),
        df_offset=np.int32(df_offset), burnin=np.int32(BURNIN),
        nbatch=np.int32(NBATCH), batch=np.int32(BATCH),
        mean_beta=bm.mean(0), mcse_beta=bm.std(0, ddof=1) / np.sqrt(NBATCH),
        mean_prb=pm.mean(0), mcse_prb=pm.std(0, ddof=1) / np.sqrt(NBATCH),
        final_beta=state[0], final_omega=state[1])
    print("chain_c0.npz", pb.V, "voxels; median MCSE beta",
          float(np.median(bm.std(0, ddof=1) / np.sqrt(NBATCH))))


if __name__ == "__main__":
    main()
