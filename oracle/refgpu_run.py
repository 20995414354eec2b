"""TEST / MEASUREMENT INFRASTRUCTURE ONLY: times the reference's own GPU
sweep (covarGPU.cu's kernels, JIT-loaded from oracle/_ref/covarGPU.ptx and
driven by librefgpu.so as the reference's launchers drive them) on one
synthetic study, and prints one JSON line.  Run as a child process (bench.py's
reference arm and the tests do, under a time limit):

    python oracle/refgpu_run.py <study> <warmup sweeps> <timed sweeps> [seed]
    python oracle/refgpu_run.py chain <model> <burn-in> <kept sweeps> [seed]

study: c0 (20^3 sphere, N = 50, P = 3) or c1 (91x109x91 ellipsoid,
N = 1000, P = 5).  The chain form runs the box study (BOX below: both
colours fill whole 192-voxel blocks, which the reference's weighted
Spat_Coef needs) with the link `model` (1 probit, 0 logistic, 2 t) and
prints, per kept sweep, the mean over the mask of every coefficient map.  Inputs are finite and the chain starts from beta = 0,
Omega = I (mcmc.cpp:149-154,227), so the reference's unbounded rejection
loops (covarGPU.cu:1126-1143,1170-1194) see finite means only.
"""
from __future__ import annotations

import json
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
sys.path.insert(0, str(HERE))

import oracle  # noqa: E402
from bsglmm_gb300 import synth  # noqa: E402

STUDIES = {"c0": lambda: synth.config0(0), "c1": lambda: synth.config1(seed=1)}


def box_study():
    """24 x 16 x 12 box (4,608 voxels, 2,304 per colour), N = 60, P = 3."""
    mask = np.ones((12, 16, 24), np.uint8)
    return synth.make_study("box", mask, 60, 3, 3.0, 0.2, 17)


def chain(argv):
    model, burn, kept = int(argv[0]), int(argv[1]), int(argv[2])
    seed = int(argv[3]) if len(argv) > 3 else 1
    st = box_study()
    pb = oracle.Problem(st.mask, st.covar, st.data, st.nsubtypes)
    rg = oracle.RefGpu(pb, seed=seed)
    rg.set_model(model)
    lat = pb.lattice()
    cols = lat["idxsc"][lat["idx"] >= 0]
    rg.sweeps(burn)
    series = []
    for _ in range(kept):
        rg.sweeps(1)
        series.append([float(x) for x in rg.beta()[:, cols].mean(axis=1)])
    rg.close()
    print(json.dumps({"model": model, "burnin": burn, "kept": kept, "V": int(st.V),
                      "series": series}))


def main(argv):
    if argv[0] == "chain":
        chain(argv[1:])
        return
    name, warm, timed = argv[0], int(argv[1]), int(argv[2])
    seed = int(argv[3]) if len(argv) > 3 else 1
    st = STUDIES[name]()
    pb = oracle.Problem(st.mask, st.covar, st.data, st.nsubtypes)
    t0 = time.perf_counter()
    rg = oracle.RefGpu(pb, seed=seed)
    setup_s = time.perf_counter() - t0
    if warm:
        rg.sweeps(warm)
    ms = rg.sweeps(timed)
    b = rg.beta()
    lat = pb.lattice()
    cols = lat["idxsc"][lat["idx"] >= 0]
    bm = b[:, cols]
    om = rg.omega()
    rg.close()
    upd = st.N * st.V
    print(json.dumps({
        "study": name, "V": int(st.V), "N": int(st.N), "P": int(st.P),
        "warmup_sweeps": warm, "timed_sweeps": timed, "ms_per_sweep": ms,
        "updates_per_s": upd / (ms * 1e-3), "sweeps_per_s": 1e3 / ms,
        "setup_s": setup_s, "finite": bool(np.isfinite(bm).all() and np.isfinite(om).all()),
        "coef_mean_over_voxels": [float(x) for x in bm.mean(axis=1)],
        "omega_diag": [float(om[i, i]) for i in range(st.P)]}))


if __name__ == "__main__":
    main(sys.argv[1:])
