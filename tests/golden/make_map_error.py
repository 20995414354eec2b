"""Generates map_error_fp64.json: the error of the FP32 sampler's posterior
maps against the FP64 GPU chain on the brain-sized studies, where a CPU FP64
chain would take days (about 4 s per sweep of the 230k-voxel study on 8
host cores).

For each study: the FP64 chain, the FP32 chain on the same counters and an
independent FP32 chain run `burnin` sweeps and then `batches` x `batch` kept
sweeps (bsglmm_gb300.precision.map_error_vs_fp64); the MCSE of every map
entry comes from the FP64 chain's batch means.  Needs a GPU:

    python tests/golden/make_map_error.py [c1] [c2]     (default: both)

The lengths below are what one GPU call affords (the FP64 sweep costs
tens to hundreds of milliseconds at these sizes); they are recorded in the
file with the results.
"""
from __future__ import annotations

import json
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from bsglmm_gb300 import precision, synth  # noqa: E402

OUT = Path(__file__).resolve().parent / "map_error_fp64.json"

RUNS = {
    # study, seed, burnin, batches, batch
    "c1": (lambda: synth.config1(seed=1), 11, 500, 40, 200),
    "c2": (lambda: synth.config2(), 12, 300, 40, 200),
}


def main(names):
    res = json.loads(OUT.read_text()) if OUT.exists() else {}
    for name in names or list(RUNS):
        make, seed, burnin, batches, batch = RUNS[name]
        st = make()
        t0 = time.perf_counter()
        r = precision.map_error_vs_fp64(st, seed=seed, burnin=burnin, batches=batches,
                                        batch=batch)
        r["study"] = name
        r["wall_s"] = time.perf_counter() - t0
        res[name] = r
        print(name, json.dumps(r), flush=True)
        OUT.write_text(json.dumps(res, indent=1, sort_keys=True) + "\n")


if __name__ == "__main__":
    main(sys.argv[1:])
