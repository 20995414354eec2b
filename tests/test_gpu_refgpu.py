"""The reference's own GPU sweep on this GPU (covarGPU.cu's Z_GPU1,
Spat_Coef_Probit, reduce and Spat_Coef_Prec, compiled from the reference
tree to PTX and driven by oracle/refgpu_harness.cu as mcmc.cpp:314-394 drives
them), the form the GB300 sampler replaces.  Runs only where the PTX was
built (the reference tree was mounted at build time), in a child process
under a time limit.

The check is a sanity check of the harness's inputs and layouts, not a
parity test (the reference draws from cuRAND XORWOW streams the sampler
does not replay): after 220 sweeps of the 20^3 study both chains' coefficient
maps have the same spatial means to within the chains' Monte-Carlo spread,
and the reference's state is finite with a positive-definite Omega."""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]


def test_reference_gpu_sweep_runs_and_agrees_in_the_large(oracle_mod):
    if not oracle_mod.refgpu_available():
        pytest.skip("oracle/_ref/covarGPU.ptx not built (no reference tree at build time)")
    r = subprocess.run([sys.executable, str(ROOT / "oracle" / "refgpu_run.py"), "c0", "20",
                        "200"], capture_output=True, text=True, timeout=180)
    assert r.returncode == 0, r.stderr[-2000:]
    ref = json.loads(r.stdout.strip().splitlines()[-1])
    print(ref)
    assert ref["finite"]
    assert all(d > 0 for d in ref["omega_diag"])
    import bsglmm_gb300 as bsg
    from bsglmm_gb300 import synth
    st = synth.config0(0)
    with bsg.Sampler() as s:
        ds = s.add_dataset(st.mask, st.covar, st.data, st.nsubtypes)
        ch = s.add_chain(ds, seed=3, df_offset=19)  # the reference GPU path's df
        s.run(220)
        lat = s.lattice(ds)
        b = s.beta(ch)[:, lat["idxsc"][lat["idx"] >= 0]]
    ours = b.mean(axis=1)
    theirs = np.array(ref["coef_mean_over_voxels"])
    print("spatial means: ours", ours, "reference", theirs)
    assert np.allclose(ours, theirs, atol=0.15)
