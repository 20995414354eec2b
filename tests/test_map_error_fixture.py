"""The committed error of the FP32 sampler's maps against the FP64 GPU chain
on the brain-sized studies (tests/golden/map_error_fp64.json, made on a
GB300 by tests/golden/make_map_error.py): for the 230k-voxel study with
N = 1000, P = 5 and with N = 2000, P = 8, every coefficient and
lesion-probability map entry of the FP32 chain lies within 0.5 MCSE of the
FP64 chain on the same counters (the headline's accuracy condition), and an
independent FP32 chain agrees with the FP64 chain within 4 combined MCSE on
at least 99.5 % of the entries (batch means over 40 batches, whose MCSE
estimates carry t(39) tails)."""
from __future__ import annotations

import json
from pathlib import Path

import pytest

FIXTURE = Path(__file__).resolve().parent / "golden" / "map_error_fp64.json"


@pytest.mark.parametrize("study", ["c1", "c2"])
def test_committed_map_error(study):
    r = json.loads(FIXTURE.read_text())[study]
    assert r["V"] == 230261 and r["N"] == {"c1": 1000, "c2": 2000}[study]
    for what in ("beta", "prb"):
        same = r[what]["same_counters"]
        assert same["max"] <= 0.5 and same["frac_le_0.5"] == 1.0, (what, same)
        assert r[what]["independent_chain_z"]["frac_within_4"] >= 0.995, what
