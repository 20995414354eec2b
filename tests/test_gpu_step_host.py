"""bsg_step_host: the per-sweep host round trip (Omega in, sweeps, Omega and
column means out) in one call equals the same steps as separate calls
(bsg_set_omega, bsg_run, bsg_get_omega, bsg_get_colmeans) bit for bit,
including a supplied Omega, several sweeps per call, zero sweeps and NULL
inputs and outputs; a wrong Omega size is refused before any work.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _two(st, seed):
    import bsglmm_gb300 as bsg
    a, b = bsg.Sampler(), bsg.Sampler()
    for s in (a, b):
        ds = s.add_dataset(st.mask, st.covar, st.data, st.nsubtypes)
        s.add_chain(ds, seed=seed)
    return a, b


def test_step_host_equals_separate_calls():
    from bsglmm_gb300 import synth
    st = synth.small_study(12, shape=(12, 11, 10), N=70, P=4, S=2)
    a, b = _two(st, 5)
    try:
        om = np.eye(4) * 2.0 + 0.1
        for k in range(4):
            n = 1 + k % 3
            o1, c1 = a.step_host(0, om if k % 2 == 0 else None, n)
            if k % 2 == 0:
                b.set_omega(0, om)
            b.run(n)
            o2, c2 = b.omega(0), b.colmeans(0)
            assert np.array_equal(o1, o2) and np.array_equal(c1, c2)
            om = o1
        # zero sweeps: a read-out only; an input Omega is installed
        o1, c1 = a.step_host(0, None, 0)
        assert np.array_equal(o1, b.omega(0)) and np.array_equal(c1, b.colmeans(0))
        o1, _ = a.step_host(0, om * 1.5, 0)
        assert np.array_equal(o1, om * 1.5)
        assert np.array_equal(a.beta(0), b.beta(0))
        # NULL outputs
        assert a._L.bsg_step_host(a._h, 0, None, 1, None, None) == 0
        b.set_omega(0, om * 1.5)
        b.run(1)
        assert np.array_equal(a.beta(0), b.beta(0))
        with pytest.raises(ValueError):
            a.step_host(0, np.eye(3), 1)
        assert a._L.bsg_step_host(a._h, 7, None, 1, None, None) != 0
        assert a._L.bsg_step_host(a._h, 0, None, -1, None, None) != 0
    finally:
        a.close()
        b.close()
