"""GPU test of bsg_omega_update_noalloc, the allocation-free Omega | beta
draw.

It exists for callers that cannot allocate device memory while they run --
for example a plugin executing inside a runtime that owns every device
allocation, where a cudaMalloc would be refused or would stall the whole
device.  The caller passes device buffers it already owns; the reduction's
scratch comes from a fixed array inside the library.

The test calls it through the C ABI and checks its Omega against the one
the sampler draws at the end of a sweep (bsg_sweep_supplied / bsg_run) from
the same beta and variates, on two calls in a row so that the second call
runs on the scratch the first one left behind.  The two are computed
differently -- this entry point sums the pair products per thread in FP64
and factors by chol -> invert -> chol, the sampler sums them in FP32 warp
trees and uses a reverse Cholesky -- so they agree to rounding, checked at
1e-5 relative.  Device buffers for the test come from torch; the entry point
itself allocates nothing, which the last test checks through the device's
free memory around a call.  This file is collected last so a failure here
does not hide the other GPU tests.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-5
ATOL = 1e-5


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _noalloc(L, torch, s, ds, beta, P, chi2=None, wnorm=None, seed=0,
             chain=0, sweep=0):
    info = s.info(ds)
    lat = s.lattice(ds)
    vox = torch.from_numpy(np.concatenate(lat["vox"])).cuda()
    idxsc = torch.from_numpy(lat["idxsc"]).cuda()
    d_beta = torch.from_numpy(np.ascontiguousarray(beta)).cuda()
    d_om = torch.zeros((P, P), dtype=torch.float64, device="cuda")
    d_st = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    d_c2 = None if chi2 is None else torch.from_numpy(np.asarray(chi2, np.float64)).cuda()
    d_wn = None if wnorm is None else torch.from_numpy(
        np.asarray(wnorm if np.size(wnorm) else [0.0], np.float64)).cuda()
    torch.cuda.synchronize()
    status = L.bsg_omega_update_noalloc(
        _ptr(d_beta), _ptr(vox), _ptr(idxsc), info["X"], info["Y"], info["V"],
        info["Vp"], P, P, None if d_c2 is None else _ptr(d_c2),
        None if d_wn is None else _ptr(d_wn), seed, chain, sweep, _ptr(d_om),
        _ptr(d_st), None)
    torch.cuda.synchronize()
    return status, d_om.cpu().numpy(), int(d_st.cpu()[0])


def _study():
    from bsglmm_gb300 import synth
    return synth.small_study(61, shape=(12, 11, 10), N=50, P=4, S=1)


def test_noalloc_matches_sampler_with_supplied_variates():
    torch = pytest.importorskip("torch")
    import bsglmm_gb300 as bsg
    st = _study()
    rng = np.random.default_rng(8)
    with bsg.Sampler() as s:
        L = s._L
        ds = s.add_dataset(st.mask, st.covar, st.data, 1)
        ch = s.add_chain(ds, seed=3)
        info = s.info(ds)
        N, V, P = info["N"], info["V"], info["P"]
        for call in range(2):
            ub = rng.integers(0, 2**32, (N, V), dtype=np.uint64).astype(np.uint32)
            nm = rng.standard_normal((V, P)).astype(np.float32)
            c2 = np.array([rng.chisquare(V + P - i) for i in range(P)])
            wn = rng.standard_normal(P * (P - 1) // 2)
            s.sweep_supplied(ch, ub, nm, c2, wn, form=1)
            beta, om_ref = s.beta(ch), s.omega(ch)
            status, om, err = _noalloc(L, torch, s, ds, beta, P, c2, wn)
            assert status == 0 and err == 0, (call, status, err)
            assert np.allclose(om, om_ref, rtol=RTOL, atol=ATOL * np.abs(om_ref).max()), call


def test_noalloc_matches_sampler_with_philox_variates():
    torch = pytest.importorskip("torch")
    import bsglmm_gb300 as bsg
    st = _study()
    seed = 0xABCDEF12345
    with bsg.Sampler() as s:
        L = s._L
        ds = s.add_dataset(st.mask, st.covar, st.data, 1)
        ch = s.add_chain(ds, seed=seed)
        P = s.info(ds)["P"]
        for call in range(2):
            sweep, _ = s.sweep_count(ch)
            s.run(1)
            beta, om_ref = s.beta(ch), s.omega(ch)
            status, om, err = _noalloc(L, torch, s, ds, beta, P, seed=seed,
                                       chain=ch, sweep=sweep)
            assert status == 0 and err == 0, (call, status, err)
            assert np.allclose(om, om_ref, rtol=RTOL, atol=ATOL * np.abs(om_ref).max()), call


def test_noalloc_call_leaves_device_memory_unchanged():
    """After a first call (which loads the module), a further call takes no
    device memory: cudaMemGetInfo's free bytes are the same before and
    after it, with every buffer allocated beforehand."""
    torch = pytest.importorskip("torch")
    import bsglmm_gb300 as bsg
    st = _study()
    with bsg.Sampler() as s:
        L = s._L
        ds = s.add_dataset(st.mask, st.covar, st.data, 1)
        ch = s.add_chain(ds, seed=5)
        s.run(1)
        P = s.info(ds)["P"]
        info, lat = s.info(ds), s.lattice(ds)
        vox = torch.from_numpy(np.concatenate(lat["vox"])).cuda()
        idxsc = torch.from_numpy(lat["idxsc"]).cuda()
        d_beta = torch.from_numpy(np.ascontiguousarray(s.beta(ch))).cuda()
        d_om = torch.zeros((P, P), dtype=torch.float64, device="cuda")
        d_st = torch.zeros((1,), dtype=torch.int32, device="cuda")

        def call():
            return L.bsg_omega_update_noalloc(
                _ptr(d_beta), _ptr(vox), _ptr(idxsc), info["X"], info["Y"], info["V"],
                info["Vp"], P, P, None, None, 5, ch, 0, _ptr(d_om), _ptr(d_st), None)

        assert call() == 0
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        assert call() == 0
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        assert int(d_st.cpu()[0]) == 0
        assert free1 == free0, (free0, free1)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    import bsglmm_gb300 as bsg
    from bsglmm_gb300 import _lib
    L = _lib.lib()
    big = C.c_void_p(1)  # never dereferenced: sizes are checked first
    too_many = 4194304 + 1
    assert L.bsg_omega_update_noalloc(big, big, big, 10, 10, too_many, too_many, 4, 4,
                                      None, None, 0, 0, 0, big, None, None) == 8
    assert L.bsg_omega_update_noalloc(big, big, big, 10, 10, 100, 100, 9, 9,
                                      None, None, 0, 0, 0, big, None, None) == 8
    assert bsg  # package import keeps the GPU guard of the other tests
