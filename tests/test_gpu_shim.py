"""GPU test of the drop-in shim (bsglmm_gb300/csrc/shim/covarGPU_shim.cu):
a harness that calls the reference's launcher signatures in mcmc.cpp's
order must reproduce the native API's chain on the same Philox key, with
the host Omega round trip of the reference (float SpatCoefPrec)."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


def _kiss(s):
    m = (1 << 64) - 1
    s[1] = (s[1] ^ (s[1] << 17)) & m
    s[2] = ((s[2] ^ (s[2] << 18)) & 0x7FFFFFFF)
    s[0] = (69069 * s[0] + 23606797) & m
    s[1] ^= s[1] >> 15
    s[2] ^= s[2] >> 13
    return float((s[0] + s[1] + s[2]) & m) * 5.421010862427522e-20


def _build(tmp: Path) -> Path:
    from bsglmm_gb300 import build as B
    lib = B.build()
    exe = tmp / "shim_harness"
    nvcc = B.nvcc()
    cmd = [nvcc, *B.ARCH, "-O2", "-std=c++17", "-o", str(exe),
           str(ROOT / "tests" / "shim" / "shim_harness.cpp"),
           str(ROOT / "bsglmm_gb300" / "csrc" / "shim" / "covarGPU_shim.cu"),
           "-L", str(lib.parent), "-lbsglmm_gb300", f"-Xlinker=-rpath={lib.parent}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_shim_reproduces_native_chain(tmp_path):
    import bsglmm_gb300 as bsg
    from bsglmm_gb300 import synth
    st = synth.small_study(71, shape=(11, 10, 9), N=60, P=4, S=2)
    seed0 = [12345, 67891, 13579]
    with bsg.Sampler() as s:
        ds = s.add_dataset(st.mask, st.covar, st.data, 2)
        info = s.info(ds)
        lat = s.lattice(ds)
    hdr = np.array([info["X"], info["Y"], info["Z"], info["N"], info["P"], info["S"],
                    info["V"], info["Vp"]], np.int32)
    study = tmp_path / "study.bin"
    with open(study, "wb") as f:
        for a in (hdr, lat["idx"].astype(np.int32), st.covar.astype(np.float32),
                  st.data.astype(np.uint8), np.array(seed0, np.uint64)):
            f.write(np.ascontiguousarray(a).tobytes())
    exe = _build(tmp_path)
    K = 6
    out = tmp_path / "out.bin"
    r = subprocess.run([str(exe), str(study), str(K), str(out)], capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    P, Vp, V, S = info["P"], info["Vp"], info["V"], info["S"]
    raw = out.read_bytes()
    o = 0
    prec = np.frombuffer(raw, np.float32, P * P, o).reshape(P, P); o += 4 * P * P
    beta = np.frombuffer(raw, np.float32, P * Vp, o).reshape(P, Vp); o += 4 * P * Vp
    prb = np.frombuffer(raw, np.float32, S * V, o).reshape(S, V); o += 4 * S * V
    # the native API on the same key, with the shim's float Omega round trip
    ks = list(seed0)
    hi = int(_kiss(ks) * 4294967296.0)
    lo = int(_kiss(ks) * 4294967296.0)
    key = ((hi << 32) ^ lo) & ((1 << 64) - 1)
    o += 4 * P + 8 * 3  # column means, seed
    ed_shim = np.frombuffer(raw, np.float64, 1, o)[0]; o += 8
    q_shim = np.frombuffer(raw, np.float64, info["N"] * S, o).reshape(info["N"], S)
    from oracle import qhat_update, subtypes
    sub = subtypes(st.covar, S)
    q = np.zeros((info["N"], S))
    ed = 0.0
    with bsg.Sampler() as s:
        ds = s.add_dataset(st.mask, st.covar, st.data, 2)
        ch = s.add_chain(ds, seed=key, df_offset=19, burnin=2**31 - 1)
        om = np.eye(P, dtype=np.float32)
        for it in range(K):
            s.set_omega(ch, om.astype(np.float64))
            s.run(1)
            om = s.omega(ch).astype(np.float32)
            if it > 0:
                mp = s.predict(ch)
                for i in range(info["N"]):
                    ed += mp[i, sub[i]]
                qhat_update(q, mp, sub, first=it == 1)
        assert np.array_equal(s.beta(ch), beta)
        assert np.array_equal(om, prec)
        assert np.allclose(s.compute_prb(ch), prb)
    # compute_predictGPU through the shim = the library pass + the
    # reference's host update of ED and Qhat
    assert ed_shim == pytest.approx(ed, rel=1e-13)
    assert np.allclose(q_shim, q, rtol=1e-12, atol=1e-12)


def test_shim_wm_update_reproduces_native_chain(tmp_path):
    """With the WM argument (UPDATE_WM) the harness calls updateBetaGPU
    before every coefficient update, as mcmc.cpp:344-345 does; the shimmed
    program equals the native chain with its beta_WM update on."""
    import bsglmm_gb300 as bsg
    from bsglmm_gb300 import synth
    st = synth.small_study(73, shape=(10, 9, 8), N=48, P=3, S=1)
    wm = np.random.default_rng(74).random(st.V).astype(np.float32)
    seed0 = [2468, 1357, 9753]
    with bsg.Sampler() as s:
        ds = s.add_dataset(st.mask, st.covar, st.data, 1, wm)
        info = s.info(ds)
        lat = s.lattice(ds)
    hdr = np.array([info["X"], info["Y"], info["Z"], info["N"], info["P"], info["S"],
                    info["V"], info["Vp"]], np.int32)
    study = tmp_path / "study.bin"
    with open(study, "wb") as f:
        for a in (hdr, lat["idx"].astype(np.int32), st.covar.astype(np.float32),
                  st.data.astype(np.uint8), np.array(seed0, np.uint64), wm):
            f.write(np.ascontiguousarray(a).tobytes())
    exe = _build(tmp_path)
    K = 5
    out = tmp_path / "out.bin"
    r = subprocess.run([str(exe), str(study), str(K), str(out), "wm"],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    P, Vp, V, S, N = info["P"], info["Vp"], info["V"], info["S"], info["N"]
    raw = out.read_bytes()
    o = 0
    prec = np.frombuffer(raw, np.float32, P * P, o).reshape(P, P); o += 4 * P * P
    beta = np.frombuffer(raw, np.float32, P * Vp, o).reshape(P, Vp); o += 4 * P * Vp
    o += 4 * S * V + 4 * P + 8 * 3 + 8 + 8 * N * S  # prb, means, seed, ED, Qhat
    bwm_shim = np.frombuffer(raw, np.float32, 1, o)[0]
    ks = list(seed0)
    hi = int(_kiss(ks) * 4294967296.0)
    lo = int(_kiss(ks) * 4294967296.0)
    key = ((hi << 32) ^ lo) & ((1 << 64) - 1)
    with bsg.Sampler() as s:
        ds = s.add_dataset(st.mask, st.covar, st.data, 1, wm)
        ch = s.add_chain(ds, seed=key, df_offset=19, burnin=2**31 - 1)
        s.set_wm_update(ch, True)
        om = np.eye(P, dtype=np.float32)
        for _ in range(K):
            s.set_omega(ch, om.astype(np.float64))
            s.run(1)
            om = s.omega(ch).astype(np.float32)
        assert np.array_equal(s.beta(ch), beta)
        assert np.array_equal(om, prec)
        b_native, _ = s.beta_wm(ch)
    assert bwm_shim == b_native and bwm_shim != 0.0


def test_shim_t_link_reproduces_native_chain(tmp_path):
    """With MODEL = 2 (t link) the shimmed program runs the library's
    scale-mixture chain: equal to the native chain with set_model(2)."""
    import bsglmm_gb300 as bsg
    from bsglmm_gb300 import synth
    st = synth.small_study(75, shape=(9, 9, 8), N=40, P=3, S=1)
    seed0 = [1111, 2222, 3333]
    with bsg.Sampler() as s:
        ds = s.add_dataset(st.mask, st.covar, st.data, 1)
        info = s.info(ds)
        lat = s.lattice(ds)
    hdr = np.array([info["X"], info["Y"], info["Z"], info["N"], info["P"], info["S"],
                    info["V"], info["Vp"]], np.int32)
    study = tmp_path / "study.bin"
    with open(study, "wb") as f:
        for a in (hdr, lat["idx"].astype(np.int32), st.covar.astype(np.float32),
                  st.data.astype(np.uint8), np.array(seed0, np.uint64)):
            f.write(np.ascontiguousarray(a).tobytes())
    exe = _build(tmp_path)
    K = 4
    out = tmp_path / "out.bin"
    r = subprocess.run([str(exe), str(study), str(K), str(out), "model=2"],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    P, Vp = info["P"], info["Vp"]
    raw = out.read_bytes()
    prec = np.frombuffer(raw, np.float32, P * P, 0).reshape(P, P)
    beta = np.frombuffer(raw, np.float32, P * Vp, 4 * P * P).reshape(P, Vp)
    ks = list(seed0)
    hi = int(_kiss(ks) * 4294967296.0)
    lo = int(_kiss(ks) * 4294967296.0)
    key = ((hi << 32) ^ lo) & ((1 << 64) - 1)
    with bsg.Sampler() as s:
        ds = s.add_dataset(st.mask, st.covar, st.data, 1)
        ch = s.add_chain(ds, seed=key, df_offset=19, burnin=2**31 - 1)
        s.set_model(ch, 2)
        om = np.eye(P, dtype=np.float32)
        for _ in range(K):
            s.set_omega(ch, om.astype(np.float64))
            s.run(1)
            om = s.omega(ch).astype(np.float32)
        assert np.array_equal(s.beta(ch), beta)
        assert np.array_equal(om, prec)
