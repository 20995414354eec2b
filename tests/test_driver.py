"""The BinCar-compatible driver: NIfTI-1 reading and writing, the design and
mask readers, the empirical maps, the KISS seed stream and the command line
(CPU), and a whole run through the command line on the GPU."""
from __future__ import annotations

import gzip
import struct

import numpy as np
import pytest

from bsglmm_gb300 import driver, nifti


def _ref_kiss(O, seed):
    """The reference harness (oracle/_ref) when it was built, else None."""
    if not O.REF_KISS.exists():
        return None
    from bsglmm_gb300 import synth
    st = synth.small_study(1)
    return O.RefKiss(O.Problem(st.mask, st.covar, st.data, 1), seed=tuple(seed))


def write_study(root, seed=5, shape=(9, 8, 7), N=23, ntypes=2, extra=1):
    """A study on disk as the reference program reads it: images/mask.nii.gz
    (FLOAT64), one lesion map per subject (FLOAT32 and FLOAT64, .nii and
    .nii.gz), design.txt with group indicator columns then covariates."""
    rng = np.random.default_rng(seed)
    X, Y, Z = shape
    img = root / "images"
    img.mkdir(parents=True, exist_ok=True)
    mask = (rng.random((Z, Y, X)) < 0.6).astype(np.float64)
    mask[mask > 0] = rng.choice([1.0, 1.9, 3.0], int(mask.sum()))  # truncates to nonzero
    mask[0, 0, :3] = 0.4                                         # truncates to 0
    nifti.write_nifti(img / "mask.nii.gz", mask, (X, Y, Z))
    m = driver._as_byte(mask) != 0
    V = int(m.sum())
    grp = rng.integers(0, ntypes, N)
    P = ntypes + extra
    covar = np.zeros((P, N), np.float32)
    for g in range(ntypes):
        covar[g] = grp == g
    for p in range(ntypes, P):
        covar[p] = np.round(rng.standard_normal(N), 3)
    eta = -0.8 + 0.6 * (grp[:, None] == 1) + 0.3 * rng.standard_normal((N, V))
    data = (rng.random((N, V)) < 1.0 / (1.0 + np.exp(-2 * eta))).astype(np.uint8)
    names = [f"G{g}" for g in range(ntypes)] + [f"Cov{p}" for p in range(extra)]
    lines = ["ID\t" + "\t".join(names) + "\tImage"]
    for i in range(N):
        vol = np.zeros((Z, Y, X))
        vol[m] = data[i]
        fn = f"sub{i:03d}.nii" + (".gz" if i % 3 else "")
        dt = nifti.FLOAT32 if i % 2 else nifti.FLOAT64
        nifti.write_nifti(img / fn, vol, (X, Y, Z), datatype=dt)
        lines.append(f"S{i}\t" + "\t".join(f"{covar[p, i]:g}" for p in range(P)) + f"\t{fn}")
    (root / "design.txt").write_text("\n".join(lines) + "\n")
    return dict(mask=m.astype(np.uint8), covar=covar, data=data, names=names,
                dims=(X, Y, Z), ntypes=ntypes, P=P)


# ------------------------------------------------------------------ NIfTI --
@pytest.mark.parametrize("suffix", [".nii", ".nii.gz"])
@pytest.mark.parametrize("dt", [nifti.FLOAT64, nifti.FLOAT32, nifti.UINT8, nifti.INT16])
def test_nifti_round_trip(tmp_path, suffix, dt):
    rng = np.random.default_rng(1)
    vol = rng.integers(0, 100, (5, 4, 3)).astype(np.float64)
    p = tmp_path / ("a" + suffix)
    nifti.write_nifti(p, vol, (3, 4, 5), datatype=dt)
    if suffix == ".nii.gz":
        assert p.read_bytes()[:2] == b"\x1f\x8b"
    img = nifti.read_nifti(p)
    assert img.dims == (3, 4, 5) and img.datatype == dt
    assert img.data.shape == (5, 4, 3)
    assert np.array_equal(img.data.astype(np.float64), vol)
    assert img.pixdim == pytest.approx((2.0, 2.0, 2.0))


def test_nifti_header_fields(tmp_path):
    """348-byte header, 4-byte extension flag, data at 352, magic n+1."""
    blob = nifti.nifti_bytes(np.arange(24.0), (2, 3, 4))
    assert len(blob) == 352 + 24 * 8
    assert struct.unpack("<i", blob[:4])[0] == 348
    assert struct.unpack("<8h", blob[40:56]) == (3, 2, 3, 4, 1, 0, 0, 0)
    assert struct.unpack("<2h", blob[70:74]) == (nifti.FLOAT64, 64)
    assert struct.unpack("<f", blob[108:112])[0] == 352.0
    assert blob[123] == 2 and blob[344:348] == b"n+1\x00"
    assert np.array_equal(np.frombuffer(blob[352:], "<f8"), np.arange(24.0))


def test_nifti_writer_matches_reference_bytes(tmp_path, oracle_mod):
    """Byte-identical to the reference's writer (nifti1_read_write.cpp) on the
    same volume, built from the reference's own source into oracle/_ref."""
    ref = _ref_kiss(oracle_mod, (1, 2, 2))
    if ref is None:
        pytest.skip("reference build (oracle/_ref) not present")
    vol = np.random.default_rng(3).random((6, 5, 4))
    rp = tmp_path / "ref.nii"
    assert ref.write_nifti(rp, vol) == 0
    assert rp.read_bytes() == nifti.nifti_bytes(vol.reshape(-1), (4, 5, 6))


def test_nifti_reads_big_endian(tmp_path):
    vol = np.arange(60, dtype=np.float32).reshape(5, 4, 3)
    hdr = bytearray(348)
    struct.pack_into(">i", hdr, 0, 348)
    struct.pack_into(">8h", hdr, 40, 3, 3, 4, 5, 1, 0, 0, 0)
    struct.pack_into(">2h", hdr, 70, nifti.FLOAT32, 32)
    struct.pack_into(">8f", hdr, 76, 0, 1.5, 1.5, 1.5, 0, 0, 0, 0)
    struct.pack_into(">f", hdr, 108, 352.0)
    hdr[344:348] = b"n+1\x00"
    p = tmp_path / "be.nii.gz"
    p.write_bytes(gzip.compress(bytes(hdr) + b"\0" * 4 + vol.astype(">f4").tobytes()))
    img = nifti.read_nifti(p)
    assert img.datatype == nifti.FLOAT32 and np.array_equal(img.data, vol)


def test_nifti_rejects_bad_files(tmp_path):
    good = nifti.nifti_bytes(np.zeros(8), (2, 2, 2))
    cases = {
        "missing.nii": None,
        "short.nii": good[:200],
        "magic.nii": good[:344] + b"ni1\0" + good[348:],
        "size.nii": b"\0\0\0\0" + good[4:],
        "trunc.nii": good[:-8],
        "dtype.nii": good[:70] + struct.pack("<h", 2304) + good[72:],
    }
    for name, blob in cases.items():
        p = tmp_path / name
        if blob is not None:
            p.write_bytes(blob)
        with pytest.raises(nifti.NiftiError):
            nifti.read_nifti(p)


# -------------------------------------------------------------- readers --
def test_read_design_and_lesions(tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    st = write_study(tmp_path)
    mask = driver.read_mask(driver.IMAGE_DIR / "mask.nii.gz")
    assert np.array_equal(mask, st["mask"])
    names, covar, images = driver.read_design("design.txt", st["P"], st["ntypes"])
    assert names == st["names"]
    assert covar.dtype == np.float32 and np.array_equal(covar, st["covar"])
    assert [p.name for p in images][:2] == ["sub000.nii", "sub001.nii.gz"]
    data = driver.read_lesions(images, mask)
    assert np.array_equal(data, st["data"])


def test_read_wm(tmp_path):
    mask = np.zeros((2, 3, 4), np.uint8)
    mask[0, 1, :3] = mask[1, 2, 1] = 1
    vol = np.arange(24, dtype=np.float64).reshape(2, 3, 4) * 10
    nifti.write_nifti(tmp_path / "wm.nii.gz", vol, (4, 3, 2), datatype=nifti.UINT8)
    wm = driver.read_wm(tmp_path / "wm.nii.gz", mask)
    assert wm.dtype == np.float32
    assert np.array_equal(wm, vol[mask.astype(bool)].astype(np.float32) / np.float32(255))
    nifti.write_nifti(tmp_path / "wm64.nii", vol, (4, 3, 2))
    with pytest.raises(driver.DriverError, match="UINT8"):
        driver.read_wm(tmp_path / "wm64.nii", mask)


def test_mask_byte_conversion():
    """(unsigned char) of the mask's doubles: truncation, then the low byte."""
    v = np.array([0.0, 0.99, 1.0, 1.7, 255.9, 256.0, 257.5])
    assert list(driver._as_byte(v)) == [0, 0, 1, 1, 255, 0, 1]


def test_reader_errors(tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    st = write_study(tmp_path, N=4)
    img = tmp_path / "images"
    nifti.write_nifti(img / "m32.nii", np.ones(8), (2, 2, 2), datatype=nifti.FLOAT32)
    with pytest.raises(driver.DriverError, match="FLOAT64"):
        driver.read_mask(img / "m32.nii")
    (tmp_path / "bad.txt").write_text("ID A B Image\n1 1 2 x.nii\n2 1\n")
    with pytest.raises(driver.DriverError, match="multiple"):
        driver.read_design(tmp_path / "bad.txt", 2, 1)
    (tmp_path / "nan.txt").write_text("ID A B Image\n1 one 2 x.nii\n")
    with pytest.raises(driver.DriverError, match="non-numeric"):
        driver.read_design(tmp_path / "nan.txt", 2, 1)
    nifti.write_nifti(img / "u8.nii", np.ones(8), (2, 2, 2), datatype=nifti.UINT8)
    with pytest.raises(driver.DriverError, match="FLOAT32"):
        driver.read_lesions([img / "u8.nii"], np.ones((2, 2, 2), np.uint8))
    X, Y, Z = st["dims"]
    with pytest.raises(driver.DriverError, match="dimensions"):
        driver.read_lesions([img / "sub000.nii"], np.ones((Z + 1, Y, X), np.uint8))


def test_empirical_maps_match_loop_restatement():
    """write_empir_prb (read_data.cpp:418-487) restated as its voxel loop."""
    rng = np.random.default_rng(2)
    mask = (rng.random((4, 5, 6)) < 0.5).astype(np.uint8)
    V, N, S = int(mask.sum()), 11, 2
    covar = np.stack([rng.integers(0, 2, N), rng.integers(0, 2, N),
                      rng.standard_normal(N)]).astype(np.float32)
    covar[1, :] = 0  # an empty group: 0/0 as in C
    data = rng.integers(0, 2, (N, V)).astype(np.uint8)
    groups, total, total_p = driver.empirical_maps(mask, covar, data, S)
    flat = mask.ravel()
    cnt = 0
    for r in range(flat.size):
        s2 = 0.0
        for g in range(S):
            if flat[r]:
                s = n = 0.0
                for i in range(N):
                    if covar[g, i]:
                        s += data[i, cnt]
                        n += 1
                s2 += s
                if n:
                    assert groups[g][r] == s / n
                else:
                    assert np.isnan(groups[g][r])
            else:
                assert groups[g][r] == 0.0
        assert total[r] == s2 and total_p[r] == s2 / N
        cnt += int(flat[r])


def test_qhat_lines_format_and_rules():
    """Qhat.dat rows (mcmc.cpp:719-751): normalised exp(Qhat) with %.6f,
    the predicted group is the last maximum, the true group the first
    nonzero group column (else 0); Qhat2.dat scales by the group prior."""
    q = np.array([[0.0, np.log(3.0)], [-1.0, -1.0], [2.0, -5.0]])
    covar = np.array([[1, 0, 0], [0, 1, 0], [0.5, 0.2, 0.1]], np.float32)
    text = driver.qhat_lines(q, covar, 2)
    assert text.splitlines() == ["0 0.250000 0.750000 1 0",
                                 "1 0.500000 0.500000 1 1",
                                 "2 0.999089 0.000911 0 0"]
    prior = driver.group_prior(np.array([[1.0, 1.0, 0.0], [0.0, 0.9, 1.0]]), 2)
    assert np.allclose(prior, [2 / 3, 1 / 3])  # (int) of each entry
    t2 = driver.qhat_lines(q, covar, 2, prior).splitlines()[0].split()
    w = np.exp(q[0] * prior - np.logaddexp.reduce(q[0] * prior))
    assert t2[1:3] == [f"{w[0]:.6f}", f"{w[1]:.6f}"]


# ------------------------------------------------------------ seed stream --
def test_kiss_matches_reference_stream(oracle_mod):
    seed = [123456789, 362436069, 521288629]
    ref = _ref_kiss(oracle_mod, seed)
    if ref is None:
        pytest.skip("reference build (oracle/_ref) not present")
    want, state = ref.kiss(2000)
    s = list(seed)
    got = np.array([driver.kiss(s) for _ in range(2000)])
    assert np.array_equal(got, want) and s == state


def test_chain_key_advances_seed():
    s = [1, 2, 2]
    k1 = driver.chain_key(s)
    k2 = driver.chain_key(s)
    assert k1 != k2 and 0 <= k1 < 2 ** 64 and s != [1, 2, 2]


def test_seed_file(tmp_path, monkeypatch, capsys):
    monkeypatch.chdir(tmp_path)
    assert driver.read_seed() == [1, 2, 2]
    assert "No seed.dat found" in capsys.readouterr().out
    (tmp_path / "seed.dat").write_text("7 8 9\n")
    assert driver.read_seed() == [7, 8, 9]
    (tmp_path / "seed.dat").write_text("7 8\n")
    with pytest.raises(driver.DriverError):
        driver.read_seed()


# ------------------------------------------------------------ command line --
def test_cli_usage_and_unsupported_options(tmp_path, monkeypatch, capsys):
    monkeypatch.chdir(tmp_path)
    assert driver.main([]) == 1
    assert "Usage" in capsys.readouterr().out
    assert driver.main(["1", "2", "1", "d.txt", "1"]) == 1
    assert driver.main(["x", "2", "1", "d.txt", "1", "0"]) == 1
    assert driver.main(["1", "2", "0", "d.txt", "1", "0"]) == 2
    assert "GPU = 0" in capsys.readouterr().err
    assert driver.main(["1", "2", "1", "d.txt", "1", "1"]) == 2
    assert "mask.nii.gz: no such file" in capsys.readouterr().err
    assert driver.main(["1", "2", "1", "d.txt", "1", "0", "10", "20"]) == 2
    out = capsys.readouterr()
    assert "Silly-small" in out.out and "Burn-in exceeds" in out.out
    assert "mask.nii.gz: no such file" in out.err


# -------------------------------------------------------------------- GPU --
@pytest.mark.gpu
def test_driver_run_equals_native_chain(tmp_path, monkeypatch, capsys):
    """A whole BinCar-style run (10,101 sweeps, 10,000 kept): every output
    image holds exactly the native sampler's maps for the key drawn from
    seed.dat, the empirical maps equal the direct computation, and seed.dat
    advances by the two KISS draws."""
    import bsglmm_gb300 as bsg
    monkeypatch.chdir(tmp_path)
    st = write_study(tmp_path, N=31, shape=(12, 11, 10))
    (tmp_path / "seed.dat").write_text("11 22 33\n")
    assert driver.main([str(st["ntypes"]), str(st["P"]), "1", "design.txt", "1",
                        "0", "10100", "100"]) == 0
    out = capsys.readouterr().out
    assert "TOTSAV = 10000" in out and "iter = 10100" in out
    seed = [11, 22, 33]
    key = driver.chain_key(seed)
    assert (tmp_path / "seed.dat").read_text().split() == [str(x) for x in seed]
    with bsg.Sampler() as s:
        ds = s.add_dataset(st["mask"], st["covar"], st["data"], st["ntypes"])
        ch = s.add_chain(ds, seed=key, burnin=100, thin=1, df_offset=19)
        s.set_predictive(ch, True)
        s.run(10101)
        maps = s.maps(ch)
        assert s.sweep_count(ch) == (10101, 10000)
        qhat, ed, npred = s.predictive(ch)
        dic = s.dic(ch)
    assert npred == 10000
    assert (tmp_path / "Qhat.dat").read_text() == driver.qhat_lines(
        qhat, st["covar"], st["ntypes"])
    assert (tmp_path / "Qhat2.dat").read_text() == driver.qhat_lines(
        qhat, st["covar"], st["ntypes"], driver.group_prior(st["covar"], st["ntypes"]))
    assert (tmp_path / "DIC.dat").read_text() == (
        "DE = {DE:f} ED = {ED:f} PD = {PD:f} DIC = {DIC:f}\n".format(**dic))
    assert dic["PD"] > 0

    def rd(name):
        return nifti.read_nifti(tmp_path / f"{name}.nii.gz").data

    for p, nm in enumerate(st["names"]):
        assert np.array_equal(rd(f"spatCoef_{nm}"), maps["spatCoef"][p])
        assert np.array_equal(rd(f"spatCoef_{nm}.Var"), maps["spatCoef.Var"][p])
        assert np.array_equal(rd(f"standCoef_{nm}"), maps["standCoef"][p])
    for g in range(st["ntypes"]):
        assert np.array_equal(rd(f"prb_{st['names'][g]}"), maps["prb"][g])
    groups, total, total_p = driver.empirical_maps(st["mask"], st["covar"],
                                                   st["data"], st["ntypes"])
    for g in range(st["ntypes"]):
        assert np.array_equal(rd(f"empir_prb_{st['names'][g]}").ravel(), groups[g],
                              equal_nan=True)
    assert np.array_equal(rd("total_lesion_cnt").ravel(), total)
    assert np.array_equal(rd("total_empir_prb").ravel(), total_p)
    m = st["mask"].astype(bool)
    assert np.all(np.isfinite(rd(f"spatCoef_{st['names'][0]}")[m]))
    assert np.all(rd(f"spatCoef_{st['names'][0]}")[~m] == 0)


@pytest.mark.gpu
def test_driver_short_run_matches_oracle_chain(tmp_path, monkeypatch, oracle_mod):
    """MaxIter 3, BurnIn 0: SAVE_ITER = 3 keeps sweep 3 only, so spatCoef is
    the coefficient field after four sweeps; equal to the FP64 oracle chain
    on the same key within 1e-4."""
    monkeypatch.chdir(tmp_path)
    st = write_study(tmp_path, seed=9, N=17)
    assert driver.main([str(st["ntypes"]), str(st["P"]), "1", "design.txt", "1",
                        "0", "3", "0"]) == 0
    key = driver.chain_key([1, 2, 2])
    pb = oracle_mod.Problem(st["mask"], st["covar"], st["data"], st["ntypes"])
    o = pb.chain(key, 4, burnin=0, thin=3, df_offset=19)
    assert o["nkept"] == 1
    m = st["mask"].astype(bool)
    for p, nm in enumerate(st["names"]):
        got = nifti.read_nifti(tmp_path / f"spatCoef_{nm}.nii.gz").data[m]
        assert np.allclose(got, o["mean"][p], rtol=1e-4, atol=1e-4)
    for g in range(st["ntypes"]):
        got = nifti.read_nifti(tmp_path / f"prb_{st['names'][g]}.nii.gz").data[m]
        assert np.allclose(got, o["prb"][g], rtol=1e-4, atol=1e-4)


@pytest.mark.gpu
def test_driver_wm_run_equals_native_chain(tmp_path, monkeypatch):
    """With a WM image the run draws beta_WM every sweep and writes bWM, the
    kept-sweep mean of beta_WM WM_v; the maps equal the native chain's."""
    import bsglmm_gb300 as bsg
    monkeypatch.chdir(tmp_path)
    st = write_study(tmp_path, seed=13, N=26)
    X, Y, Z = st["dims"]
    rng = np.random.default_rng(14)
    wmvol = rng.integers(0, 256, (Z, Y, X)).astype(np.float64)
    nifti.write_nifti(tmp_path / "images" / "wm.nii.gz", wmvol, (X, Y, Z),
                      datatype=nifti.UINT8)
    assert driver.main([str(st["ntypes"]), str(st["P"]), "1", "design.txt", "1",
                        "wm.nii.gz", "300", "100"]) == 0
    m = st["mask"].astype(bool)
    wm = (wmvol[m].astype(np.float32) / np.float32(255))
    key = driver.chain_key([1, 2, 2])
    with bsg.Sampler() as s:
        ds = s.add_dataset(st["mask"], st["covar"], st["data"], st["ntypes"], wm)
        ch = s.add_chain(ds, seed=key, burnin=100, thin=200, df_offset=19)
        s.set_wm_update(ch, True)
        s.set_predictive(ch, True)
        s.run(301)
        maps = s.maps(ch)
        cur, mean = s.beta_wm(ch)
    for p, nm in enumerate(st["names"]):
        got = nifti.read_nifti(tmp_path / f"spatCoef_{nm}.nii.gz").data
        assert np.array_equal(got, maps["spatCoef"][p])
    bwm = nifti.read_nifti(tmp_path / "bWM.nii.gz").data
    assert np.array_equal(bwm[m], mean * wm.astype(np.float64))
    assert np.all(bwm[~m] == 0) and mean != 0.0
