"""BinCar-compatible driver on the GB300 sampler.

    python -m bsglmm_gb300.driver NTypes NCov GPU Design Mask WM [MaxIter BurnIn]

Same arguments, inputs and outputs as the reference program (main.cu:82-116,
read_data.cpp:187-545, mcmc.cpp:795-964):

* Mask: a FLOAT64 NIfTI-1 image in ./images (or "1" for images/mask.nii.gz);
  voxels whose value casts to a nonzero byte are in the mask.
* Design: whitespace-separated text; a header row of NCov+2 tokens (an id
  column, the NCov covariate names, the image column), then one row per
  subject: id, NCov covariates, lesion-map file name relative to ./images.
  The first NTypes covariates are the group columns.
* Lesion maps: FLOAT32 or FLOAT64 NIfTI-1, binary.
* WM: "0" for none, "1" for images/avg152T1_white.nii.gz, else a UINT8
  NIfTI-1 image in ./images; WM_v = value / 255 (read_data.cpp:489-545) and
  the white-matter coefficient beta_WM is drawn every sweep.
* seed.dat: three integers (KISS state); rewritten at exit.
* Every segment of up to 100 sweeps prints one JSON line on stderr: the sweep
  range, device milliseconds per sweep and subject-voxel updates/s.
* Outputs (FLOAT64 NIfTI-1, gzipped in process): empir_prb_<group>,
  total_lesion_cnt, total_empir_prb, spatCoef_<cov>, spatCoef_<cov>.Var,
  standCoef_<cov>, prb_<group>; text: Qhat.dat, Qhat2.dat (mcmc.cpp:719-786)
  and DIC.dat (mcmc.cpp:966-975), from the predictive pass that runs after
  every kept sweep; bWM (mcmc.cpp:830-837) with a WM image.

The chain runs MaxIter+1 sweeps with the reference's burn-in and SAVE_ITER
rule (mcmc.cpp:303-308) and the reference GPU path's Wishart df (V + 19,
covarGPU.cu:1104).  GPU = 1 only.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

from . import nifti
from ._lib import BsgError
from .sampler import Sampler, save_iter_rule

IMAGE_DIR = Path("./images")
DEFAULT_MASK = "mask.nii.gz"
DEFAULT_WM = "avg152T1_white.nii.gz"
PRINT_EVERY = 100  # mcmc.cpp:309

USAGE = """Usage: bsglmm  NTypes  NCov  GPU  Design Mask WM [MaxIter BurnIn]
  NTypes  - Number of groups
  NCov    - Number of covariates (count must include groups)
  GPU     - 1 use GPU (this build has no CPU path)
  Design  - Text file, tab or space separated data file
  Mask    - Filename of mask image in './images' directory, or '1' to use default (mask.nii.gz)
  WM      - Filename of WM image in './images' directory, '0' to use none, or '1' to use default (avg152T1_white.nii.gz)
  MaxIter - Number of iterations (defaults to 100,000)
  BurnIn  - Number of burn-in iterations (defaults to 50,000)"""


class DriverError(RuntimeError):
    pass


def _as_byte(v: np.ndarray) -> np.ndarray:
    """C's (unsigned char) conversion of a double (read_data.cpp:235,385)."""
    t = np.trunc(np.nan_to_num(v, nan=0.0, posinf=0.0, neginf=0.0))
    return np.mod(t.astype(np.int64), 256).astype(np.uint8)


def read_mask(path: Path) -> np.ndarray:
    img = nifti.read_nifti(path)
    if img.datatype != nifti.FLOAT64:
        raise DriverError(f"Incorrect data type in file: {img.datatype}\n"
                          "Must be float (NIFTI_TYPE_FLOAT64)")
    return (_as_byte(img.data) != 0).astype(np.uint8)


def read_wm(path: Path, mask: np.ndarray) -> np.ndarray:
    """read_nifti1_WM (read_data.cpp:489-545): a UINT8 image; WM_v = value /
    255 over in-mask voxels in file order."""
    img = nifti.read_nifti(path)
    if img.datatype != nifti.UINT8:
        raise DriverError(f"Incorrect data type in file: {img.datatype}\n"
                          "Must be unsigned char (NIFTI_TYPE_UINT8)")
    if img.data.shape != mask.shape:
        raise DriverError(f"{path}: dimensions {img.dims} differ from the mask's")
    return (img.data[mask.astype(bool)].astype(np.float32) / np.float32(255.0))


def read_design(path: Path, ncov: int, ntypes: int):
    """read_data.cpp:262-320: header of NCov+2 tokens, then rows."""
    tokens = Path(path).read_text().split()
    width = ncov + 2
    if len(tokens) < width:
        raise DriverError(f"{path}: header needs {width} tokens")
    names = tokens[1:ncov + 1]
    body = tokens[width:]
    nsubs = len(body) // width
    if nsubs == 0 or len(body) % width:
        raise DriverError(f"{path}: {len(body)} tokens after the header is not a "
                          f"multiple of NCov+2 = {width}")
    rows = [body[i * width:(i + 1) * width] for i in range(nsubs)]
    try:
        covar = np.array([[float(r[1 + p]) for r in rows] for p in range(ncov)],
                         dtype=np.float32)
    except ValueError as e:
        raise DriverError(f"{path}: non-numeric covariate ({e})") from None
    images = [IMAGE_DIR / r[ncov + 1] for r in rows]
    return names, covar, images


def read_lesions(images, mask: np.ndarray) -> np.ndarray:
    """data[i, v] over in-mask voxels in file order (read_data.cpp:341-406)."""
    m = mask.astype(bool)
    out = np.zeros((len(images), int(m.sum())), dtype=np.uint8)
    sys.stderr.write("Loading images: ")
    for i, p in enumerate(images):
        img = nifti.read_nifti(p)
        if img.datatype not in (nifti.FLOAT32, nifti.FLOAT64):
            raise DriverError(f"Incorrect data type in file {p}: {img.datatype}\n"
                              "Must be float (NIFTI_TYPE_FLOAT32) or double "
                              "(NIFTI_TYPE_FLOAT64)")
        if img.data.shape != mask.shape:
            raise DriverError(f"{p}: dimensions {img.dims} differ from the mask's")
        out[i] = _as_byte(img.data[m])
        sys.stderr.write(".")
    sys.stderr.write("\n")
    return out


def empirical_maps(mask, covar, data, ntypes):
    """write_empir_prb (read_data.cpp:418-487): per group the mean lesion
    frequency of its members, the summed group counts, and that sum / N."""
    m = mask.astype(bool).ravel()
    R = m.size
    N = data.shape[0]
    sum2 = np.zeros(R)
    groups = []
    for g in range(ntypes):
        members = covar[g] != 0
        cnt = data[members].sum(0).astype(np.float64)
        full = np.zeros(R)
        with np.errstate(invalid="ignore", divide="ignore"):
            full[m] = cnt / members.sum()
        sum2[m] += cnt
        groups.append(full)
    return groups, sum2, sum2 / N


def read_seed(path=Path("seed.dat")):
    if path.exists():
        vals = [int(x) for x in path.read_text().split()[:3]]
        if len(vals) == 3:
            return vals
        raise DriverError("seed.dat must hold three integers")
    print("No seed.dat found; using [ 1 2 3 ]")
    return [1, 2, 2]  # main.cu:157-158


def kiss(s):
    """KISS step of randgen.cpp:9-23 (64-bit words, 2^-64 scale)."""
    m = (1 << 64) - 1
    s[1] = (s[1] ^ (s[1] << 17)) & m
    s[2] = (s[2] ^ (s[2] << 18)) & 0x7FFFFFFF
    s[0] = (69069 * s[0] + 23606797) & m
    s[1] ^= s[1] >> 15
    s[2] ^= s[2] >> 13
    return float((s[0] + s[1] + s[2]) & m) * 5.421010862427522e-20


def chain_key(seed):
    """64-bit Philox key from two draws of the KISS stream (the stream
    advances, so seed.dat changes from run to run as in the reference)."""
    hi = int(kiss(seed) * 4294967296.0)
    lo = int(kiss(seed) * 4294967296.0)
    return ((hi << 32) ^ lo) & ((1 << 64) - 1)


def qhat_lines(qhat, covar, ntypes, prior=None):
    """Rows of Qhat.dat / Qhat2.dat (mcmc.cpp:719-786): subject, the
    normalised exp(Qhat), the predicted group (last maximum) and the true
    group (first nonzero group column, else 0).  With `prior`, Qhat is first
    multiplied by it column-wise, as Qhat2.dat does."""
    q = np.array(qhat, dtype=np.float64)
    if prior is not None:
        q = q * np.asarray(prior, dtype=np.float64)[None, :]
    lines = []
    for i in range(q.shape[0]):
        mx = -np.finfo(np.float64).max
        for g in range(ntypes):
            mx = max(mx, q[i, g])
        qh = np.log(np.sum(np.exp(q[i, :ntypes] - mx))) + mx
        row = f"{i} " + "".join(f"{np.exp(q[i, g] - qh):.6f} " for g in range(ntypes))
        mx, pred = -np.finfo(np.float64).max, -1
        for g in range(ntypes):
            if mx <= q[i, g]:
                mx, pred = q[i, g], g
        true = 0
        for g in range(ntypes):
            if covar[g, i] != 0:
                true = g
                break
        lines.append(row + f"{pred} {true}\n")
    return "".join(lines)


def group_prior(covar, ntypes):
    """grp_prior of read_data.cpp:287-316: the integer part of each group
    column summed over subjects, divided by N."""
    return np.trunc(covar[:ntypes].astype(np.float64)).sum(1) / covar.shape[1]


def _print_state(it, omega, colmean, ntypes):
    """The periodic summary of mcmc.cpp:535-583."""
    V = np.linalg.inv(omega)
    sd = np.sqrt(np.diag(V))
    print(f"iter = {it}\t")
    print("  overall mean and SD for groups ")
    for i in range(ntypes):
        print(f"\t {colmean[i]:10.6f} {sd[i]:10.6f}")
    print("\n  overall mean and SD for spatially varying coefficients for all covariates ")
    for i in range(ntypes, len(sd)):
        print(f"\t {colmean[i]:10.6f} {sd[i]:10.6f}")
    print("\n  correlation matrix of regression parameters ")
    for i in range(len(sd)):
        print("".join(f"   {V[i, j] / (sd[i] * sd[j]):6.3f} " for j in range(i + 1)))
    print(flush=True)


def run(ntypes, ncov, design, mask_name, maxiter, burnin, outdir=Path("."),
        device=0, quiet=False, wm_name=None):
    outdir = Path(outdir)
    mask = read_mask(IMAGE_DIR / mask_name)
    wm = read_wm(IMAGE_DIR / wm_name, mask) if wm_name else None
    names, covar, images = read_design(design, ncov, ntypes)
    if ntypes > ncov:
        raise DriverError("NTypes cannot exceed NCov")
    data = read_lesions(images, mask)
    if data.max(initial=0) > 1:
        raise DriverError("lesion maps must be binary (0/1)")
    Z, Y, X = mask.shape
    dims = (X, Y, Z)
    groups, total, total_p = empirical_maps(mask, covar, data, ntypes)
    for g in range(ntypes):
        nifti.write_nifti(outdir / f"empir_prb_{names[g]}.nii.gz", groups[g], dims)
    nifti.write_nifti(outdir / "total_lesion_cnt.nii.gz", total, dims)
    nifti.write_nifti(outdir / "total_empir_prb.nii.gz", total_p, dims)

    seed = read_seed(Path("seed.dat"))
    key = chain_key(seed)
    with Sampler(device) as s:
        ds = s.add_dataset(mask, covar, data, ntypes, wm)
        ch = s.add_chain(ds, seed=key, burnin=burnin,
                         thin=save_iter_rule(maxiter, burnin), df_offset=19)
        if wm is not None:
            s.set_wm_update(ch, True)
        if ntypes >= 1:
            s.set_predictive(ch, True)
        done = 0
        while done <= maxiter:
            step = min(PRINT_EVERY, maxiter + 1 - done)
            if not quiet and done % PRINT_EVERY == 0:
                _print_state(done, s.omega(ch), s.colmeans(ch), ntypes)
            ms = s.run_timed(step)
            s.sync()
            # one machine-readable line per segment on stderr
            sys.stderr.write(json.dumps({
                "sweeps": [done, done + step - 1], "ms_per_sweep": ms / step,
                "updates_per_s": data.shape[0] * data.shape[1] * step / max(ms * 1e-3, 1e-300),
                "status": 0}) + "\n")
            done += step
        maps = s.maps(ch)
        totsav = s.sweep_count(ch)[1]
        qhat, _, npred = s.predictive(ch) if ntypes >= 1 else (None, 0.0, 0)
        bwm_mean = s.beta_wm(ch)[1]
        dic = s.dic(ch) if npred > 0 else dict.fromkeys(("DE", "ED", "PD", "DIC"), float("nan"))
    print(f"TOTSAV = {totsav}")
    if qhat is not None:
        (outdir / "Qhat.dat").write_text(qhat_lines(qhat, covar, ntypes))
        (outdir / "Qhat2.dat").write_text(
            qhat_lines(qhat, covar, ntypes, group_prior(covar, ntypes)))
    for p, nm in enumerate(names):
        nifti.write_nifti(outdir / f"spatCoef_{nm}.nii.gz", maps["spatCoef"][p], dims)
        nifti.write_nifti(outdir / f"spatCoef_{nm}.Var.nii.gz", maps["spatCoef.Var"][p], dims)
        nifti.write_nifti(outdir / f"standCoef_{nm}.nii.gz", maps["standCoef"][p], dims)
    for g in range(ntypes):
        nifti.write_nifti(outdir / f"prb_{names[g]}.nii.gz", maps["prb"][g], dims)
    if wm is not None:  # mean over kept sweeps of beta_WM WM_v (mcmc.cpp:636,799)
        bwm = np.zeros(mask.shape)
        bwm[mask.astype(bool)] = bwm_mean * wm.astype(np.float64)
        nifti.write_nifti(outdir / "bWM.nii.gz", bwm, dims)
    line = "DE = {DE:f} ED = {ED:f} PD = {PD:f} DIC = {DIC:f}".format(**dic)
    print(line)
    (outdir / "DIC.dat").write_text(line + "\n")
    Path("seed.dat").write_text(f"{seed[0]} {seed[1]} {seed[2]}\n")  # main.cu:430-432
    return maps, totsav


def main(argv=None) -> int:
    argv = sys.argv[1:] if argv is None else list(argv)
    if len(argv) not in (6, 8):
        print(USAGE)
        return 1
    try:
        ntypes, ncov, gpu = int(argv[0]), int(argv[1]), int(argv[2])
    except ValueError:
        print(USAGE)
        return 1
    design, mask_arg, wm_arg = argv[3], argv[4], argv[5]
    maxiter, burnin = 100000, 50000
    if len(argv) == 8:
        maxiter, burnin = int(argv[6]), int(argv[7])
        if maxiter < 1000:
            print("WARNING: Silly-small number of iterations used; recommend abort and use more")
        if burnin > maxiter:
            print("WARNING: Burn-in exceeds MAXITER, no results will be saved")
    try:
        if gpu != 1:
            raise DriverError("GPU = 0 (the reference's untested CPU path) is not provided")
        mask_name = DEFAULT_MASK if mask_arg == "1" else mask_arg
        wm_name = None if wm_arg == "0" else (DEFAULT_WM if wm_arg == "1" else wm_arg)
        run(ntypes, ncov, design, mask_name, maxiter, burnin, wm_name=wm_name)
    except (DriverError, nifti.NiftiError) as e:
        print(f"Error: {e}", file=sys.stderr)
        return 2
    except BsgError as e:
        print(f"Error: {e}", file=sys.stderr)
        return 3
    return 0


if __name__ == "__main__":
    sys.exit(main())
