"""TEST INFRASTRUCTURE ONLY: ctypes access to the oracle.

* ``Problem`` wraps liboracle.so, the FP64 C restatement of the reference's
  CPU sweep (bsg_oracle.c).
* ``RefSupplied`` / ``RefKiss`` wrap oracle/_ref/, the reference's own
  covar.cpp + cholesky.cpp (+ randgen.cpp) compiled from the reference tree,
  driven by supplied variates or by its own KISS generator.  These exist
  only where the reference tree was present at build time.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIBORACLE = HERE / "liboracle.so"
REF_SUPPLIED = HERE / "_ref" / "libbsgref_supplied.so"
REF_KISS = HERE / "_ref" / "libbsgref_kiss.so"

_P = C.c_void_p
_d = C.c_double
_i = C.c_int
_i64 = C.c_int64
_u32 = C.c_uint32


def reference_tree() -> Path:
    """The reference source tree the recipe compiles from: BSGLMM_REF if
    set, else the recipe's default (`make print-ref`)."""
    out = subprocess.run(["make", "-s", "-C", str(HERE), "print-ref"],
                         capture_output=True, text=True, check=True).stdout
    return Path(out.strip())


def build_oracle(ref: bool = False) -> None:
    """make liboracle.so (and, if requested and possible, oracle/_ref)."""
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", str(HERE), "ref"], check=True)


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


_O = None


def lib() -> C.CDLL:
    global _O
    if _O is None:
        if not LIBORACLE.exists():
            build_oracle()
        L = C.CDLL(str(LIBORACLE))
        sig = {
            "orc_philox4x32_10": (None, [_P, _P, _P]),
            "orc_philox_block": (None, [_u32, _u32, _u32, _u32, _u32, _i64, _P]),
            "orc_u_from_bits": (_d, [_u32]),
            "orc_ncdf": (_d, [_d]),
            "orc_ndtri": (_d, [_d]),
            "orc_normal_from_bits": (_d, [_u32]),
            "orc_tn_lower_inv": (_d, [_d, _u32]),
            "orc_tn_lower_tail": (_i, [_d, _P, _i, _P]),
            "orc_problem_new": (_P, [_i, _i, _i, _P, _i, _i, _i, _P, _P, _P]),
            "orc_problem_free": (None, [_P]),
            "orc_problem_info": (None, [_P, _P]),
            "orc_problem_lattice": (None, [_P, _P, _P, _P, _P, _P, _P]),
            "orc_problem_xtx": (None, [_P, _P]),
            "orc_update_z": (None, [_P, _d, _P, _P, _P]),
            "orc_update_spatcoef": (_i, [_P, _d, _P, _P, _P, _i, _P]),
            "orc_spatcoef_prec_S": (None, [_P, _P, _P]),
            "orc_wishart_from_S": (_i, [_i, _P, _P, _P, _P]),
            "orc_prob_sdnorm": (_d, [_d]),
            "orc_compute_prb": (None, [_P, _d, _P, _P]),
            "orc_col_means": (None, [_P, _P, _P]),
            "orc_loglik_as": (_d, [_d, _i]),
            "orc_predict": (None, [_P, _d, _P, _P, _i, _d]),
            "orc_dic_de": (_d, [_P, _P, _P, _i]),
            "orc_mix_gamma": (_d, [_d, _u32, _u32, _u32, _u32, _u32, _u32]),
            "orc_set_threads": (None, [_i]),
            "orc_chain_run": (_i, [_P, _P, _i64, _i64, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
            "orc_port_new": (_P, [_P, C.c_uint64, _i]),
            "orc_port_free": (None, [_P]),
            "orc_port_sweep": (None, [_P, _i]),
            "orc_port_updates": (_i64, [_P, _i]),
        }
        for k, (r, a) in sig.items():
            f = getattr(L, k)
            f.restype = r
            f.argtypes = a
        # the FP64 chain splits each colour's voxels over the host's cores
        L.orc_set_threads(min(os.cpu_count() or 1, 64))
        _O = L
    return _O


class ChainCfg(C.Structure):
    _fields_ = [("key0", C.c_uint32), ("key1", C.c_uint32), ("chain", C.c_uint32),
                ("df_offset", C.c_int32), ("burnin", C.c_int32), ("thin", C.c_int32),
                ("beta_wm", C.c_double), ("wm_update", C.c_int32),
                ("model", C.c_int32), ("t_df", C.c_double), ("inv_lf", C.c_double)]


def philox(ctr, key) -> np.ndarray:
    c = np.asarray(ctr, dtype=np.uint32)
    k = np.asarray(key, dtype=np.uint32)
    o = np.zeros(4, np.uint32)
    lib().orc_philox4x32_10(_p(c), _p(k), _p(o))
    return o


def philox_block(c1, c2, c3, key0, key1, n4) -> np.ndarray:
    o = np.zeros(4 * n4, np.uint32)
    lib().orc_philox_block(c1, c2, c3, key0, key1, n4, _p(o))
    return o


class Problem:
    """An oracle problem: lattice + design + outcomes (+ WM)."""

    def __init__(self, mask, covar, data, nsubtypes=1, wm=None):
        self._L = lib()
        self.mask = np.ascontiguousarray(mask, dtype=np.uint8)
        self.covar = np.ascontiguousarray(covar, dtype=np.float32)
        self.data = np.ascontiguousarray(data, dtype=np.uint8)
        self.wm = None if wm is None else np.ascontiguousarray(wm, dtype=np.float32)
        Z, Y, X = self.mask.shape
        P, N = self.covar.shape
        self.S = nsubtypes
        self.h = self._L.orc_problem_new(X, Y, Z, _p(self.mask), N, P, nsubtypes,
                                         _p(self.covar), _p(self.data), _p(self.wm))
        info = np.zeros(10, np.int64)
        self._L.orc_problem_info(self.h, _p(info))
        (self.X, self.Y, self.Z, self.nsize, self.V, self.Vp, self.n0, self.n1,
         self.N, self.P) = map(int, info)

    def __del__(self):
        if getattr(self, "h", None):
            self._L.orc_problem_free(self.h)
            self.h = None

    def lattice(self) -> dict:
        idx = np.zeros(self.nsize, np.int32)
        idxsc = np.zeros(self.nsize, np.int32)
        v0 = np.zeros(self.n0, np.int32)
        v1 = np.zeros(self.n1, np.int32)
        b0 = np.zeros(self.n0, np.uint8)
        b1 = np.zeros(self.n1, np.uint8)
        self._L.orc_problem_lattice(self.h, _p(idx), _p(idxsc), _p(v0), _p(v1),
                                    _p(b0), _p(b1))
        return dict(idx=idx, idxsc=idxsc, vox=[v0, v1], nbrs=[b0, b1])

    def xtx(self) -> np.ndarray:
        o = np.zeros((self.P, self.P), np.float32)
        self._L.orc_problem_xtx(self.h, _p(o))
        return o

    def update_z(self, spatcoef, ubits, beta_wm=0.0) -> np.ndarray:
        b = np.ascontiguousarray(spatcoef, dtype=np.float64)
        u = np.ascontiguousarray(ubits, dtype=np.uint32)
        Z = np.zeros((self.N, self.V))
        self._L.orc_update_z(self.h, beta_wm, _p(b), _p(u), _p(Z))
        return Z

    def update_spatcoef(self, spatcoef, Z, omega, normals, form=0, beta_wm=0.0):
        b = np.array(spatcoef, dtype=np.float64, order="C")
        z = np.ascontiguousarray(Z, dtype=np.float64)
        om = np.ascontiguousarray(omega, dtype=np.float64)
        e = np.ascontiguousarray(normals, dtype=np.float32)
        fails = self._L.orc_update_spatcoef(self.h, beta_wm, _p(z), _p(om), _p(e),
                                            form, _p(b))
        return b, fails

    def prec_S(self, spatcoef) -> np.ndarray:
        b = np.ascontiguousarray(spatcoef, dtype=np.float64)
        S = np.zeros((self.P, self.P))
        self._L.orc_spatcoef_prec_S(self.h, _p(b), _p(S))
        return S

    def wishart(self, S, chi2, wnorm):
        S = np.ascontiguousarray(S, dtype=np.float64)
        c = np.ascontiguousarray(chi2, dtype=np.float64)
        w = np.ascontiguousarray(wnorm, dtype=np.float64)
        om = np.zeros((self.P, self.P))
        ok = self._L.orc_wishart_from_S(self.P, _p(S), _p(c), _p(w), _p(om))
        return om, bool(ok)

    def compute_prb(self, spatcoef, beta_wm=0.0) -> np.ndarray:
        b = np.ascontiguousarray(spatcoef, dtype=np.float64)
        out = np.zeros((self.S, self.V))
        self._L.orc_compute_prb(self.h, beta_wm, _p(b), _p(out))
        return out

    def col_means(self, spatcoef) -> np.ndarray:
        b = np.ascontiguousarray(spatcoef, dtype=np.float64)
        out = np.zeros(self.P)
        self._L.orc_col_means(self.h, _p(b), _p(out))
        return out

    def predict(self, spatcoef, beta_wm=0.0, model: int = 1) -> np.ndarray:
        """Mpredict [N][S] of compute_predictGPU (covarGPU.cu:1866-1903)."""
        b = np.ascontiguousarray(spatcoef, dtype=np.float64)
        out = np.zeros((self.N, self.S))
        inv_lf = 1.0 / 0.634 if model == 0 else 1.0
        self._L.orc_predict(self.h, beta_wm, _p(b), _p(out), model, inv_lf)
        return out

    def dic_de(self, mean, mwm=None, model: int = 1) -> float:
        """DE of compute_prb_DIC (covar.cpp:442-486) at the posterior means
        mean [P][V] and mwm [V] (None = 0)."""
        m = np.ascontiguousarray(mean, dtype=np.float64)
        w = None if mwm is None else np.ascontiguousarray(mwm, dtype=np.float64)
        return self._L.orc_dic_de(self.h, _p(m), _p(w), model)

    def sweep_supplied(self, spatcoef, omega, ubits, normals, chi2, wnorm,
                       form=0, beta_wm=0.0):
        """One full sweep (Z, beta both colours, Omega) from supplied
        variates, in the reference's order; returns (beta, omega, Z)."""
        Z = self.update_z(spatcoef, ubits, beta_wm)
        b, fails = self.update_spatcoef(spatcoef, Z, omega, normals, form, beta_wm)
        S = self.prec_S(b)
        om, ok = self.wishart(S, chi2, wnorm)
        return b, om, Z, S, fails, ok

    def chain(self, seed: int, nsweeps: int, chain_id: int = 0, burnin: int = 0,
              thin: int = 1, df_offset=None, beta_wm=0.0, s0: int = 0,
              spatcoef=None, omega=None, wm_update: bool = False, model: int = 1,
              phi=None):
        """FP64 chain on the sampler's counters.  Returns the state (beta,
        omega, beta_wm, phi) and the posterior summaries of the kept sweeps.
        model: the reference's MODEL (1 probit, 0 logistic, 2 t)."""
        t_df, inv_lf = {0: (8.0, 1.0 / 0.634), 1: (1000.0, 1.0), 2: (3.0, 1.0)}[model]
        cfg = ChainCfg(seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF, chain_id,
                       self.P if df_offset is None else df_offset, burnin, thin,
                       beta_wm, int(bool(wm_update)), model, t_df, inv_lf)
        ph = None
        if model != 1:
            ph = (np.ones((self.N, self.V)) if phi is None
                  else np.array(phi, dtype=np.float64, order="C"))
        bw = C.c_double(beta_wm)
        wsum = C.c_double(0.0)
        b = (np.zeros((self.P, self.Vp)) if spatcoef is None
             else np.array(spatcoef, dtype=np.float64, order="C"))
        om = np.eye(self.P) if omega is None else np.array(omega, dtype=np.float64, order="C")
        s1 = np.zeros((self.P, self.V))
        s2 = np.zeros((self.P, self.V))
        sp = np.zeros((max(self.S, 1), self.V))
        nk = C.c_int64(0)
        err = self._L.orc_chain_run(self.h, C.byref(cfg), s0, nsweeps, _p(b), _p(om),
                                    _p(s1), _p(s2), _p(sp), C.byref(nk), C.byref(bw),
                                    C.byref(wsum), _p(ph))
        T = nk.value
        with np.errstate(invalid="ignore", divide="ignore"):
            mean = s1 / T
            var = (s2 - T * mean * mean) / (T - 1)
            prb = sp[: self.S] / T
            wm_mean = wsum.value / T if T else float("nan")
        return dict(beta=b, omega=om, mean=mean, var=var, prb=prb,
                    sum=s1, sumsq=s2, nkept=T, err=err, beta_wm=bw.value,
                    wm_sum=wsum.value, wm_mean=wm_mean, phi=ph)


def subtypes(covar, S: int) -> np.ndarray:
    """compute_predictGPU's group of each subject (covarGPU.cu:1929-1935):
    the first of the S group columns that is nonzero, else 0."""
    c = np.asarray(covar)[:S] != 0
    return np.where(c.any(0), np.argmax(c, axis=0), 0)


def qhat_update(qhat, mpredict, sub, first: bool) -> None:
    """The host part of compute_predictGPU (covarGPU.cu:1937-1953), in place:
    d = Mpredict[i][g] - Mpredict[i][sub_i]; on the first kept sweep
    Qhat[i][0] = d_0 and Qhat[i][g] = log(exp(Qhat) + exp(d_g)) for g >= 1
    (Qhat starts at 0, mcmc.cpp:223-225); afterwards the log-sum for all g."""
    mp = np.asarray(mpredict, dtype=np.float64)
    n = mp.shape[0]
    d = mp - mp[np.arange(n), np.asarray(sub)][:, None]
    for i in range(n):
        for g in range(mp.shape[1]):
            if first and g == 0:
                qhat[i, 0] = d[i, 0]
                continue
            m = max(d[i, g], qhat[i, g])
            qhat[i, g] = np.log(np.exp(qhat[i, g] - m) + np.exp(d[i, g] - m)) + m


class Port:
    """The CPU timing port of the reference sweep (float, KISS)."""

    def __init__(self, problem: Problem, seed: int = 1, df_offset=None):
        self._L = lib()
        self.pb = problem
        self.h = self._L.orc_port_new(problem.h, seed,
                                      problem.P if df_offset is None else df_offset)

    def sweep(self, nvox_limit: int = -1):
        self._L.orc_port_sweep(self.h, nvox_limit)

    def updates(self, nvox_limit: int = -1) -> int:
        return int(self._L.orc_port_updates(self.h, nvox_limit))

    def __del__(self):
        if getattr(self, "h", None):
            self._L.orc_port_free(self.h)
            self.h = None


# ------------------------------------------------- the reference itself --
class _Ref:
    path: Path

    def __init__(self, problem: Problem):
        if not self.path.exists():
            raise FileNotFoundError(f"{self.path} (build with `make -C oracle ref`)")
        self._L = C.CDLL(str(self.path))
        self.pb = problem
        lat = problem.lattice()
        self._keep = lat
        L = self._L
        L.ref_setup.argtypes = [_i] * 8 + [_P, _P, _i, _P, _P, _i, _P, _P, _P]
        L.ref_setup(problem.X, problem.Y, problem.Z, problem.N, problem.P,
                    problem.S, problem.V, problem.Vp, _p(lat["idx"]),
                    _p(lat["idxsc"]), problem.n0, _p(lat["vox"][0]),
                    _p(lat["nbrs"][0]), problem.n1, _p(lat["vox"][1]),
                    _p(lat["nbrs"][1]), _p(problem.covar))
        self.wm = (problem.wm if problem.wm is not None
                   else np.ones(problem.V, np.float32))
        for n, a in {"ref_update_z": [_P, _P, _P, C.c_float, _P, _P],
                     "ref_update_spatcoef": [_P, _P, _P, _P, C.c_float, _P],
                     "ref_update_spatcoef_prec": [_P, _P],
                     "ref_compute_prb": [_P, _P, _P, C.c_float],
                     "ref_xtx": [_P],
                     "ref_cholesky_decomp": [_P, _i],
                     "ref_cholesky_invert": [_P, _i]}.items():
            getattr(L, n).argtypes = a
        L.ref_prob_sdnorm.argtypes = [_d]
        L.ref_prob_sdnorm.restype = _d
        L.ref_compute_prb_dic.argtypes = [_P, _P, _P, _P]
        L.ref_set_model.argtypes = [_i]
        L.ref_compute_prb_dic.restype = _d
        L.ref_cholesky_decomp.restype = _i

    def xtx(self):
        o = np.zeros((self.pb.P, self.pb.P), np.float32)
        self._L.ref_xtx(_p(o))
        return o

    def update_z(self, spatcoef_f32, beta=0.0):
        Z = np.zeros((self.pb.N, self.pb.V), np.float32)
        b = np.ascontiguousarray(spatcoef_f32, dtype=np.float32)
        self._L.ref_update_z(_p(Z), _p(self.pb.data), _p(self.wm), beta, _p(b),
                             _p(self.pb.covar))
        return Z

    def update_spatcoef(self, spatcoef_f32, Z, omega_f32, beta=0.0):
        b = np.array(spatcoef_f32, dtype=np.float32, order="C")
        z = np.ascontiguousarray(Z, dtype=np.float32)
        om = np.array(omega_f32, dtype=np.float32, order="C")
        self._L.ref_update_spatcoef(_p(b), _p(z), _p(om), _p(self.wm), beta,
                                    _p(self.pb.covar))
        return b

    def update_spatcoef_prec(self, spatcoef_f32):
        om = np.zeros((self.pb.P, self.pb.P), np.float32)
        b = np.ascontiguousarray(spatcoef_f32, dtype=np.float32)
        self._L.ref_update_spatcoef_prec(_p(om), _p(b))
        return om

    def compute_prb(self, spatcoef_f32, beta=0.0):
        out = np.zeros((self.pb.S, self.pb.V), np.float32)
        b = np.ascontiguousarray(spatcoef_f32, dtype=np.float32)
        self._L.ref_compute_prb(_p(out), _p(b), _p(self.wm), beta)
        return out

    def prob_sdnorm(self, x: float) -> float:
        return self._L.ref_prob_sdnorm(x)

    def compute_prb_dic(self, mean, mwm=None, model: int = 1) -> float:
        """The reference's compute_prb_DIC on posterior means [P][V]."""
        self._L.ref_set_model(model)
        pb = self.pb
        R = pb.X * pb.Y * pb.Z
        lat = self._keep
        inmask = lat["idx"] >= 0
        # unpadded grid index of each compact voxel v
        pad = np.nonzero(inmask)[0]
        i = pad % (pb.X + 2) - 1
        j = (pad // (pb.X + 2)) % (pb.Y + 2) - 1
        k = pad // ((pb.X + 2) * (pb.Y + 2)) - 1
        grid = i + pb.X * j + pb.X * pb.Y * k
        v = lat["idx"][pad]
        mc = np.zeros((pb.P, R))
        mc[:, grid] = np.asarray(mean, dtype=np.float64)[:, v]
        mw = np.zeros(R)
        if mwm is not None:
            mw[grid] = np.asarray(mwm, dtype=np.float64)[v]
        return self._L.ref_compute_prb_dic(_p(mc), _p(mw), _p(pb.covar),
                                           _p(pb.data))


class RefSupplied(_Ref):
    path = REF_SUPPLIED

    def __init__(self, problem: Problem):
        super().__init__(problem)
        L = self._L
        L.ref_set_supplied.argtypes = [_P, _P, _P, _P]
        L.ref_underrun.restype = _i
        L.ref_gamma_shapes.argtypes = [_P, _i]
        L.ref_gamma_shapes.restype = _i
        L.ref_rwishart2.argtypes = [_P, _P, _i, _i, _P, _P]
        L.ref_rwishart2.restype = _i

    def set_supplied(self, ubits, normals, chi2, wnorm):
        self._sup = [np.ascontiguousarray(ubits, dtype=np.uint32),
                     np.ascontiguousarray(normals, dtype=np.float32),
                     np.ascontiguousarray(chi2, dtype=np.float64),
                     np.ascontiguousarray(wnorm if np.size(wnorm) else [0.0],
                                          dtype=np.float64)]
        self._L.ref_set_supplied(*[_p(a) for a in self._sup])

    def underrun(self) -> bool:
        return bool(self._L.ref_underrun())

    def gamma_shapes(self):
        o = np.zeros(64)
        n = self._L.ref_gamma_shapes(_p(o), 64)
        return o[:n]

    def sweep(self, spatcoef_f32, omega_f32, beta=0.0):
        """updateZ -> updateSpatCoef -> updateSpatCoefPrec
        (mcmc.cpp:400,418,428) on the supplied variates."""
        Z = self.update_z(spatcoef_f32, beta)
        b = self.update_spatcoef(spatcoef_f32, Z, omega_f32, beta)
        om = self.update_spatcoef_prec(b)
        return b, om, Z


class RefKiss(_Ref):
    path = REF_KISS

    def __init__(self, problem: Problem, seed=(1, 2, 3)):
        super().__init__(problem)
        L = self._L
        L.ref_kiss_seed.argtypes = [C.c_uint64] * 3
        L.ref_truncnorm_many.argtypes = [_d, _d, _d, _i, _P]
        L.ref_snorm_many.argtypes = [_i, _P]
        L.ref_rgamma_many.argtypes = [_d, _d, _i, _P]
        L.ref_cpu_sweep.argtypes = [_P, _P, _P, _P, _P, _P]
        L.ref_kiss_many.argtypes = [_i, _P, _P]
        L.ref_write_nifti.argtypes = [_i, _i, _i, C.c_char_p, _P]
        L.ref_kiss_seed(*seed)

    def write_nifti(self, path, data_zyx):
        """The reference's .nii writer on a [Z][Y][X] volume."""
        d = np.ascontiguousarray(data_zyx, dtype=np.float64)
        Z, Y, X = d.shape
        return self._L.ref_write_nifti(X, Y, Z, str(path).encode(), _p(d))

    def kiss(self, n):
        """n raw KISS draws and the generator state after them."""
        out = np.zeros(n)
        state = np.zeros(3, np.uint64)
        self._L.ref_kiss_many(n, _p(out), _p(state))
        return out, [int(x) for x in state]

    def truncnorm(self, mu, lo, hi, n):
        out = np.zeros(n)
        self._L.ref_truncnorm_many(mu, lo, hi, n, _p(out))
        return out

    def snorm(self, n):
        out = np.zeros(n)
        self._L.ref_snorm_many(n, _p(out))
        return out

    def rgamma(self, a, b, n):
        out = np.zeros(n)
        self._L.ref_rgamma_many(a, b, n, _p(out))
        return out


# ------------------------------------------- the reference's GPU sweep ---
LIBREFGPU = HERE / "librefgpu.so"
REF_PTX = HERE / "_ref" / "covarGPU.ptx"


def refgpu_available() -> bool:
    """The reference's covarGPU.cu compiled to PTX (made where the
    reference tree is mounted; the file travels with the repository copy)
    and the host harness that drives it."""
    return REF_PTX.exists() and LIBREFGPU.exists()


class RefGpu:
    """The reference's own GPU kernels (Z_GPU1, Spat_Coef_Probit, reduce,
    Spat_Coef_Prec from covarGPU.cu, JIT-loaded from PTX) driven as its
    launchers do (refgpu_harness.cu).  One study per process."""

    def __init__(self, pb: Problem, device: int = 0, seed: int = 1):
        L = C.CDLL(str(LIBREFGPU))
        L.rg_error.restype = C.c_char_p
        L.rg_open.argtypes = [C.c_char_p, _i]
        L.rg_setup.argtypes = [_i, _i, _i, _i, _i, _i, _i, _P, _P, _i, _P, _P, _i, _P,
                               _P, _P, _P, _P, C.c_uint64]
        L.rg_sweeps.argtypes = [_i, _P]
        L.rg_set_model.argtypes = [_i]
        L.rg_get_beta.argtypes = [_P]
        L.rg_get_omega.argtypes = [_P]
        self._L = L
        self.pb = pb
        if L.rg_open(str(REF_PTX).encode(), device):
            raise RuntimeError(L.rg_error().decode())
        lat = pb.lattice()
        self._keep = [np.ascontiguousarray(a) for a in (
            lat["idx"], lat["idxsc"], lat["vox"][0], lat["nbrs"][0], lat["vox"][1],
            lat["nbrs"][1], pb.covar, pb.data, pb.xtx())]
        k = self._keep
        if L.rg_setup(pb.X, pb.Y, pb.Z, pb.N, pb.P, pb.V, pb.Vp, _p(k[0]), _p(k[1]),
                      pb.n0, _p(k[2]), _p(k[3]), pb.n1, _p(k[4]), _p(k[5]), _p(k[6]),
                      _p(k[7]), _p(k[8]), seed):
            raise RuntimeError(L.rg_error().decode())

    def set_model(self, model: int):
        """The reference's MODEL: 1 probit, 0 logistic, 2 t."""
        if self._L.rg_set_model(int(model)):
            raise RuntimeError(self._L.rg_error().decode())

    def sweeps(self, n: int) -> float:
        """Runs n sweeps; returns milliseconds per sweep."""
        ms = C.c_double()
        if self._L.rg_sweeps(n, C.byref(ms)):
            raise RuntimeError(self._L.rg_error().decode())
        return ms.value

    def beta(self) -> np.ndarray:
        out = np.zeros((self.pb.P, self.pb.Vp), np.float32)
        self._L.rg_get_beta(_p(out))
        return out

    def omega(self) -> np.ndarray:
        out = np.zeros((self.pb.P, self.pb.P), np.float32)
        self._L.rg_get_omega(_p(out))
        return out

    def close(self):
        self._L.rg_close()
