"""Host-side interface of the GB300 sampler, mirroring the reference's
driver: ``mcmc()`` (mcmc.cpp:76) runs MAXITER+1 sweeps with the reference's
burn-in / thinning rule and returns its output maps; ``Sampler`` exposes the
per-sweep update (updateZ + updateSpatCoef + updateSpatCoefPrec, fused on
the device) and the state for tests.

Everything runs through libbsglmm_gb300.so (C ABI); numpy arrays are only
host buffers.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import BsgError, ChainDesc, DatasetDesc


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def save_iter_rule(maxiter: int, burnin: int) -> int:
    """SAVE_ITER of mcmc.cpp:303-308."""
    if maxiter - burnin < 10000:
        return max(1, maxiter - burnin)
    return (maxiter - burnin) // 10000


class Sampler:
    """One device context holding studies (datasets) and chains."""

    def __init__(self, device: int = 0):
        self._L = _lib.lib()
        h = C.c_void_p()
        self._check(self._L.bsg_create(device, C.byref(h)), "bsg_create", None)
        self._h = h
        self._ds = []   # per dataset: info dict
        self._ch = []   # per chain: dataset id

    # ------------------------------------------------------------ basics --
    def _check(self, st: int, where: str, h=...):
        if st != _lib.BSG_OK:
            hh = self._h if h is ... else h
            detail = self._L.bsg_last_error(hh).decode() if hh else ""
            raise BsgError(st, where, detail)

    def close(self):
        if getattr(self, "_h", None):
            self._L.bsg_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------ setup ---
    def add_dataset(self, mask, covar, data, nsubtypes: int = 1, wm=None) -> int:
        mask = np.ascontiguousarray(mask, dtype=np.uint8)
        covar = np.ascontiguousarray(covar, dtype=np.float32)
        data = np.ascontiguousarray(data, dtype=np.uint8)
        wm = None if wm is None else np.ascontiguousarray(wm, dtype=np.float32)
        Z, Y, X = mask.shape
        P, N = covar.shape
        d = DatasetDesc(X, Y, Z, N, P, nsubtypes, _ptr(mask), _ptr(covar),
                        _ptr(data), _ptr(wm))
        out = C.c_int32()
        self._check(self._L.bsg_add_dataset(self._h, C.byref(d), C.byref(out)),
                    "bsg_add_dataset")
        info = np.zeros(11, np.int64)
        self._check(self._L.bsg_dataset_info(self._h, out.value, _ptr(info)),
                    "bsg_dataset_info")
        keys = ["X", "Y", "Z", "nsize", "V", "Vp", "n0", "n1", "N", "P", "S"]
        self._ds.append(dict(zip(keys, map(int, info))))
        return out.value

    def add_chain(self, dataset: int, seed: int = 1, burnin: int = 0,
                  thin: int = 1, df_offset: int | None = None,
                  beta_wm: float = 0.0) -> int:
        """df_offset None = the reference CPU path's df = V + P
        (covar.cpp:291); the reference GPU path uses 19 (covarGPU.cu:1104)."""
        P = self._ds[dataset]["P"]
        desc = ChainDesc(seed, P if df_offset is None else df_offset, burnin,
                         thin, beta_wm)
        out = C.c_int32()
        self._check(self._L.bsg_add_chain(self._h, dataset, C.byref(desc),
                                          C.byref(out)), "bsg_add_chain")
        self._ch.append(dataset)
        return out.value

    def set_tuning(self, lanes_per_voxel: int = 0, block_threads: int = 0):
        self._check(self._L.bsg_set_tuning(self._h, lanes_per_voxel,
                                           block_threads), "bsg_set_tuning")

    def set_tensor_xz(self, enable: bool = True):
        """X'Z of the probit colour kernel on the tensor cores (BF16x3
        split product) instead of f32x2 FMAs."""
        self._check(self._L.bsg_set_tensor_xz(self._h, int(bool(enable))),
                    "bsg_set_tensor_xz")

    def set_step_subjects(self, subjects: int = 0):
        """Subjects per whole-word step of the probit colour kernel: 8, 16,
        or 0 to choose per P group (identical results either way)."""
        self._check(self._L.bsg_set_step_subjects(self._h, int(subjects)),
                    "bsg_set_step_subjects")

    def step_subjects(self) -> int:
        n = C.c_int32()
        self._check(self._L.bsg_get_step_subjects(self._h, C.byref(n)),
                    "bsg_get_step_subjects")
        return n.value

    def tuning(self):
        a, b = C.c_int32(), C.c_int32()
        self._check(self._L.bsg_get_tuning(self._h, C.byref(a), C.byref(b)),
                    "bsg_get_tuning")
        return a.value, b.value

    def info(self, dataset: int = 0) -> dict:
        return dict(self._ds[dataset])

    # ---------------------------------------------------------- sampling --
    def run(self, nsweeps: int, sync: bool = True):
        self._check(self._L.bsg_run(self._h, int(nsweeps)), "bsg_run")
        if sync:
            self.sync()

    def step_host(self, chain: int, omega=None, nsweeps: int = 1, out=None):
        """One call: Omega in (None keeps the chain's), nsweeps sweeps of
        every chain, the chain's Omega and column means out, one wait
        (bsg_step_host).  `out` = (omega [P][P] float64, colmeans [P]
        float32) arrays to fill, else new ones."""
        P = self._dims(chain)["P"]
        a = None if omega is None else np.ascontiguousarray(omega, dtype=np.float64)
        if a is not None and a.size != P * P:
            raise ValueError(f"omega must have {P * P} entries")
        om, cm = out if out is not None else (np.empty((P, P), np.float64),
                                              np.empty(P, np.float32))
        self._check(self._L.bsg_step_host(self._h, chain, _ptr(a), int(nsweeps),
                                          _ptr(om), _ptr(cm)), "bsg_step_host")
        return om, cm

    def sync(self):
        self._check(self._L.bsg_sync(self._h), "bsg_sync")

    def run_timed(self, nsweeps: int) -> float:
        ms = C.c_double()
        self._check(self._L.bsg_run_timed(self._h, int(nsweeps), C.byref(ms)),
                    "bsg_run_timed")
        return ms.value

    def profile(self, nsweeps: int):
        ms = np.zeros(3, np.float64)
        nl = np.zeros(3, np.int64)
        self._check(self._L.bsg_profile(self._h, int(nsweeps), _ptr(ms),
                                        _ptr(nl)), "bsg_profile")
        return ms, nl

    def launches_per_sweep(self) -> int:
        return int(self._L.bsg_launches_per_sweep(self._h))

    def stream(self) -> int:
        return int(self._L.bsg_stream(self._h) or 0)

    # ------------------------------------------------------------- state --
    def _dims(self, chain):
        return self._ds[self._ch[chain]]

    def lattice(self, dataset: int = 0) -> dict:
        d = self._ds[dataset]
        idx = np.zeros(d["nsize"], np.int32)
        idxsc = np.zeros(d["nsize"], np.int32)
        v0 = np.zeros(d["n0"], np.int32)
        v1 = np.zeros(d["n1"], np.int32)
        n0 = np.zeros(d["n0"], np.uint8)
        n1 = np.zeros(d["n1"], np.uint8)
        self._check(self._L.bsg_get_lattice(self._h, dataset, _ptr(idx),
                                            _ptr(idxsc), _ptr(v0), _ptr(v1),
                                            _ptr(n0), _ptr(n1)),
                    "bsg_get_lattice")
        return dict(idx=idx, idxsc=idxsc, vox=[v0, v1], nbrs=[n0, n1])

    def beta(self, chain: int = 0) -> np.ndarray:
        d = self._dims(chain)
        out = np.zeros((d["P"], d["Vp"]), np.float32)
        self._check(self._L.bsg_get_beta(self._h, chain, _ptr(out)), "bsg_get_beta")
        return out

    def set_beta(self, chain: int, spatcoef: np.ndarray):
        d = self._dims(chain)
        a = np.ascontiguousarray(spatcoef, dtype=np.float32).reshape(d["P"], d["Vp"])
        self._check(self._L.bsg_set_beta(self._h, chain, _ptr(a)), "bsg_set_beta")

    def omega(self, chain: int = 0) -> np.ndarray:
        P = self._dims(chain)["P"]
        out = np.zeros((P, P), np.float64)
        self._check(self._L.bsg_get_omega(self._h, chain, _ptr(out)), "bsg_get_omega")
        return out

    def set_omega(self, chain: int, omega: np.ndarray):
        P = self._dims(chain)["P"]
        a = np.ascontiguousarray(omega, dtype=np.float64).reshape(P, P)
        self._check(self._L.bsg_set_omega(self._h, chain, _ptr(a)), "bsg_set_omega")

    def set_beta_wm(self, chain: int, beta_wm: float):
        self._check(self._L.bsg_set_beta_wm(self._h, chain, float(beta_wm)),
                    "bsg_set_beta_wm")

    def colmeans(self, chain: int = 0) -> np.ndarray:
        out = np.zeros(self._dims(chain)["P"], np.float32)
        self._check(self._L.bsg_get_colmeans(self._h, chain, _ptr(out)),
                    "bsg_get_colmeans")
        return out

    def sweep_count(self, chain: int = 0):
        s, k = C.c_int64(), C.c_int64()
        self._check(self._L.bsg_get_sweep(self._h, chain, C.byref(s), C.byref(k)),
                    "bsg_get_sweep")
        return s.value, k.value

    def compute_prb(self, chain: int = 0) -> np.ndarray:
        d = self._dims(chain)
        out = np.zeros((d["S"], d["V"]), np.float32)
        self._check(self._L.bsg_compute_prb(self._h, chain, _ptr(out)),
                    "bsg_compute_prb")
        return out

    def posterior(self, chain: int = 0):
        d = self._dims(chain)
        mean = np.zeros((d["P"], d["V"]))
        var = np.zeros((d["P"], d["V"]))
        prb = np.zeros((max(d["S"], 1), d["V"]))
        nk = C.c_int64()
        self._check(self._L.bsg_get_posterior(self._h, chain, _ptr(mean),
                                              _ptr(var), _ptr(prb), C.byref(nk)),
                    "bsg_get_posterior")
        return mean, var, prb[: d["S"]], nk.value

    def maps(self, chain: int = 0) -> dict:
        """The reference's output maps (mcmc.cpp:871-964) on the [Z][Y][X]
        grid: spatCoef, spatCoef.Var, standCoef per covariate and prb per
        group column."""
        d = self._dims(chain)
        R = (d["Z"], d["Y"], d["X"])
        sc = np.zeros((d["P"],) + R)
        var = np.zeros((d["P"],) + R)
        st = np.zeros((d["P"],) + R)
        prb = np.zeros((max(d["S"], 1),) + R)
        self._check(self._L.bsg_get_maps(self._h, chain, _ptr(sc), _ptr(var),
                                         _ptr(st), _ptr(prb)), "bsg_get_maps")
        return {"spatCoef": sc, "spatCoef.Var": var, "standCoef": st,
                "prb": prb[: d["S"]]}

    def reset_accumulators(self, chain: int = 0):
        self._check(self._L.bsg_reset_accumulators(self._h, chain),
                    "bsg_reset_accumulators")

    # --------------------------------------------------------- the link --
    MODELS = {"logistic": 0, "probit": 1, "t": 2}

    def set_model(self, chain: int = 0, model="probit"):
        """Latent link of the chain: "probit" (default), "logistic" or "t"
        (the reference's MODEL 1, 0, 2), or the MODEL number."""
        m = self.MODELS[model] if isinstance(model, str) else int(model)
        self._check(self._L.bsg_set_model(self._h, chain, m), "bsg_set_model")

    # ------------------------------------------------------ FP64 chains --
    def set_precision(self, chain: int = 0, bits: int = 64):
        """64: the chain's whole sweep in FP64 on the same counters (the GPU
        reference chain); 32: the FP32 sampler (default)."""
        self._check(self._L.bsg_set_precision(self._h, chain, int(bits)),
                    "bsg_set_precision")

    def beta64(self, chain: int = 0) -> np.ndarray:
        """Coefficients [P][Vp] in FP64 (an FP64 chain's own)."""
        d = self._dims(chain)
        out = np.zeros((d["P"], d["Vp"]), np.float64)
        self._check(self._L.bsg_get_beta64(self._h, chain, _ptr(out)), "bsg_get_beta64")
        return out

    # ------------------------------------------------ beta_WM update --
    def set_wm_update(self, chain: int = 0, enable: bool = True):
        """Draw beta_WM | Z, beta every sweep (updateBetaGPU)."""
        self._check(self._L.bsg_set_wm_update(self._h, chain, int(bool(enable))),
                    "bsg_set_wm_update")

    def beta_wm(self, chain: int = 0):
        """(current beta_WM, its mean over kept sweeps)."""
        b, m = C.c_float(), C.c_double()
        self._check(self._L.bsg_get_beta_wm(self._h, chain, C.byref(b), C.byref(m)),
                    "bsg_get_beta_wm")
        return b.value, m.value

    # ------------------------------------------------- DIC / Qhat pass --
    def set_predictive(self, chain: int = 0, enable: bool = True):
        """Run the DIC / Qhat pass (compute_predictGPU) after every kept
        sweep of the chain."""
        self._check(self._L.bsg_set_predictive(self._h, chain, int(bool(enable))),
                    "bsg_set_predictive")

    def predict(self, chain: int = 0) -> np.ndarray:
        """Mpredict [N][S] of the current coefficients."""
        d = self._dims(chain)
        out = np.zeros((d["N"], d["S"]))
        self._check(self._L.bsg_predict(self._h, chain, _ptr(out)), "bsg_predict")
        return out

    def predictive(self, chain: int = 0):
        """(Qhat [N][S] on the log scale, ED sum, kept sweeps covered)."""
        d = self._dims(chain)
        q = np.zeros((d["N"], d["S"]))
        ed, n = C.c_double(), C.c_int64()
        self._check(self._L.bsg_get_predictive(self._h, chain, _ptr(q), C.byref(ed),
                                                C.byref(n)), "bsg_get_predictive")
        return q, ed.value, n.value

    def dic(self, chain: int = 0) -> dict:
        """DE, ED, PD and DIC as mcmc.cpp:966-975 reports them."""
        out = np.zeros(4)
        self._check(self._L.bsg_get_dic(self._h, chain, _ptr(out)), "bsg_get_dic")
        return dict(zip(("DE", "ED", "PD", "DIC"), map(float, out)))

    def checkpoint(self, chain: int = 0) -> bytes:
        n = int(self._L.bsg_checkpoint_size(self._h, chain))
        buf = np.zeros(n, np.uint8)
        self._check(self._L.bsg_checkpoint(self._h, chain, _ptr(buf), n), "bsg_checkpoint")
        return buf.tobytes()

    def restore(self, chain: int, state: bytes):
        buf = np.frombuffer(state, np.uint8).copy()
        self._check(self._L.bsg_restore(self._h, chain, _ptr(buf), buf.size), "bsg_restore")

    def autotune(self, sweeps: int = 5):
        a, b = C.c_int32(), C.c_int32()
        self._check(self._L.bsg_autotune(self._h, sweeps, C.byref(a), C.byref(b)),
                    "bsg_autotune")
        return a.value, b.value

    def sweep_supplied(self, chain: int, ubits, normals, chi2, wnorm,
                       form: int = 0):
        """One sweep from supplied variates (parity interface)."""
        d = self._dims(chain)
        ub = np.ascontiguousarray(ubits, dtype=np.uint32).reshape(d["N"], d["V"])
        nm = np.ascontiguousarray(normals, dtype=np.float32).reshape(d["V"], d["P"])
        c2 = np.ascontiguousarray(chi2, dtype=np.float64).reshape(d["P"])
        wn = np.ascontiguousarray(wnorm, dtype=np.float64).reshape(-1)
        if wn.size == 0:
            wn = np.zeros(1)
        self._check(self._L.bsg_sweep_supplied(self._h, chain, _ptr(ub), _ptr(nm),
                                               _ptr(c2), _ptr(wn), form),
                    "bsg_sweep_supplied")


def mcmc(mask, covar, data, ntypes: int = 1, maxiter: int = 100000,
         burnin: int = 50000, seed: int = 1, wm=None, beta_wm: float = 0.0,
         df_offset: int | None = None, device: int = 0, model="probit",
         wm_update: bool = False, predictive: bool = False) -> dict:
    """The reference's chain (mcmc.cpp:311-651): sweeps 0..MAXITER, kept
    iff iter > BURNIN and iter % SAVE_ITER == 0; returns the output maps
    and the number of kept sweeps (TOTSAV).

    model: "probit", "logistic" or "t" (the reference's MODEL 1, 0, 2).
    wm_update: draw beta_WM every sweep (the reference's WM argument); adds
    "bWM" (the kept-sweep mean of beta_WM WM_v) and "beta_WM".
    predictive: run the DIC/Qhat pass on kept sweeps; adds "DIC" (DE, ED,
    PD, DIC) and "Qhat" (log scale, [N][ntypes])."""
    with Sampler(device) as s:
        ds = s.add_dataset(mask, covar, data, ntypes, wm)
        ch = s.add_chain(ds, seed=seed, burnin=burnin,
                         thin=save_iter_rule(maxiter, burnin),
                         df_offset=df_offset, beta_wm=beta_wm)
        if model != "probit" and model != 1:
            s.set_model(ch, model)
        if wm_update:
            s.set_wm_update(ch, True)
        if predictive:
            s.set_predictive(ch, True)
        s.run(maxiter + 1)
        out = s.maps(ch)
        out["TOTSAV"] = s.sweep_count(ch)[1]
        if wm_update:
            cur, mean = s.beta_wm(ch)
            m = np.asarray(mask).astype(bool)
            bwm = np.zeros(m.shape)
            bwm[m] = mean * (np.ones(int(m.sum())) if wm is None
                             else np.asarray(wm, dtype=np.float64))
            out["bWM"], out["beta_WM"] = bwm, cur
        if predictive and out["TOTSAV"] > 0:
            out["DIC"] = s.dic(ch)
            out["Qhat"] = s.predictive(ch)[0]
        return out
