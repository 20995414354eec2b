"""ctypes bindings of libbsglmm_gb300.so (declared in include/bsglmm_gb300.h).

The library is built in-tree by ``bsglmm_gb300.build``.  Loading fails
loudly when it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

_LIB = None
_LOCK = threading.Lock()

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libbsglmm_gb300.so"

BSG_OK = 0
STATUS_NAMES = {
    0: "BSG_OK", 1: "BSG_ERR_INVALID", 2: "BSG_ERR_CUDA", 3: "BSG_ERR_NOT_SPD",
    4: "BSG_ERR_SAMPLER_CAP", 5: "BSG_ERR_NAN", 6: "BSG_ERR_STATE",
    7: "BSG_ERR_NO_DEVICE", 8: "BSG_ERR_UNSUPPORTED",
}

# Every function the header declares, with (restype, argtypes).
_P = C.c_void_p
_i32 = C.c_int32
_i64 = C.c_int64
SIGNATURES = {
    "bsg_create": (_i32, [_i32, C.POINTER(_P)]),
    "bsg_destroy": (_i32, [_P]),
    "bsg_status_string": (C.c_char_p, [_i32]),
    "bsg_last_error": (C.c_char_p, [_P]),
    "bsg_add_dataset": (_i32, [_P, _P, C.POINTER(_i32)]),
    "bsg_add_chain": (_i32, [_P, _i32, _P, C.POINTER(_i32)]),
    "bsg_set_tuning": (_i32, [_P, _i32, _i32]),
    "bsg_get_tuning": (_i32, [_P, C.POINTER(_i32), C.POINTER(_i32)]),
    "bsg_set_tensor_xz": (_i32, [_P, _i32]),
    "bsg_set_step_subjects": (_i32, [_P, _i32]),
    "bsg_get_step_subjects": (_i32, [_P, C.POINTER(_i32)]),
    "bsg_run": (_i32, [_P, _i64]),
    "bsg_sync": (_i32, [_P]),
    "bsg_run_timed": (_i32, [_P, _i64, C.POINTER(C.c_double)]),
    "bsg_step_host": (_i32, [_P, _i32, _P, _i64, _P, _P]),
    "bsg_profile": (_i32, [_P, _i64, _P, _P]),
    "bsg_launches_per_sweep": (_i64, [_P]),
    "bsg_stream": (_P, [_P]),
    "bsg_dataset_info": (_i32, [_P, _i32, _P]),
    "bsg_get_lattice": (_i32, [_P, _i32, _P, _P, _P, _P, _P, _P]),
    "bsg_get_beta": (_i32, [_P, _i32, _P]),
    "bsg_set_beta": (_i32, [_P, _i32, _P]),
    "bsg_get_omega": (_i32, [_P, _i32, _P]),
    "bsg_set_omega": (_i32, [_P, _i32, _P]),
    "bsg_get_colmeans": (_i32, [_P, _i32, _P]),
    "bsg_set_beta_wm": (_i32, [_P, _i32, C.c_float]),
    "bsg_get_sweep": (_i32, [_P, _i32, C.POINTER(_i64), C.POINTER(_i64)]),
    "bsg_compute_prb": (_i32, [_P, _i32, _P]),
    "bsg_get_posterior": (_i32, [_P, _i32, _P, _P, _P, C.POINTER(_i64)]),
    "bsg_get_maps": (_i32, [_P, _i32, _P, _P, _P, _P]),
    "bsg_reset_accumulators": (_i32, [_P, _i32]),
    "bsg_set_predictive": (_i32, [_P, _i32, _i32]),
    "bsg_set_wm_update": (_i32, [_P, _i32, _i32]),
    "bsg_set_model": (_i32, [_P, _i32, _i32]),
    "bsg_set_precision": (_i32, [_P, _i32, _i32]),
    "bsg_get_beta64": (_i32, [_P, _i32, _P]),
    "bsg_get_beta_wm": (_i32, [_P, _i32, C.POINTER(C.c_float), C.POINTER(C.c_double)]),
    "bsg_predict": (_i32, [_P, _i32, _P]),
    "bsg_get_predictive": (_i32, [_P, _i32, _P, C.POINTER(C.c_double),
                                  C.POINTER(C.c_int64)]),
    "bsg_get_dic": (_i32, [_P, _i32, _P]),
    "bsg_sweep_supplied": (_i32, [_P, _i32, _P, _P, _P, _P, _i32]),
    "bsg_fp32_peak": (_i32, [_i32, C.POINTER(C.c_double)]),
    "bsg_selftest_pairs": (_i32, [_i32, C.c_int64, C.c_uint64, C.POINTER(C.c_int64)]),
    "bsg_checkpoint_size": (_i64, [_P, _i32]),
    "bsg_checkpoint": (_i32, [_P, _i32, _P, _i64]),
    "bsg_restore": (_i32, [_P, _i32, _P, _i64]),
    "bsg_autotune": (_i32, [_P, _i32, C.POINTER(_i32), C.POINTER(_i32)]),
    "bsg_omega_update_noalloc": (_i32, [_P, _P, _P, _i32, _i32, _i32, _i32, _i32,
                                        _i32, _P, _P, C.c_uint64, C.c_uint32,
                                        _i64, _P, _P, _P]),
}


class DatasetDesc(C.Structure):
    """bsg_dataset_desc."""
    _fields_ = [
        ("nrow", _i32), ("ncol", _i32), ("ndepth", _i32),
        ("nsubs", _i32), ("ncovar", _i32), ("nsubtypes", _i32),
        ("mask", _P), ("covar", _P), ("data", _P), ("wm", _P),
    ]


class ChainDesc(C.Structure):
    """bsg_chain_desc."""
    _fields_ = [
        ("seed", C.c_uint64), ("df_offset", _i32), ("burnin", _i32),
        ("thin", _i32), ("beta_wm", C.c_float),
    ]


class BsgError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        name = STATUS_NAMES.get(status, str(status))
        super().__init__(f"{where}: {name}" + (f" ({detail})" if detail else ""))


def lib() -> C.CDLL:
    """The loaded library; raises if it was not built."""
    global _LIB
    with _LOCK:
        if _LIB is None:
            if not LIB_PATH.exists():
                raise RuntimeError(
                    f"{LIB_PATH} is missing: build it with "
                    "`python -m bsglmm_gb300.build` (there is no CPU fallback)")
            L = C.CDLL(str(LIB_PATH))
            for name, (res, args) in SIGNATURES.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _LIB = L
        return _LIB
