"""GB300-native (sm_103a) Gibbs sampler for BSGLMM's Bayesian spatial probit
GLMM: C ABI in include/bsglmm_gb300.h, CUDA kernels in csrc/, this package
is the host-side interface (ctypes) and the synthetic-study generator."""
from ._lib import BsgError, LIB_PATH  # noqa: F401
from .sampler import Sampler, mcmc, save_iter_rule  # noqa: F401

__all__ = ["Sampler", "mcmc", "save_iter_rule", "BsgError", "LIB_PATH"]
