/*
 * bsglmm_gb300.h -- C ABI of libbsglmm_gb300.so, a GB300 (sm_103a) Gibbs
 * sampler for the Bayesian spatial probit GLMM of BSGLMM.
 *
 * The reference (nicholst/BSGLMM) has no plugin layer: mcmc() calls the
 * launchers of covarGPU.cu through prototypes declared in mcmc.cpp:101-125
 * and shares state through extern globals.  This header is the native API
 * that replaces those launchers; bsglmm_gb300/csrc/shim/covarGPU_shim.cpp
 * maps the reference's own launcher signatures onto it.
 *
 * One context owns a CUDA stream and all device memory.  A context holds
 * datasets (a mask lattice, a design matrix and binary outcome maps) and
 * chains (sampler state over one dataset).  Every chain of a context is
 * advanced by one batched launch sequence per sweep; bsg_run() replays
 * CUDA-graph segments of sweeps.  Calls are asynchronous until a bsg_get_*
 * or bsg_sync(); errors are returned as bsg_status, never by exit/assert.
 *
 * Array layouts are the reference's:
 *   mask      X*Y*Z bytes, x fastest (NIfTI order, read_data.cpp:231-240)
 *   covar     [P][N] floats, column-major   (read_data.cpp:302)
 *   data      [N][V] bytes 0/1 by compact mask index (read_data.cpp:385)
 *   spatcoef  [P][Vp] floats by compact dilated-mask index
 *                                            (mcmc.cpp:227, main.cu:308-329)
 *   omega     [P][P] precision of the MCAR prior, element (i,j) at j + i*P
 *   maps      [P][X*Y*Z] doubles, x fastest  (mcmc.cpp:871-964)
 */
#ifndef BSGLMM_GB300_H
#define BSGLMM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t bsg_status;
enum {
  BSG_OK = 0,
  BSG_ERR_INVALID = 1,      /* bad argument or size out of range */
  BSG_ERR_CUDA = 2,         /* a CUDA runtime call failed */
  BSG_ERR_NOT_SPD = 3,      /* a Cholesky pivot was not positive */
  BSG_ERR_SAMPLER_CAP = 4,  /* a bounded rejection loop hit its cap */
  BSG_ERR_NAN = 5,          /* non-finite sampler state */
  BSG_ERR_STATE = 6,        /* call out of order (e.g. no chain) */
  BSG_ERR_NO_DEVICE = 7,    /* no CUDA device / driver */
  BSG_ERR_UNSUPPORTED = 8   /* outside the sizes this build supports */
};

#define BSG_MAX_COVAR 8 /* P; the reference allows 20 (covarGPU.cu:65-68) */

typedef struct bsg_ctx bsg_ctx;

/* One lesion-map study: the inputs BinCar reads (main.cu:82-116). */
typedef struct {
  int32_t nrow, ncol, ndepth; /* X, Y, Z: NROW, NCOL, NDEPTH */
  int32_t nsubs;              /* N: NSUBS */
  int32_t ncovar;             /* P: NCOVAR, 1..BSG_MAX_COVAR */
  int32_t nsubtypes;          /* S: NSUBTYPES, 0..P (group columns) */
  const uint8_t *mask;        /* X*Y*Z bytes, nonzero = in mask */
  const float *covar;         /* [P][N] */
  const uint8_t *data;        /* [N][V] 0/1 (values > 1 are rejected) */
  const float *wm;            /* [V] white-matter covariate or NULL (= 1) */
} bsg_dataset_desc;

/* Sampler settings of one chain. */
typedef struct {
  uint64_t seed;     /* Philox key; the chain id is part of every counter */
  int32_t df_offset; /* Wishart df = V + df_offset.  Reference CPU path:
                        P (covar.cpp:291); reference GPU path: 19
                        (covarGPU.cu:1104). */
  int32_t burnin;    /* sweep s is kept iff s > burnin && s % thin == 0 */
  int32_t thin;      /* (mcmc.cpp:303-308,584); thin >= 1 */
  float beta_wm;     /* fixed WM coefficient; 0 when WM is off */
} bsg_chain_desc;

/* ---------------------------------------------------------- lifecycle -- */
bsg_status bsg_create(int32_t device, bsg_ctx **out);
bsg_status bsg_destroy(bsg_ctx *ctx);
const char *bsg_status_string(bsg_status s);
/* Message of the last error on this context ("" if none). */
const char *bsg_last_error(const bsg_ctx *ctx);

/* Builds the lattice (main.cu:189-394) and uploads the study. */
bsg_status bsg_add_dataset(bsg_ctx *ctx, const bsg_dataset_desc *desc,
                           int32_t *dataset_id);
/* Adds a chain with beta = 0 and Omega = I (mcmc.cpp:149-154,227). */
bsg_status bsg_add_chain(bsg_ctx *ctx, int32_t dataset_id,
                         const bsg_chain_desc *desc, int32_t *chain_id);
/* Tile shape of the fused colour kernel: lanes per voxel (1, 2, 4, 8) and
 * threads per block (64, 128, 256); 0 keeps the current choice. */
bsg_status bsg_set_tuning(bsg_ctx *ctx, int32_t lanes_per_voxel,
                          int32_t block_threads);
bsg_status bsg_get_tuning(const bsg_ctx *ctx, int32_t *lanes_per_voxel,
                          int32_t *block_threads);

/* X'(Z - beta_WM WM) of the probit colour kernel (the reference's loop at
 * covarGPU.cu:327-351) on the tensor cores: a BF16x3 split product (x = hi +
 * lo, z = hi + lo, x_hi z_hi + x_hi z_lo + x_lo z_hi) with m16n8k16 MMAs per
 * warp, accumulated in FP32.  Off by default (the SIMT path: f32x2 FMAs);
 * it applies to probit chains without the beta_WM update at one lane per
 * voxel, the others keep their kernels.  The draws are the same; the
 * contraction differs from the SIMT path by the split's rounding (about
 * 2^-16 relative per product).  No counterpart in the reference. */
bsg_status bsg_set_tensor_xz(bsg_ctx *ctx, int32_t enable);

/* Subjects per whole-word step of the probit colour kernel (with or without
 * the beta_WM update; one lane per voxel, SIMT X'Z): 16 draws four Philox
 * calls per step at two resident blocks of 128 registers, 8 draws two at
 * three blocks of 80 (P <= 5).  0 (the default) chooses per P group: 16
 * when P > 5, when the group's chains average N >= 384 subjects per voxel,
 * or when its grid is at most two blocks per SM; else 8.  The variates and
 * the arithmetic are the same, so the results are identical bit for bit.
 * bsg_get_step_subjects gives the largest step the context's plan uses
 * (0 when no chain is probit FP32).  No counterpart in the reference. */
bsg_status bsg_set_step_subjects(bsg_ctx *ctx, int32_t subjects);
bsg_status bsg_get_step_subjects(bsg_ctx *ctx, int32_t *subjects);

/* ------------------------------------------------------------ sampling -- */
/* Advances every chain by nsweeps sweeps (one sweep = latent Z + beta for
 * both colours, the Omega Wishart draw, and on kept sweeps the posterior
 * accumulators).  Asynchronous. */
bsg_status bsg_run(bsg_ctx *ctx, int64_t nsweeps);
/* Waits for the context's stream; returns the first sampler error seen. */
bsg_status bsg_sync(bsg_ctx *ctx);
/* One host-driven step of one chain, the round trip the reference makes
 * per sweep (updateSpatCoefGPU uploads Omega and reads the column means,
 * updateSpatCoefPrecGPU reads the new Omega: covarGPU.cu:540,582,1106-1108)
 * in a single call: Omega from omega_in (P x P, NULL keeps the chain's),
 * nsweeps sweeps of every chain as bsg_run, then the chain's Omega and
 * column means into omega_out / colmeans_out (either may be NULL).  The
 * copies go through a pinned staging buffer of the context and the call
 * waits once, at the end, for the stream; it returns the first sampler
 * error seen, as bsg_sync does. */
bsg_status bsg_step_host(bsg_ctx *ctx, int32_t chain, const double *omega_in,
                         int64_t nsweeps, double *omega_out, float *colmeans_out);
/* Runs nsweeps and reports elapsed device time (CUDA events on the
 * context's stream around the whole batch). */
bsg_status bsg_run_timed(bsg_ctx *ctx, int64_t nsweeps, double *ms);
/* Runs nsweeps without graphs with CUDA events around each kernel class:
 * ms[0] colour-0 kernels, ms[1] colour-1 kernels (which also reduce the
 * Omega pairs and draw Omega), ms[2] whole sweeps; launches[0..2] counts. */
bsg_status bsg_profile(bsg_ctx *ctx, int64_t nsweeps, double *ms,
                       int64_t *launches);
/* Kernel launches issued per sweep by bsg_run (for launch accounting). */
int64_t bsg_launches_per_sweep(const bsg_ctx *ctx);
/* The context's cudaStream_t, for callers that record their own events. */
void *bsg_stream(bsg_ctx *ctx);

/* ----------------------------------------------------------- state I/O -- */
bsg_status bsg_dataset_info(const bsg_ctx *ctx, int32_t dataset_id,
                            int64_t *info /* X,Y,Z,nsize,V,Vp,n0,n1,N,P,S */);
bsg_status bsg_get_lattice(const bsg_ctx *ctx, int32_t dataset_id,
                           int32_t *idx, int32_t *idxsc, int32_t *vox0,
                           int32_t *vox1, uint8_t *nbrs0, uint8_t *nbrs1);
bsg_status bsg_get_beta(bsg_ctx *ctx, int32_t chain, float *spatcoef);
bsg_status bsg_set_beta(bsg_ctx *ctx, int32_t chain, const float *spatcoef);
bsg_status bsg_get_omega(bsg_ctx *ctx, int32_t chain, double *omega);
bsg_status bsg_set_omega(bsg_ctx *ctx, int32_t chain, const double *omega);
/* Sets the white-matter coefficient beta_WM of a chain (eta gains
 * beta_WM WM_v, covarGPU.cu:1386); fixed unless its update is on. */
bsg_status bsg_set_beta_wm(bsg_ctx *ctx, int32_t chain, float beta_wm);
/* The beta_WM update (updateBetaGPU, covarGPU.cu:686-724, called by
 * mcmc.cpp:344-345 when the WM argument is given): each sweep draws
 * beta_WM ~ N(var sum_v WM_v sum_i (Z_iv - x_i' beta_v), var), var = 1 /
 * (N sum_v WM_v^2), after both colours' coefficient updates (the sweep is
 * Z_0, beta_0, Z_1, beta_1, beta_WM, Omega).  Needs design columns that sum
 * to 1 for every subject (BSG_ERR_UNSUPPORTED otherwise) and a nonzero WM.
 * Off by default; kept in checkpoints. */
bsg_status bsg_set_wm_update(bsg_ctx *ctx, int32_t chain, int32_t enable);
/* Link of the chain's latent model, the reference's compile-time MODEL
 * (main.cu:42,168-175): 1 probit (default); 0 logistic and 2 t, both as a t
 * scale mixture of normals (nu = 8 with logit_factor 0.634, nu = 3 with 1):
 * Z_iv ~ N(eta, 1 / phi_iv) truncated by Y, phi_iv ~ Gamma((nu + 1) / 2,
 * (nu + (Z - eta)^2) / 2), the coefficient draw weighted by phi (Z_GPU2,
 * Phi_GPU, Spat_Coef, covarGPU.cu:398-513,1430-1563).  The weights (N V
 * floats) start at 1 and are kept in checkpoints.  Lesion probabilities are
 * 1 / (1 + exp(-beta_g / logit_factor)) (ProbLogitGPU, covarGPU.cu:1695-1721).
 * The t/logit links take production (Philox) variates only and no beta_WM
 * update. */
bsg_status bsg_set_model(bsg_ctx *ctx, int32_t chain, int32_t model);
/* Arithmetic of a chain's sweep: 32 (default) is the FP32 sampler with FP64
 * Omega and posterior sums; 64 runs the whole sweep in FP64 on the same
 * Philox counters (latent draws with CUDA's double normcdf / normcdfinv,
 * X'Z, the Cholesky and coefficient draw, the Omega pair sums and Bartlett
 * variates, the A&S lesion probabilities), the scheme of the reference's
 * CPU path (covar.cpp:121-325) and of the project's FP64 oracle chain.  It
 * is the GPU reference chain that FP32 maps are measured against at sizes
 * the CPU cannot run; it is several times slower than FP32.  Probit link
 * with beta_WM fixed only (BSG_ERR_UNSUPPORTED otherwise); FP64 state is
 * kept in checkpoints.  No counterpart in the reference. */
bsg_status bsg_set_precision(bsg_ctx *ctx, int32_t chain, int32_t bits);
/* The chain's coefficients in FP64 ([P][Vp]): an FP64 chain's own, else the
 * FP32 ones widened. */
bsg_status bsg_get_beta64(bsg_ctx *ctx, int32_t chain, double *spatcoef);
/* Current beta_WM and its mean over kept sweeps (the bWM map of
 * mcmc.cpp:795-840 is that mean times WM_v).  Either pointer may be NULL. */
bsg_status bsg_get_beta_wm(bsg_ctx *ctx, int32_t chain, float *beta_wm,
                           double *mean_kept);
/* Column means of the last sweep (covarGPU.cu:563-583). */
bsg_status bsg_get_colmeans(bsg_ctx *ctx, int32_t chain, float *means);
bsg_status bsg_get_sweep(bsg_ctx *ctx, int32_t chain, int64_t *sweep,
                         int64_t *nkept);
/* Lesion probability of the current state (compute_prbGPU,
 * covarGPU.cu:1814-1824): prb[g*V + v], A&S 26.2.17. */
bsg_status bsg_compute_prb(bsg_ctx *ctx, int32_t chain, float *prb);
/* Posterior summaries by compact mask index: mean[p*V+v], var[p*V+v]
 * (divisor nkept-1), prb[g*V+v]. */
bsg_status bsg_get_posterior(bsg_ctx *ctx, int32_t chain, double *mean,
                             double *var, double *prb, int64_t *nkept);
/* The reference's output maps on the X*Y*Z grid, zero outside the mask
 * (mcmc.cpp:871-964): spatCoef_*, spatCoef_*.Var, standCoef_*, prb_*.
 * Any pointer may be NULL. */
bsg_status bsg_get_maps(bsg_ctx *ctx, int32_t chain, double *spatcoef,
                        double *spatcoef_var, double *standcoef, double *prb);
/* Clears the posterior accumulators and the kept-sweep count. */
bsg_status bsg_reset_accumulators(bsg_ctx *ctx, int32_t chain);

/* ------------------------------------------------ DIC / Qhat predictive -- */
/* Replaces compute_predictGPU (covarGPU.cu:1866-1957), which mcmc.cpp:595
 * calls on every kept sweep, and the DIC of mcmc.cpp:966-975 with
 * compute_prb_DIC (covar.cpp:442-486).  For subject i and group column g,
 * Mpredict[i*S+g] = sum over in-mask v of log P(Y_iv | eta), eta =
 * beta_vg + beta_WM WM_v + sum_{p>=S} beta_vp X_pi, P(Y=1) the A&S 26.2.17
 * normal CDF.  All need S >= 1.
 *
 * bsg_set_predictive: when enabled, each kept sweep also runs the pass
 * (two more launches per sweep and P group, inside the graph segments) and
 * accumulates ED = sum over kept sweeps of sum_i Mpredict[i*S + own_i]
 * (own_i = the first nonzero group column of subject i, else 0) and Qhat
 * (log scale, covarGPU.cu:1937-1953).  Off by default.  Cleared by
 * bsg_reset_accumulators; kept in checkpoints. */
bsg_status bsg_set_predictive(bsg_ctx *ctx, int32_t chain, int32_t enable);
/* Mpredict [N][S] of the chain's current coefficients (does not touch ED
 * or Qhat). */
bsg_status bsg_predict(bsg_ctx *ctx, int32_t chain, double *mpredict);
/* Qhat [N][S] (may be NULL), the ED sum and the number of kept sweeps it
 * covers. */
bsg_status bsg_get_predictive(bsg_ctx *ctx, int32_t chain, double *qhat,
                              double *ed_sum, int64_t *npred);
/* dic[4] = {DE, ED, PD, DIC} as mcmc.cpp:966-975 prints them: DE = -2 sum
 * log P(Y | posterior-mean coefficients), ED = -2 (ED sum) / npred,
 * PD = ED - DE, DIC = DE + 2 PD.  BSG_ERR_STATE without kept sweeps. */
bsg_status bsg_get_dic(bsg_ctx *ctx, int32_t chain, double *dic);

/* ------------------------------------------------- checkpoint / tuning -- */
/* A chain's complete state: coefficients, Omega, sweep counters, posterior
 * sums, Philox key and chain id.  Counter-based variates make a restored
 * chain continue bit-exactly, in this or another context (same study
 * shape).  The reference's save_iter/restart_iter (mcmc.cpp:1265-1336) are
 * never called; this replaces them. */
int64_t bsg_checkpoint_size(const bsg_ctx *ctx, int32_t chain);
bsg_status bsg_checkpoint(bsg_ctx *ctx, int32_t chain, void *buf, int64_t size);
bsg_status bsg_restore(bsg_ctx *ctx, int32_t chain, const void *buf,
                       int64_t size);
/* Times each supported tile shape (lanes per voxel x threads per block,
 * and at one lane per voxel both X'Z paths of bsg_set_tensor_xz and, on
 * the SIMT path, the settings 0, 16 and 8 of bsg_set_step_subjects) on the
 * context's chains for `sweeps` sweeps, keeps the fastest (the X'Z path and
 * the step setting stay set on the context) and puts every chain back to
 * its state before the call. */
bsg_status bsg_autotune(bsg_ctx *ctx, int32_t sweeps, int32_t *lanes_per_voxel,
                        int32_t *block_threads);

/* ---------------------------------------------------- parity interface -- */
/* One sweep of one chain driven by supplied variates instead of Philox:
 * ubits [N][V] 32-bit uniforms for the latent draws (u = (k+1/2)/2^32,
 * inverted through the truncated normal CDF), normals [V][P] for the beta
 * draws, chi2[P] and wnorm[P(P-1)/2] for the Bartlett Wishart draw.
 * form 0 draws beta = m + chol(Q^-1) e as covar.cpp:168-177 does; form 1
 * draws beta = m + G^-T e with Q = G G' (the production form). */
bsg_status bsg_sweep_supplied(bsg_ctx *ctx, int32_t chain,
                              const uint32_t *ubits, const float *normals,
                              const double *chi2, const double *wnorm,
                              int32_t form);

/* ------------------------------------------------ allocation-free call -- */
/* Largest V accepted by bsg_omega_update_noalloc. */
#define BSG_NOALLOC_MAX_VOXELS 4194304

/* The Omega | beta Wishart draw of one chain, for callers that cannot
 * allocate device memory (a plugin inside a runtime that owns every
 * allocation, a pipeline that allocates only at start-up): it calls no
 * cudaMalloc/cudaFree and no allocating library routine.  No counterpart in
 * the reference (whose updateSpatCoefPrecGPU mallocs per call,
 * covarGPU.cu:1072).
 *
 * All pointers are device memory owned by the caller: spatcoef [P][Vp],
 * vox [V] padded indices of the in-mask voxels (colour 0 then colour 1 as
 * bsg_get_lattice returns them), idxsc the padded -> compact dilated map,
 * omega [P][P] (output, FP64), status (optional, 1 int: 0 or error bits).
 * chi2 [P] and wnorm [P(P-1)/2] supply the Bartlett variates; pass both
 * NULL to draw them from (seed, chain_id, sweep) as bsg_run does.  Omega
 * equals the sampler's draw from the same coefficients and variates to
 * rounding (the tests hold it to 1e-5 relative): the pair sums are formed
 * in a different order and the factor chol((S + I)^-1) by chol -> invert ->
 * chol instead of the sampler's reverse Cholesky.
 *
 * Its reduction scratch is a fixed 1.4 MB array inside the library, held
 * by every GPU that loads it until exit and shared by every call on that
 * device: calls that can overlap on the GPU race and must be serialised by
 * the caller.  The first call on each device (and the first after a
 * cudaDeviceReset) looks the array up (cudaGetSymbolAddress) and, as the
 * library's kernels load lazily, loads this kernel's module: make that
 * first call at start-up, before any stream capture.  Later calls reserve
 * nothing.  Asynchronous on `stream`.  V > BSG_NOALLOC_MAX_VOXELS returns
 * BSG_ERR_UNSUPPORTED. */
bsg_status bsg_omega_update_noalloc(const float *spatcoef, const int32_t *vox,
                                    const int32_t *idxsc, int32_t nrow,
                                    int32_t ncol, int32_t V, int32_t Vp,
                                    int32_t P, int32_t df_offset,
                                    const double *chi2, const double *wnorm,
                                    uint64_t seed, uint32_t chain_id,
                                    int64_t sweep, double *omega,
                                    int32_t *status, void *stream);

/* ------------------------------------------------------- measurement -- */
/* FP32 FMA throughput of the device in TFLOP/s (2 flops per FMA), best of
 * five launches: the denominator of the fused kernel's roofline.  No
 * counterpart in the reference. */
bsg_status bsg_fp32_peak(int32_t device, double *tflops);

/* Self-check of the paired (f32x2) forms of the latent-draw, gamma and
 * log-likelihood helpers against their scalar forms on n seeded random
 * inputs, compared bit for bit; *mismatches receives the count (0 when the
 * two forms agree).  No counterpart in the reference. */
bsg_status bsg_selftest_pairs(int32_t device, int64_t n, uint64_t seed,
                              int64_t *mismatches);

#ifdef __cplusplus
}
#endif
#endif
