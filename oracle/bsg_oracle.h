/*
 * bsg_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement (FP64) of the reference's probit Gibbs sweep
 * (nicholst/BSGLMM, bsglmm/covar.cpp, bsglmm/cholesky.cpp, bsglmm/main.cu,
 * bsglmm/mcmc.cpp).  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg may load this library, and only as the checker or as the
 * timed CPU baseline.  The product (libbsglmm_gb300.so) never links or calls
 * it.
 *
 * Parity of this restatement is pinned against the reference's own
 * covar.cpp + cholesky.cpp, compiled from source with a supplied-variates
 * interposer (oracle/ref_harness.cpp, built into oracle/_ref/); the golden
 * fixtures in tests/golden/ are the reference's outputs from that build.
 *
 * Layout conventions follow the reference exactly:
 *   covar[p*N + i]          design matrix, column-major (read_data.cpp:302)
 *   data[i*V + v]           outcomes, subject-major, compact mask index v
 *   spatcoef[p*Vp + sc]     coefficients, compact dilated-mask index sc
 *   omega[j + i*P]          P x P precision (symmetric)
 *   padded index            i + (X+2)*j + (X+2)*(Y+2)*k   (main.cu:56)
 */
#ifndef BSG_ORACLE_H
#define BSG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- RNG ---- */
/* Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11). */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                       uint32_t out[4]);
/* out[4*c0 + r], c0 in [0, n4): the stream with counter (c0, c1, c2, c3). */
void orc_philox_block(uint32_t c1, uint32_t c2, uint32_t c3, uint32_t key0,
                      uint32_t key1, int64_t n4, uint32_t *out);

/* The canonical 32-bit -> (0,1) mapping: u = (k + 1/2) 2^-32. */
double orc_u_from_bits(uint32_t k);
double orc_ncdf(double x);              /* Phi(x) */
double orc_ndtri(double p);             /* Phi^{-1}(p), 0 < p < 1 */
double orc_normal_from_bits(uint32_t k);/* Phi^{-1}(u(k)) with exact tails */
/* N(0,1) truncated to (a, +inf) by inversion of the canonical uniform. */
double orc_tn_lower_inv(double a, uint32_t k);
/* Robert (1995) exponential-proposal rejection for a > 0, driven by
 * uniform pairs; returns the number of attempts used (0 = cap hit). */
int orc_tn_lower_tail(double a, const uint32_t *kpairs, int max_attempts,
                      double *x);

/* ------------------------------------------------------------ problem ---- */
typedef struct orc_problem orc_problem;

/* mask: X*Y*Z bytes, x fastest (nonzero = in mask).  covar: [P][N].
 * data: [N][V] 0/1 by compact mask index.  wm: V floats or NULL (WM = 1). */
orc_problem *orc_problem_new(int X, int Y, int Z, const uint8_t *mask, int N,
                             int P, int S, const float *covar,
                             const uint8_t *data, const float *wm);
void orc_problem_free(orc_problem *pb);
/* out[0..9] = X, Y, Z, nsize, V, Vp, n0, n1, N, P */
void orc_problem_info(const orc_problem *pb, int64_t *out);
/* Copies of the lattice maps (main.cu:189-394,471-502). */
void orc_problem_lattice(const orc_problem *pb, int32_t *idx, int32_t *idxsc,
                         int32_t *vox0, int32_t *vox1, uint8_t *nbrs0,
                         uint8_t *nbrs1);
void orc_problem_xtx(const orc_problem *pb, float *xtx);

/* ------------------------------------------------ one sweep, FP64 -------- */
/* covar.cpp:302-325.  ubits: [N][V] 32-bit uniforms.  Z: [N][V]. */
void orc_update_z(const orc_problem *pb, double beta_wm,
                  const double *spatcoef, const uint32_t *ubits, double *Z);
/* covar.cpp:121-217.  normals: [V][P].  form 0 = reference draw
 * m + chol(Q^-1) e (covar.cpp:168-177); form 1 = m + G^-T e with Q = G G'.
 * Returns the number of voxels whose Cholesky failed. */
int orc_update_spatcoef(const orc_problem *pb, double beta_wm,
                        const double *Z, const double *omega,
                        const float *normals, int form, double *spatcoef);
/* covar.cpp:220-262,276-284: S (without the +I) as P*P, symmetric. */
void orc_spatcoef_prec_S(const orc_problem *pb, const double *spatcoef,
                         double *S);
/* covar.cpp:286-295 + cholesky.cpp:13-86,245-286: Omega ~ Wishart from
 * (S + I)^-1 given chi2[i] ~ chi^2(df - i) and lower normals
 * wnorm[i(i-1)/2 + j], j < i.  Returns 1 on success. */
int orc_wishart_from_S(int P, const double *S, const double *chi2,
                       const double *wnorm, double *omega);
/* covar.cpp:327-348 (Abramowitz & Stegun 26.2.17). */
double orc_prob_sdnorm(double x);
/* covar.cpp:350-364: prb[g*V + v]. */
void orc_compute_prb(const orc_problem *pb, double beta_wm,
                     const double *spatcoef, double *prb);
/* log of the A&S probability of outcome y given eta. */
double orc_loglik_as(double eta, int y);
/* compute_predictGPU (covarGPU.cu:1783-1903): mpredict[i*S + g], the log
 * predictive of subject i's outcomes as a member of group column g. */
void orc_predict(const orc_problem *pb, double beta_wm, const double *spatcoef,
                 double *mpredict, int model, double inv_lf);
/* compute_prb_DIC (covar.cpp:442-486): DE at the posterior means
 * mean[p*V + v] with mwm[v] (NULL = 0); model != 1 takes its logistic
 * branch. */
double orc_dic_de(const orc_problem *pb, const double *mean, const double *mwm,
                  int model);
/* Column means (covarGPU.cu:563-583): sum over Vp entries / V. */
void orc_col_means(const orc_problem *pb, const double *spatcoef,
                   double *means);

/* --------------------------------- Philox-driven FP64 chain (oracle) ----- */
typedef struct {
  uint32_t key0, key1;    /* Philox key */
  uint32_t chain;         /* chain id, part of every counter */
  int32_t df_offset;      /* Wishart df = V + df_offset */
  int32_t burnin, thin;   /* kept iff sweep > burnin && sweep % thin == 0 */
  double beta_wm;         /* initial beta_WM */
  int32_t wm_update;      /* draw beta_WM | Z, beta after both colours */
  int32_t model;          /* 1 probit; 0 logistic, 2 t (scale mixture) */
  double t_df, inv_lf;    /* nu and 1 / logit_factor of the t/logit links */
} orc_chain_cfg;

/* Runs sweeps [s0, s0 + nsweeps) from state (spatcoef, omega, *beta_wm) in
 * FP64 using the same counter layout and scan as the GPU sampler: per
 * colour Z_v then beta_v, then (wm_update) beta_WM | Z, beta, then Omega.
 * beta_wm may be NULL (cfg->beta_wm, fixed).  Accumulates (if acc_sum !=
 * NULL) the running sums acc_sum[P][V], acc_sq[P][V], prb_sum[S][V] of
 * mcmc.cpp:637-645, *wm_sum (if not NULL, the kept beta_WM values) and
 * *nkept.  With model != 1, phi [N][V] holds the scale-mixture weights (in
 * and out).  Returns an OR of error flags (0 = ok). */
int orc_chain_run(const orc_problem *pb, const orc_chain_cfg *cfg, int64_t s0,
                  int64_t nsweeps, double *spatcoef, double *omega,
                  double *acc_sum, double *acc_sq, double *prb_sum,
                  int64_t *nkept, double *beta_wm, double *wm_sum,
                  double *phi);

/* Host threads orc_chain_run splits each colour's voxels over (default 1). */
void orc_set_threads(int n);

/* The scale-mixture Gamma(alpha, 1) draw of subject i at voxel v (the
 * counters and Marsaglia-Tsang test the GPU uses). */
double orc_mix_gamma(double alpha, uint32_t i, uint32_t v, uint32_t sweep,
                     uint32_t key0, uint32_t key1, uint32_t chain);

/* ------------------------------- CPU timing port of the reference sweep -- */
/* A reentrant restatement of the reference's CPU sweep (mcmc.cpp:395-434:
 * updateZ with Robert-1995 rejection, FP32 Spat_Coefff with chol/invert/chol,
 * FP64 Wishart), driven by a KISS stream (randgen.cpp:9-23), restricted to
 * the first `nvox_limit` voxels of each colour list (<0 = all).  Used only as
 * the timed CPU baseline.  State in reference precision (float). */
typedef struct orc_port orc_port;
orc_port *orc_port_new(const orc_problem *pb, uint64_t seed, int df_offset);
void orc_port_free(orc_port *pt);
void orc_port_sweep(orc_port *pt, int nvox_limit);
int64_t orc_port_updates(const orc_port *pt, int nvox_limit);

/* error flags shared with the GPU sampler */
#define ORC_ERR_TN_CAP 1
#define ORC_ERR_CHOL 2
#define ORC_ERR_NAN 4
#define ORC_ERR_GAMMA_CAP 8
#define ORC_ERR_WISHART 16

/* Counter tags (c3 = chain << 8 | tag). */
#define ORC_TAG_Z 1u
#define ORC_TAG_ZTAIL 2u
#define ORC_TAG_BETA 3u
#define ORC_TAG_WNORM 4u
#define ORC_TAG_GAMMA 5u
#define ORC_TAG_WM 6u
#define ORC_TAG_PHI 7u
#define ORC_TAG_PHI_MORE 8u

#define ORC_A_TAIL 5.0      /* inversion below, Robert rejection above */
#define ORC_TAIL_MAX 16     /* rejection attempts per draw */
#define ORC_GAMMA_MAX 64    /* Marsaglia-Tsang attempts per draw */

#ifdef __cplusplus
}
#endif
#endif
