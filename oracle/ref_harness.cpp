/*
 * ref_harness.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * Links the reference's own CPU update code (nicholst/BSGLMM
 * bsglmm/covar.cpp and bsglmm/cholesky.cpp, compiled from the reference
 * tree by oracle/Makefile, never copied) into a shared library that tests
 * can drive.  It supplies the globals those files expect (they are defined
 * by the reference's main.cu / mcmc.cpp, which need a GPU and the NIfTI
 * reader and are not built) and exposes extern "C" entry points.
 *
 * Two builds:
 *   -DBSG_REF_SUPPLIED  this file also defines the reference's variate
 *                       functions snorm / rgamma / truncNorm2 (randgen.h) so
 *                       that the reference's updateZ, Spat_Coefff and
 *                       rwishart2 consume supplied uniforms and normals, in
 *                       the call order the reference makes them;
 *   (default)           the reference's randgen.cpp is linked too (KISS
 *                       generator), for distributional tests and timing.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "binCAR.h"
#include "bsg_oracle.h"
#include "randgen.h"

/* ---- globals defined by the reference's main.cu / mcmc.cpp ------------- */
int NSUBS, NROW, NCOL, NDEPTH, TOTVOX, TOTVOXp, NCOVAR, NSIZE, NSUBTYPES;
int iter = 0;
int MODEL = 1;
int PREC = 64;
double M = 5.421010862427522e-20; /* 2^-64, main.cu:54 with PREC = 64 */
INDEX *INDX = nullptr;
int *hostIdx = nullptr;
int *hostIdxSC = nullptr;
float *XXprime = nullptr;
float *XXprime_Fix = nullptr;

/* ---- reference functions (C++ linkage, covar.cpp / cholesky.cpp) ------- */
void updateZ(float *, float *, unsigned char *, unsigned char *, float,
             float *, float *, float *, unsigned long *);
void updateSpatCoef(float *, float *, float *, float *, float *, float *,
                    unsigned char *, float, float *, unsigned long *);
void updateSpatCoefPrec(float *, float *, unsigned char *, unsigned long *);
void compute_prb(float *, float *, float *, float, float *, unsigned char *);
double compute_prb_DIC(double *, double *, float *, unsigned char *,
                       unsigned char *, int);
double ProbSDNorm(const double x);
int cholesky_decomp(double *A, int num_col);
void cholesky_invert(int len, double *H);
int rwishart2(double *result, double *S, int size_S, int df,
              unsigned long *seed);

static std::vector<unsigned char> g_mskpad;
static unsigned long g_seed[3] = {1, 2, 3};

#ifdef BSG_REF_SUPPLIED
/* ---- supplied-variate interposers (replace randgen.cpp) ---------------- */
enum { PH_NONE = 0, PH_Z, PH_BETA, PH_WISHART };
static int g_phase = PH_NONE;
static const uint32_t *g_ubits = nullptr;
static const float *g_normals = nullptr;
static const double *g_chi2 = nullptr, *g_wnorm = nullptr;
static std::vector<int64_t> g_zorder, g_eorder;
static size_t g_zk = 0, g_ek = 0, g_gk = 0, g_wk = 0;
static std::vector<double> g_gamma_shapes;
static int g_underrun = 0;

/* Called by the reference's updateZ (covar.cpp:316-321) with bounds
 * (0, 500) for Y = 1 and (-500, -0) for Y = 0.  Returns the canonical
 * inverse-CDF draw of the next supplied uniform. */
double truncNorm2(double mu, double std, double u, double v,
                  unsigned long *) {
  if (g_phase != PH_Z || g_zk >= g_zorder.size()) {
    g_underrun = 1;
    return mu;
  }
  uint32_t k = g_ubits[g_zorder[g_zk++]];
  if (v >= 500.0) return mu + std * orc_tn_lower_inv((u - mu) / std, k);
  return mu - std * orc_tn_lower_inv((mu - v) / std, k);
}

double snorm(unsigned long *) {
  if (g_phase == PH_BETA && g_ek < g_eorder.size())
    return (double)g_normals[g_eorder[g_ek++]];
  if (g_phase == PH_WISHART) return g_wnorm[g_wk++];
  g_underrun = 1;
  return 0.0;
}

double rgamma(double alpha, double beta, unsigned long *) {
  g_gamma_shapes.push_back(alpha);
  (void)beta;
  return g_chi2[g_gk++];
}
#else
double kiss(unsigned long *);
int write_nifti_file(int, int, int, int, char *, char *, double *);  /* nifti1_read_write.cpp */
double sgamma(double, unsigned long *);
#endif

extern "C" {

/* Installs a problem; the lattice arrays come from the caller (the oracle's
 * restatement of main.cu) and X'X is formed here as read_data.cpp:321-327
 * forms it. */
int ref_setup(int X, int Y, int Z, int N, int P, int S, int V, int Vp,
              const int32_t *idx, const int32_t *idxsc, int n0,
              const int32_t *vox0, const uint8_t *nbrs0, int n1,
              const int32_t *vox1, const uint8_t *nbrs1, const float *covar) {
  NROW = X;
  NCOL = Y;
  NDEPTH = Z;
  NSUBS = N;
  NCOVAR = P;
  NSUBTYPES = S;
  TOTVOX = V;
  TOTVOXp = Vp;
  NSIZE = (X + 2) * (Y + 2) * (Z + 2);
  free(hostIdx);
  free(hostIdxSC);
  hostIdx = (int *)malloc(sizeof(int) * NSIZE);
  hostIdxSC = (int *)malloc(sizeof(int) * NSIZE);
  memcpy(hostIdx, idx, sizeof(int) * NSIZE);
  memcpy(hostIdxSC, idxsc, sizeof(int) * NSIZE);
  g_mskpad.assign(NSIZE, 0);
  for (int p = 0; p < NSIZE; ++p) g_mskpad[p] = idx[p] >= 0;
  if (!INDX) INDX = (INDEX *)calloc(2, sizeof(INDEX));
  const int32_t *vx[2] = {vox0, vox1};
  const uint8_t *nb[2] = {nbrs0, nbrs1};
  int nn[2] = {n0, n1};
  for (int c = 0; c < 2; ++c) {
    free(INDX[c].hostVox);
    free(INDX[c].hostNBRS);
    INDX[c].hostN = nn[c];
    INDX[c].hostVox = (int *)malloc(sizeof(int) * (nn[c] + 1));
    INDX[c].hostNBRS = (unsigned char *)malloc(nn[c] + 1);
    memcpy(INDX[c].hostVox, vx[c], sizeof(int) * nn[c]);
    memcpy(INDX[c].hostNBRS, nb[c], nn[c]);
  }
  free(XXprime);
  XXprime = (float *)calloc((size_t)P * P, sizeof(float));
  for (int isub = 0; isub < N; ++isub)
    for (int i = 0; i < P; ++i)
      for (int j = 0; j < P; ++j)
        XXprime[j + i * P] += covar[i * N + isub] * covar[j * N + isub];
  return 0;
}

void ref_xtx(float *out) { memcpy(out, XXprime, sizeof(float) * NCOVAR * NCOVAR); }

/* covar.cpp:302-325 */
void ref_update_z(float *Zout, const uint8_t *data, const float *wm,
                  float beta, const float *spatcoef, const float *covar) {
#ifdef BSG_REF_SUPPLIED
  g_phase = PH_Z;
  g_zk = 0;
#endif
  updateZ(Zout, nullptr, (unsigned char *)data, g_mskpad.data(), beta,
          (float *)wm, (float *)spatcoef, (float *)covar, g_seed);
}

/* covar.cpp:189-217 */
void ref_update_spatcoef(float *spatcoef, const float *Z, float *omega,
                         const float *wm, float beta, const float *covar) {
#ifdef BSG_REF_SUPPLIED
  g_phase = PH_BETA;
  g_ek = 0;
#endif
  float alpha_mean[64];
  updateSpatCoef((float *)covar, spatcoef, omega, nullptr, alpha_mean,
                 (float *)Z, g_mskpad.data(), beta, (float *)wm, g_seed);
}

/* covar.cpp:264-299 */
void ref_update_spatcoef_prec(float *omega, const float *spatcoef) {
#ifdef BSG_REF_SUPPLIED
  g_phase = PH_WISHART;
  g_gk = g_wk = 0;
  g_gamma_shapes.clear();
#endif
  updateSpatCoefPrec(omega, (float *)spatcoef, g_mskpad.data(), g_seed);
}

/* covar.cpp:350-364 */
void ref_compute_prb(float *prb, const float *spatcoef, const float *wm,
                     float beta) {
  compute_prb(prb, nullptr, (float *)spatcoef, beta, (float *)wm,
              g_mskpad.data());
}

double ref_prob_sdnorm(double x) { return ProbSDNorm(x); }

/* The reference's MODEL global (main.cu:42). */
void ref_set_model(int model) { MODEL = model; }

/* covar.cpp:442-486: DE from the posterior-mean maps mcov[p][X*Y*Z] and
 * mwm[X*Y*Z] on the unpadded grid (x fastest), outcomes data[i*V + v]. */
double ref_compute_prb_dic(double *mcov, double *mwm, float *covar,
                           const uint8_t *data) {
  return compute_prb_DIC(mcov, mwm, covar, (unsigned char *)data,
                         g_mskpad.data(), NROW * NCOL * NDEPTH);
}

int ref_cholesky_decomp(double *A, int n) { return cholesky_decomp(A, n); }
void ref_cholesky_invert(double *H, int n) { cholesky_invert(n, H); }

#ifdef BSG_REF_SUPPLIED
/* Supplied variates: ubits [N][V]; normals [V][P] by compact mask index;
 * chi2[P]; wnorm[P(P-1)/2] in rwishart2's call order.  The call order of
 * the reference is rebuilt from the installed colour lists. */
void ref_set_supplied(const uint32_t *ubits, const float *normals,
                      const double *chi2, const double *wnorm) {
  g_ubits = ubits;
  g_normals = normals;
  g_chi2 = chi2;
  g_wnorm = wnorm;
  g_zorder.clear();
  g_eorder.clear();
  for (int c = 0; c < 2; ++c)
    for (int j = 0; j < INDX[c].hostN; ++j) {
      int v = hostIdx[INDX[c].hostVox[j]];
      for (int i = 0; i < NSUBS; ++i)
        g_zorder.push_back((int64_t)i * TOTVOX + v);
      for (int p = 0; p < NCOVAR; ++p) g_eorder.push_back((int64_t)v * NCOVAR + p);
    }
  g_underrun = 0;
}

int ref_underrun(void) { return g_underrun; }

int ref_gamma_shapes(double *out, int cap) {
  int n = (int)g_gamma_shapes.size();
  for (int i = 0; i < n && i < cap; ++i) out[i] = g_gamma_shapes[i];
  return n;
}

/* rwishart2 (cholesky.cpp:245-286) on a caller-given factor with supplied
 * variates. */
int ref_rwishart2(double *result, double *S, int P, int df, const double *chi2,
                  const double *wnorm) {
  g_phase = PH_WISHART;
  g_chi2 = chi2;
  g_wnorm = wnorm;
  g_gk = g_wk = 0;
  return rwishart2(result, S, P, df, g_seed);
}
#else
void ref_kiss_seed(uint64_t a, uint64_t b, uint64_t c) {
  g_seed[0] = (unsigned long)a;
  g_seed[1] = (unsigned long)b;
  g_seed[2] = (unsigned long)c;
}
/* The reference's single-file NIfTI-1 writer (nifti1_read_write.cpp:198-322)
 * on a volume of FLOAT64 values, x fastest. */
int ref_write_nifti(int nrow, int ncol, int ndepth, const char *path, double *data) {
  return write_nifti_file(nrow, ncol, ndepth, 1, (char *)path, (char *)path, data);
}
/* n raw draws of the reference's KISS generator (randgen.cpp:9-23), then
 * its state, as the program writes it back to seed.dat (main.cu:430-432). */
void ref_kiss_many(int n, double *out, uint64_t *state) {
  for (int i = 0; i < n; ++i) out[i] = kiss(g_seed);
  for (int i = 0; i < 3; ++i) state[i] = (uint64_t)g_seed[i];
}
/* The reference's own samplers on its KISS stream (randgen.cpp). */
void ref_truncnorm_many(double mu, double lo, double hi, int n, double *out) {
  for (int i = 0; i < n; ++i) out[i] = truncNorm2(mu, 1.0, lo, hi, g_seed);
}
void ref_snorm_many(int n, double *out) {
  for (int i = 0; i < n; ++i) out[i] = snorm(g_seed);
}
void ref_rgamma_many(double a, double b, int n, double *out) {
  for (int i = 0; i < n; ++i) out[i] = rgamma(a, b, g_seed);
}
/* One reference CPU sweep (mcmc.cpp:400,418,428) for timing. */
void ref_cpu_sweep(float *Z, const uint8_t *data, const float *wm,
                   float *spatcoef, float *omega, const float *covar) {
  updateZ(Z, nullptr, (unsigned char *)data, g_mskpad.data(), 0.0f,
          (float *)wm, spatcoef, (float *)covar, g_seed);
  float alpha_mean[64];
  updateSpatCoef((float *)covar, spatcoef, omega, nullptr, alpha_mean, Z,
                 g_mskpad.data(), 0.0f, (float *)wm, g_seed);
  updateSpatCoefPrec(omega, spatcoef, g_mskpad.data(), g_seed);
}
#endif

} /* extern "C" */
