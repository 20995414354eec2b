/*
 * bsg_oracle.c -- TEST INFRASTRUCTURE ONLY (see bsg_oracle.h).
 *
 * FP64 CPU restatement of the reference's probit Gibbs sweep, written from
 * the reference's behaviour; every function names the reference lines it
 * follows.  Loaded only by tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg.
 */
#include "bsg_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ===================================================================== RNG */

static inline void mulhilo32(uint32_t a, uint32_t b, uint32_t *hi,
                             uint32_t *lo) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  *lo = (uint32_t)p;
}

/* Philox-4x32 with 10 rounds: multipliers 0xD2511F53 / 0xCD9E8D57 and Weyl
 * key increments 0x9E3779B9 / 0xBB67AE85 (Salmon et al., SC'11, sec. 5). */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                       uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo32(0xD2511F53u, c0, &hi0, &lo0);
    mulhilo32(0xCD9E8D57u, c2, &hi1, &lo1);
    uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

void orc_philox_block(uint32_t c1, uint32_t c2, uint32_t c3, uint32_t key0,
                      uint32_t key1, int64_t n4, uint32_t *out) {
  uint32_t key[2] = {key0, key1};
  for (int64_t c0 = 0; c0 < n4; ++c0) {
    uint32_t ctr[4] = {(uint32_t)c0, c1, c2, c3};
    orc_philox4x32_10(ctr, key, out + 4 * c0);
  }
}

static inline void philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                          uint32_t k0, uint32_t k1, uint32_t out[4]) {
  uint32_t ctr[4] = {c0, c1, c2, c3};
  uint32_t key[2] = {k0, k1};
  orc_philox4x32_10(ctr, key, out);
}

double orc_u_from_bits(uint32_t k) {
  return ((double)k + 0.5) * 2.3283064365386963e-10; /* 2^-32 */
}

static inline double u_complement(uint32_t k) { /* 1 - u(k), exact */
  return ((double)(0xFFFFFFFFu - k) + 0.5) * 2.3283064365386963e-10;
}

double orc_ncdf(double x) { return 0.5 * erfc(-x * 0.70710678118654752440); }

/* Initial guess: Wichura (1988), Algorithm AS 241, PPND7 (about seven
 * significant digits), refined by two Newton steps on Phi(x) - p with
 * Phi from erfc, which makes it accurate to double precision. */
double orc_ndtri(double p) {
  if (!(p > 0.0) || !(p < 1.0)) return p <= 0.0 ? -INFINITY : INFINITY;
  double q = p - 0.5, x;
  if (fabs(q) <= 0.425) {
    double r = 0.180625 - q * q;
    x = q * (((59.109374720 * r + 159.29113202) * r + 50.434271938) * r +
             3.3871327179) /
        (((67.187563600 * r + 78.757757664) * r + 17.895169469) * r + 1.0);
  } else {
    double r = q < 0 ? p : 1.0 - p;
    r = sqrt(-log(r));
    if (r <= 5.0) {
      r -= 1.6;
      x = (((0.17023821103 * r + 1.3067284816) * r + 2.7568153900) * r +
           1.4234372777) /
          ((0.12021132975 * r + 0.73700164250) * r + 1.0);
    } else {
      r -= 5.0;
      x = (((0.017337203997 * r + 0.42868294337) * r + 3.0812263860) * r +
           6.6579051150) /
          ((0.012258202635 * r + 0.24197894225) * r + 1.0);
    }
    if (q < 0) x = -x;
  }
  /* Newton refinement of f(x) = Phi(x) - p, evaluated in the tail that
   * keeps relative precision: for p >= 1/2, f = (1 - p) - Phi(-x). */
  for (int it = 0; it < 3; ++it) {
    double pdf = 0.39894228040143267794 * exp(-0.5 * x * x);
    if (!(pdf > 0)) break;
    double err = (p < 0.5) ? (orc_ncdf(x) - p) : ((1.0 - p) - orc_ncdf(-x));
    x -= err / pdf;
  }
  return x;
}

double orc_normal_from_bits(uint32_t k) {
  if (k < 0x80000000u) return orc_ndtri(orc_u_from_bits(k));
  return -orc_ndtri(u_complement(k));
}

double orc_tn_lower_inv(double a, uint32_t k) {
  double Pa = orc_ncdf(a), Qa = orc_ncdf(-a);
  double pl = Pa + orc_u_from_bits(k) * Qa;
  if (pl < 0.5) return orc_ndtri(pl);
  return -orc_ndtri(Qa * u_complement(k));
}

/* Robert (1995), one-sided exponential proposal with rate
 * alpha* = (a + sqrt(a^2 + 4)) / 2; the same scheme as the reference's
 * truncNormLeft (randgen.cpp:781-814), here driven by explicit pairs. */
int orc_tn_lower_tail(double a, const uint32_t *kpairs, int max_attempts,
                      double *x) {
  double as = 0.5 * (a + sqrt(a * a + 4.0));
  for (int t = 0; t < max_attempts; ++t) {
    double u1 = orc_u_from_bits(kpairs[2 * t]);
    double u2 = orc_u_from_bits(kpairs[2 * t + 1]);
    double xx = a - log(u1) / as;
    double d = xx - as;
    if (log(u2) < -0.5 * d * d) {
      *x = xx;
      return t + 1;
    }
  }
  *x = a;
  return 0;
}

/* ============================================================ problem == */

struct orc_problem {
  int X, Y, Z, PX, PY, PZ, nsize, V, Vp, N, P, S;
  uint8_t *msk, *mskp;
  int32_t *idx, *idxsc;
  int32_t n[2];
  int32_t *vox[2];
  uint8_t *nbrs[2];
  float *covar, *wm, *xtx;
  uint8_t *data;
};

/* Lattice: padding (main.cu:56), dilation (main.cu:189-205), compact maps
 * (main.cu:308-329), colour lists and in-mask neighbour counts
 * (main.cu:333-394, cnt_nbrs main.cu:471-502).  Colour 0 <=> i+j+k odd in
 * 1-based padded coordinates (main.cu:216-252). */
static void build_lattice(orc_problem *pb, const uint8_t *mask) {
  int X = pb->X, Y = pb->Y, Z = pb->Z;
  int PX = X + 2, PY = Y + 2, PZ = Z + 2;
  pb->PX = PX;
  pb->PY = PY;
  pb->PZ = PZ;
  pb->nsize = PX * PY * PZ;
  pb->msk = (uint8_t *)calloc(pb->nsize, 1);
  pb->mskp = (uint8_t *)calloc(pb->nsize, 1);
  pb->idx = (int32_t *)malloc(sizeof(int32_t) * pb->nsize);
  pb->idxsc = (int32_t *)malloc(sizeof(int32_t) * pb->nsize);
  int t = 0;
  pb->V = 0;
  for (int k = 1; k <= Z; ++k)
    for (int j = 1; j <= Y; ++j)
      for (int i = 1; i <= X; ++i, ++t) {
        int p = i + PX * j + PX * PY * k;
        pb->msk[p] = mask[t] ? 1 : 0;
        pb->V += pb->msk[p];
      }
  int sx = 1, sy = PX, sz = PX * PY;
  for (int k = 1; k <= Z; ++k)
    for (int j = 1; j <= Y; ++j)
      for (int i = 1; i <= X; ++i) {
        int p = i + sy * j + sz * k;
        if (!pb->msk[p]) continue;
        pb->mskp[p] = 1;
        pb->mskp[p - sx] = pb->mskp[p + sx] = 1;
        pb->mskp[p - sy] = pb->mskp[p + sy] = 1;
        pb->mskp[p - sz] = pb->mskp[p + sz] = 1;
      }
  int cnt = 0, cntp = 0;
  for (int p = 0; p < pb->nsize; ++p) {
    pb->idx[p] = pb->msk[p] ? cnt++ : -1;
    pb->idxsc[p] = pb->mskp[p] ? cntp++ : -1;
  }
  pb->Vp = cntp;
  pb->n[0] = pb->n[1] = 0;
  for (int k = 1; k <= Z; ++k)
    for (int j = 1; j <= Y; ++j)
      for (int i = 1; i <= X; ++i)
        if (pb->msk[i + sy * j + sz * k]) pb->n[((i + j + k) & 1) ? 0 : 1]++;
  for (int c = 0; c < 2; ++c) {
    pb->vox[c] = (int32_t *)malloc(sizeof(int32_t) * (pb->n[c] + 1));
    pb->nbrs[c] = (uint8_t *)calloc(pb->n[c] + 1, 1);
  }
  int m[2] = {0, 0};
  for (int k = 1; k <= Z; ++k)
    for (int j = 1; j <= Y; ++j)
      for (int i = 1; i <= X; ++i) {
        int p = i + sy * j + sz * k;
        if (!pb->msk[p]) continue;
        int c = ((i + j + k) & 1) ? 0 : 1;
        pb->vox[c][m[c]] = p;
        pb->nbrs[c][m[c]] = (uint8_t)(pb->msk[p - sx] + pb->msk[p + sx] +
                                      pb->msk[p - sy] + pb->msk[p + sy] +
                                      pb->msk[p - sz] + pb->msk[p + sz]);
        m[c]++;
      }
}

orc_problem *orc_problem_new(int X, int Y, int Z, const uint8_t *mask, int N,
                             int P, int S, const float *covar,
                             const uint8_t *data, const float *wm) {
  orc_problem *pb = (orc_problem *)calloc(1, sizeof(orc_problem));
  pb->X = X;
  pb->Y = Y;
  pb->Z = Z;
  pb->N = N;
  pb->P = P;
  pb->S = S;
  build_lattice(pb, mask);
  int V = pb->V;
  pb->covar = (float *)malloc(sizeof(float) * (size_t)P * N + 4);
  memcpy(pb->covar, covar, sizeof(float) * (size_t)P * N);
  pb->data = (uint8_t *)malloc((size_t)N * V + 1);
  if (data)
    memcpy(pb->data, data, (size_t)N * V);
  else
    memset(pb->data, 0, (size_t)N * V);
  pb->wm = (float *)malloc(sizeof(float) * (V + 1));
  for (int v = 0; v < V; ++v) pb->wm[v] = wm ? wm[v] : 1.0f;
  /* X'X accumulated in float in subject order (read_data.cpp:321-327). */
  pb->xtx = (float *)calloc((size_t)P * P, sizeof(float));
  for (int i = 0; i < N; ++i)
    for (int a = 0; a < P; ++a)
      for (int b = 0; b < P; ++b)
        pb->xtx[b + a * P] += covar[a * N + i] * covar[b * N + i];
  return pb;
}

void orc_problem_free(orc_problem *pb) {
  if (!pb) return;
  free(pb->msk);
  free(pb->mskp);
  free(pb->idx);
  free(pb->idxsc);
  for (int c = 0; c < 2; ++c) {
    free(pb->vox[c]);
    free(pb->nbrs[c]);
  }
  free(pb->covar);
  free(pb->data);
  free(pb->wm);
  free(pb->xtx);
  free(pb);
}

void orc_problem_info(const orc_problem *pb, int64_t *out) {
  out[0] = pb->X;
  out[1] = pb->Y;
  out[2] = pb->Z;
  out[3] = pb->nsize;
  out[4] = pb->V;
  out[5] = pb->Vp;
  out[6] = pb->n[0];
  out[7] = pb->n[1];
  out[8] = pb->N;
  out[9] = pb->P;
}

void orc_problem_lattice(const orc_problem *pb, int32_t *idx, int32_t *idxsc,
                         int32_t *vox0, int32_t *vox1, uint8_t *nbrs0,
                         uint8_t *nbrs1) {
  memcpy(idx, pb->idx, sizeof(int32_t) * pb->nsize);
  memcpy(idxsc, pb->idxsc, sizeof(int32_t) * pb->nsize);
  memcpy(vox0, pb->vox[0], sizeof(int32_t) * pb->n[0]);
  memcpy(vox1, pb->vox[1], sizeof(int32_t) * pb->n[1]);
  memcpy(nbrs0, pb->nbrs[0], pb->n[0]);
  memcpy(nbrs1, pb->nbrs[1], pb->n[1]);
}

void orc_problem_xtx(const orc_problem *pb, float *xtx) {
  memcpy(xtx, pb->xtx, sizeof(float) * pb->P * pb->P);
}

/* ================================================= dense linear algebra == */

/* Outer-product Cholesky of the lower triangle, element (r, c) at
 * A[c + r*n] (cholesky.cpp:13-33).  Returns 0 if A is not SPD. */
static int chol_lower(double *A, int n) {
  for (int k = 0; k < n; ++k) {
    double d = A[k + k * n];
    if (!(d > 0)) return 0;
    d = sqrt(d);
    A[k + k * n] = d;
    for (int j = k + 1; j < n; ++j) A[k + j * n] /= d;
    for (int j = k + 1; j < n; ++j)
      for (int i = j; i < n; ++i) A[j + i * n] -= A[k + i * n] * A[k + j * n];
  }
  return 1;
}

/* Inverse of G G' from the lower factor G by forward/back substitution on
 * the identity columns (cholesky.cpp:55-86); writes the full inverse. */
static void chol_inverse(const double *G, int n, double *out) {
  double col[64];
  for (int k = 0; k < n; ++k) {
    for (int i = 0; i < n; ++i) col[i] = (i == k) ? 1.0 : 0.0;
    for (int i = 0; i < n; ++i) {
      double s = col[i];
      for (int j = 0; j < i; ++j) s -= G[j + i * n] * col[j];
      col[i] = s / G[i + i * n];
    }
    for (int i = n - 1; i >= 0; --i) {
      double s = col[i];
      for (int j = i + 1; j < n; ++j) s -= G[i + j * n] * col[j];
      col[i] = s / G[i + i * n];
    }
    for (int i = 0; i < n; ++i) out[k + i * n] = col[i];
  }
}

/* ================================================================ sweep == */

#define NB(pb, vox, t)                                                      \
  ((t) == 0 ? (vox)-1                                                       \
   : (t) == 1 ? (vox) + 1                                                   \
   : (t) == 2 ? (vox) - (pb)->PX                                            \
   : (t) == 3 ? (vox) + (pb)->PX                                            \
   : (t) == 4 ? (vox) - (pb)->PX * (pb)->PY                                 \
              : (vox) + (pb)->PX * (pb)->PY)

/* covar.cpp:302-325: eta = beta_wm*WM + sum_p beta_p x_ip; Z ~ TN(eta, 1)
 * on (0, inf) if Y = 1 and (-inf, 0) otherwise, by inversion of ubits. */
void orc_update_z(const orc_problem *pb, double beta_wm,
                  const double *spatcoef, const uint32_t *ubits, double *Z) {
  int N = pb->N, P = pb->P, V = pb->V, Vp = pb->Vp;
  for (int c = 0; c < 2; ++c)
    for (int j = 0; j < pb->n[c]; ++j) {
      int vox = pb->vox[c][j], v = pb->idx[vox], sc = pb->idxsc[vox];
      double base = beta_wm * pb->wm[v];
      for (int i = 0; i < N; ++i) {
        double mu = base;
        for (int p = 0; p < P; ++p)
          mu += spatcoef[(size_t)p * Vp + sc] * pb->covar[p * N + i];
        uint32_t k = ubits[(size_t)i * V + v];
        if (pb->data[(size_t)i * V + v] == 1)
          Z[(size_t)i * V + v] = mu + orc_tn_lower_inv(-mu, k);
        else
          Z[(size_t)i * V + v] = mu - orc_tn_lower_inv(mu, k);
      }
    }
}

/* One voxel of Spat_Coefff (covar.cpp:137-181) in FP64: b = X'(Z - bWM) +
 * Omega s, Q = X'X + n_v Omega, then the MVN draw.  Returns 0 on a failed
 * Cholesky (beta left unchanged). */
/* qw: X' Phi X of the voxel (t/logit links, Spat_Coef covarGPU.cu:398-513)
 * or NULL for X'X. */
static int beta_voxel(const orc_problem *pb, int c, int j, const double *b_in,
                      const double *omega, const double *e, int form,
                      double *spatcoef, const double *qw) {
  int P = pb->P, Vp = pb->Vp;
  int vox = pb->vox[c][j], sc = pb->idxsc[vox];
  double b[16], sumV[16], Q[256], W[256], m[16], out[16];
  for (int p = 0; p < P; ++p) {
    double s = 0;
    for (int t = 0; t < 6; ++t)
      s += spatcoef[(size_t)p * Vp + pb->idxsc[NB(pb, vox, t)]];
    sumV[p] = s;
    b[p] = b_in[p];
  }
  double nb = (double)pb->nbrs[c][j];
  for (int a = 0; a < P; ++a)
    for (int q = 0; q < P; ++q) {
      b[a] += omega[q + a * P] * sumV[q];
      Q[q + a * P] = (qw ? qw[q + a * P] : (double)pb->xtx[q + a * P]) +
                     nb * omega[q + a * P];
    }
  if (!chol_lower(Q, P)) return 0;
  if (form == 0) {
    /* reference form: V = Q^-1 (cholesky_invert), m = V b, L = chol(V),
     * beta = m + L e (covar.cpp:168-177, rmvnorm_float covar.cpp:93-119) */
    chol_inverse(Q, P, W);
    for (int a = 0; a < P; ++a) {
      double s = 0;
      for (int q = 0; q < P; ++q) s += W[q + a * P] * b[q];
      m[a] = s;
    }
    if (!chol_lower(W, P)) return 0;
    for (int a = 0; a < P; ++a) {
      double s = 0;
      for (int q = 0; q <= a; ++q) s += W[q + a * P] * e[q];
      out[a] = s + m[a];
    }
  } else {
    /* production form: Q = G G'; m solves G G' m = b; beta = m + G'^-1 e */
    double y[16];
    for (int a = 0; a < P; ++a) {
      double s = b[a];
      for (int q = 0; q < a; ++q) s -= Q[q + a * P] * y[q];
      y[a] = s / Q[a + a * P];
    }
    for (int a = P - 1; a >= 0; --a) {
      double s = y[a] + e[a];
      for (int q = a + 1; q < P; ++q) s -= Q[a + q * P] * out[q];
      out[a] = s / Q[a + a * P];
    }
  }
  for (int a = 0; a < P; ++a) spatcoef[(size_t)a * Vp + sc] = out[a];
  return 1;
}

/* covar.cpp:121-217 (updateSpatCoef -> Spat_Coefff per colour). */
int orc_update_spatcoef(const orc_problem *pb, double beta_wm,
                        const double *Z, const double *omega,
                        const float *normals, int form, double *spatcoef) {
  int N = pb->N, P = pb->P, V = pb->V, fails = 0;
  for (int c = 0; c < 2; ++c)
    for (int j = 0; j < pb->n[c]; ++j) {
      int vox = pb->vox[c][j], v = pb->idx[vox];
      double bwm = beta_wm * pb->wm[v], b[16], e[16];
      for (int p = 0; p < P; ++p) {
        double s = 0;
        for (int i = 0; i < N; ++i)
          s += (double)pb->covar[p * N + i] * (Z[(size_t)i * V + v] - bwm);
        b[p] = s;
        e[p] = normals[(size_t)v * P + p];
      }
      if (!beta_voxel(pb, c, j, b, omega, e, form, (double *)spatcoef, NULL))
        fails++;
    }
  return fails;
}

/* covar.cpp:220-262 (Spat_Coef_Precision) summed as in covar.cpp:276-284:
 * for each pair (r >= c) and each in-mask voxel, the three forward
 * neighbours contribute (b_r - b_r')(b_c - b_c') when b_r' != 0. */
void orc_spatcoef_prec_S(const orc_problem *pb, const double *spatcoef,
                         double *S) {
  int P = pb->P, Vp = pb->Vp;
  int off[3] = {1, pb->PX, pb->PX * pb->PY};
  memset(S, 0, sizeof(double) * P * P);
  for (int r = 0; r < P; ++r)
    for (int c = 0; c <= r; ++c) {
      const double *b1 = spatcoef + (size_t)r * Vp;
      const double *b2 = spatcoef + (size_t)c * Vp;
      double acc = 0;
      for (int col = 0; col < 2; ++col) {
        double y = 0;
        for (int j = 0; j < pb->n[col]; ++j) {
          int vox = pb->vox[col][j], sc = pb->idxsc[vox];
          for (int t = 0; t < 3; ++t) {
            int sn = pb->idxsc[vox + off[t]];
            double t1 = b1[sn], t2 = b2[sn];
            if (t1 != 0) y += (b1[sc] - t1) * (b2[sc] - t2);
          }
        }
        acc += y;
      }
      S[c + r * P] = S[r + c * P] = acc;
    }
}

/* covar.cpp:276-295 with cholesky.cpp:13-86 and the Bartlett construction
 * of rwishart2 (cholesky.cpp:245-286). */
int orc_wishart_from_S(int P, const double *S, const double *chi2,
                       const double *wnorm, double *omega) {
  double A[256], Ai[256], T[256], B[256];
  for (int i = 0; i < P * P; ++i) A[i] = S[i];
  for (int i = 0; i < P; ++i) A[i + i * P] += 1.0;
  if (!chol_lower(A, P)) return 0;
  chol_inverse(A, P, Ai);
  if (!chol_lower(Ai, P)) return 0;
  memset(T, 0, sizeof(T));
  for (int i = 0; i < P; ++i) {
    T[i + i * P] = sqrt(chi2[i]);
    for (int j = 0; j < i; ++j) T[j + i * P] = wnorm[i * (i - 1) / 2 + j];
  }
  for (int i = 0; i < P; ++i)
    for (int j = 0; j <= i; ++j) {
      double s = 0;
      for (int k = j; k <= i; ++k) s += Ai[k + i * P] * T[j + k * P];
      B[j + i * P] = s;
    }
  for (int i = 0; i < P; ++i)
    for (int j = 0; j < P; ++j) {
      int K = i < j ? i : j;
      double s = 0;
      for (int k = 0; k <= K; ++k) s += B[k + i * P] * B[k + j * P];
      omega[j + i * P] = s;
    }
  return 1;
}

/* Abramowitz & Stegun 26.2.17, as used by the reference (covar.cpp:327-348;
 * the published coefficients are necessarily the same). */
double orc_prob_sdnorm(double x) {
  const double b1 = 0.319381530, b2 = -0.356563782, b3 = 1.781477937;
  const double b4 = -1.821255978, b5 = 1.330274429, p = 0.2316419;
  const double c = 0.39894228;
  double ax = fabs(x);
  double t = 1.0 / (1.0 + p * ax);
  double tail =
      c * exp(-x * x / 2.0) * t * (t * (t * (t * (t * b5 + b4) + b3) + b2) + b1);
  return x >= 0.0 ? 1.0 - tail : tail;
}

void orc_compute_prb(const orc_problem *pb, double beta_wm,
                     const double *spatcoef, double *prb) {
  int V = pb->V, Vp = pb->Vp;
  for (int p = 0; p < pb->nsize; ++p) {
    if (!pb->msk[p]) continue;
    int v = pb->idx[p], sc = pb->idxsc[p];
    for (int g = 0; g < pb->S; ++g)
      prb[(size_t)g * V + v] =
          orc_prob_sdnorm(spatcoef[(size_t)g * Vp + sc] + beta_wm * pb->wm[v]);
  }
}

/* log of the A&S probability (covar.cpp:327-348) of the observed outcome:
 * log PhiAS(eta) for y = 1, log PhiAS(-eta) = log(1 - PhiAS(eta)) for
 * y = 0 (the A&S form satisfies PhiAS(-x) = 1 - PhiAS(x) exactly).  On the
 * tail side log(c t poly(t)) - eta^2 / 2 is taken without forming exp. */
double orc_loglik_as(double eta, int y) {
  const double b1 = 0.319381530, b2 = -0.356563782, b3 = 1.781477937;
  const double b4 = -1.821255978, b5 = 1.330274429, p = 0.2316419;
  const double c = 0.39894228;
  double ax = fabs(eta);
  double t = 1.0 / (1.0 + p * ax);
  double r = c * t * (t * (t * (t * (t * b5 + b4) + b3) + b2) + b1);
  double h = 0.5 * eta * eta;
  int tail = y ? (eta < 0.0) : (eta >= 0.0);
  return tail ? log(r) - h : log1p(-r * exp(-h));
}

/* compute_predictGPU (covarGPU.cu:1866-1903) with ProbSDNormGPU_prediction
 * (covarGPU.cu:1783-1812) and reduce_for_Mpredict (covarGPU.cu:1826-1864):
 *   mpredict[i*S + g] = sum over in-mask v of log P(Y_iv | eta_igv),
 *   eta_igv = beta_vg + beta_WM WM_v + sum_{p >= S} beta_vp X_pi,
 * i.e. subject i's prediction as a member of group column g.  The
 * reference's y log(p + 1e-35) + (1 - y) log(1 - p + 1e-35) in FP32 is the
 * same quantity up to its guard and its cancellation when 1 - p < 2^-24. */
/* log P(Y = y | z) with P(Y = 1) = 1 / (1 + exp(-z)). */
static double loglik_logit(double z, int y) {
  double a = y ? z : -z;  /* log sigma(a) = -log(1 + exp(-a)) */
  return a >= 0 ? -log1p(exp(-a)) : a - log1p(exp(a));
}

void orc_predict(const orc_problem *pb, double beta_wm, const double *spatcoef,
                 double *mpredict, int model, double inv_lf) {
  int N = pb->N, P = pb->P, S = pb->S, V = pb->V, Vp = pb->Vp;
  for (int i = 0; i < N * S; ++i) mpredict[i] = 0.0;
  for (int q = 0; q < pb->nsize; ++q) {
    if (!pb->msk[q]) continue;
    int v = pb->idx[q], sc = pb->idxsc[q];
    double bwm = beta_wm * pb->wm[v];
    for (int i = 0; i < N; ++i) {
      double rest = bwm;
      for (int p = S; p < P; ++p)
        rest += spatcoef[(size_t)p * Vp + sc] * (double)pb->covar[(size_t)p * N + i];
      int y = pb->data[(size_t)i * V + v] != 0;
      for (int g = 0; g < S; ++g) {
        double eta = spatcoef[(size_t)g * Vp + sc] + rest;
        /* t/logit links: ProbLogitGPU_prediction, covarGPU.cu:1750-1781 */
        mpredict[(size_t)i * S + g] +=
            model != 1 ? loglik_logit(eta * inv_lf, y) : orc_loglik_as(eta, y);
      }
    }
  }
}

/* compute_prb_DIC (covar.cpp:442-486), probit branch, as written there:
 *   DE = -2 sum_i sum_v [y log(x + DBL_MIN) + (1 - y) log(1 - x + DBL_MIN)],
 *   x = PhiAS((float)(sum_p mean_vp X_pi + mwm_v))
 * at the posterior means mean[p*V + v] (all P columns with the subject's own
 * covariates) and mwm[v] = mean of beta_WM WM_v.  The reference rounds eta
 * to float before its FP64 A&S evaluation, and its 1 - x cancels for
 * eta > 5 (relative error 1e-16 / (1 - x)); both are kept here. */
double orc_dic_de(const orc_problem *pb, const double *mean, const double *mwm,
                  int model) {
  int N = pb->N, P = pb->P, V = pb->V;
  double de = 0.0;
  for (int i = 0; i < N; ++i)
    for (int v = 0; v < V; ++v) {
      double y = 0.0;
      for (int p = 0; p < P; ++p)
        y += mean[(size_t)p * V + v] * (double)pb->covar[(size_t)p * N + i];
      double x;
      if (model != 1) { /* covar.cpp:457-465: exp(eta) / (1 + exp(eta)) */
        x = exp(y + (mwm ? mwm[v] : 0.0));
        x /= (1.0 + x);
      } else {
        x = orc_prob_sdnorm((double)(float)(y + (mwm ? mwm[v] : 0.0)));
      }
      int t = pb->data[(size_t)i * V + v];
      de += t * log(x + DBL_MIN) + (1 - t) * log(1.0 - x + DBL_MIN);
    }
  return -2.0 * de;
}

void orc_col_means(const orc_problem *pb, const double *spatcoef,
                   double *means) {
  for (int p = 0; p < pb->P; ++p) {
    double s = 0;
    for (int i = 0; i < pb->Vp; ++i) s += spatcoef[(size_t)p * pb->Vp + i];
    means[p] = s / (double)pb->V;
  }
}

/* ================================================== Philox FP64 chain == */

/* Marsaglia & Tsang (2000) gamma(a, 1) for a >= 1; a < 1 by the boost
 * gamma(a) = gamma(a + 1) U^(1/a).  Attempt t of draw `slot` uses counter
 * (slot*64 + t, 0, sweep, chain<<8 | GAMMA). */
static double gamma_mt(double a, uint32_t slot, uint32_t sweep,
                       const orc_chain_cfg *cfg, int *err) {
  double boost = 1.0, aa = a;
  int need_boost = a < 1.0;
  if (need_boost) aa = a + 1.0;
  double d = aa - 1.0 / 3.0, c = 1.0 / sqrt(9.0 * d);
  for (int t = 0; t < ORC_GAMMA_MAX; ++t) {
    uint32_t o[4];
    philox(slot * 64u + (uint32_t)t, 0u, sweep,
           (cfg->chain << 8) | ORC_TAG_GAMMA, cfg->key0, cfg->key1, o);
    double x = orc_normal_from_bits(o[0]);
    double cx = c * x;
    if (!(cx > -1.0)) continue;
    double v3 = (1.0 + cx) * (1.0 + cx) * (1.0 + cx);
    double u = orc_u_from_bits(o[1]), x2 = x * x;
    /* the squeeze u < 1 - 0.0331 x^4 lies inside the acceptance region:
     * it decides as the log test would, without the logarithms */
    if (u < 1.0 - 0.0331 * x2 * x2 ||
        log(u) < 0.5 * x * x + d * (1.0 - v3 + 3.0 * log1p(cx))) {
      if (need_boost) boost = pow(orc_u_from_bits(o[2]), 1.0 / a);
      return d * v3 * boost;
    }
  }
  *err |= ORC_ERR_GAMMA_CAP;
  return aa - 1.0 / 3.0;
}

static int chain_wishart(const orc_problem *pb, const orc_chain_cfg *cfg,
                         uint32_t sweep, const double *spatcoef,
                         double *omega) {
  int P = pb->P, err = 0;
  double S[256], chi2[16], wn[128];
  orc_spatcoef_prec_S(pb, spatcoef, S);
  double df = (double)pb->V + (double)cfg->df_offset;
  for (int i = 0; i < P; ++i)
    chi2[i] = 2.0 * gamma_mt(0.5 * (df - i), (uint32_t)i, sweep, cfg, &err);
  int nw = P * (P - 1) / 2;
  for (int m = 0; m < nw; m += 4) {
    uint32_t o[4];
    philox((uint32_t)(m >> 2), 0u, sweep, (cfg->chain << 8) | ORC_TAG_WNORM,
           cfg->key0, cfg->key1, o);
    for (int r = 0; r < 4 && m + r < nw; ++r)
      wn[m + r] = orc_normal_from_bits(o[r]);
  }
  double om[256];
  if (!orc_wishart_from_S(P, S, chi2, wn, om)) return err | ORC_ERR_WISHART;
  memcpy(omega, om, sizeof(double) * P * P);
  return err;
}

/* One Marsaglia & Tsang (2000) attempt at Gamma(alpha, 1), alpha >= 1, with
 * d = alpha - 1/3, c = 1/sqrt(9 d), from a normal and a uniform (bits kn,
 * ku); the squeeze u < 1 - 0.0331 x^4 first, then log u < x^2/2 + d (1 -
 * v^3 + log v^3).  The same test as the GPU's scale-mixture draw. */
static int mt_try(double d, double c, uint32_t kn, uint32_t ku, double *g) {
  double x = orc_normal_from_bits(kn), v = 1.0 + c * x, v3 = v * v * v;
  *g = d * v3;
  if (!(v > 0.0)) return 0;
  double u = orc_u_from_bits(ku), x2 = x * x;
  if (u < 1.0 - 0.0331 * x2 * x2) return 1;
  return log(u) < 0.5 * x2 + d * (1.0 - v3 + log(v3));
}

/* phi | Z, beta ~ Gamma((nu + 1) / 2, rate (nu + r^2) / 2) for subject i of
 * voxel v: attempt 0 from counter (i / 2, v, sweep, PHI) (normal, uniform
 * in the first or second pair of words), further attempt pairs from
 * (i * 32 + q, v, sweep, PHI_MORE).  For alpha = 2 (the t link, nu = 3) the
 * same pair of words gives -ln(u1 u2), a sum of two Exp(1). */
static double mix_gamma(const orc_chain_cfg *cfg, double d, double c, uint32_t i,
                        uint32_t v, uint32_t sw, int *err) {
  uint32_t o[4];
  double g;
  philox(i >> 1, v, sw, (cfg->chain << 8) | ORC_TAG_PHI, cfg->key0, cfg->key1, o);
  if (fabs(d - (2.0 - 1.0 / 3.0)) < 1e-12) /* alpha = 2: -ln(u1 u2), exactly */
    return -log(orc_u_from_bits(o[(i & 1) * 2]) * orc_u_from_bits(o[(i & 1) * 2 + 1]));
  if (mt_try(d, c, o[(i & 1) * 2], o[(i & 1) * 2 + 1], &g)) return g;
  for (int q = 0; q < (ORC_GAMMA_MAX - 1) / 2; ++q) {
    philox(i * 32u + (uint32_t)q, v, sw, (cfg->chain << 8) | ORC_TAG_PHI_MORE,
           cfg->key0, cfg->key1, o);
    if (mt_try(d, c, o[0], o[1], &g)) return g;
    if (mt_try(d, c, o[2], o[3], &g)) return g;
  }
  *err |= ORC_ERR_GAMMA_CAP;
  return d;
}

double orc_mix_gamma(double alpha, uint32_t i, uint32_t v, uint32_t sweep,
                     uint32_t key0, uint32_t key1, uint32_t chain) {
  orc_chain_cfg cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.key0 = key0;
  cfg.key1 = key1;
  cfg.chain = chain;
  double d = alpha - 1.0 / 3.0;
  int err = 0;
  return mix_gamma(&cfg, d, 1.0 / sqrt(9.0 * d), i, v, sweep, &err);
}

/* Host threads of orc_chain_run (voxels of one colour are independent given
 * the other colour, so a colour's voxel list is split into contiguous
 * ranges; results do not depend on the thread count except for the order
 * of the beta_WM sum). */
static int g_orc_threads = 1;
void orc_set_threads(int n) { g_orc_threads = n < 1 ? 1 : (n > 256 ? 256 : n); }

typedef struct {
  const orc_problem *pb;
  const orc_chain_cfg *cfg;
  double *spatcoef, *phi;
  const double *omega, *xsum;
  double bw, md, mc, nu;
  int mix, c;
  uint32_t sw;
  int j0, j1;
  double wmr; /* out: this range's term of the beta_WM conditional mean */
  int err;    /* out */
} chain_range;

/* Z_v then beta_v for the voxels j0..j1-1 of colour c (covar.cpp:302-325
 * and 121-187 on the sampler's counters). */
static void chain_colour_range(chain_range *r) {
  const orc_problem *pb = r->pb;
  const orc_chain_cfg *cfg = r->cfg;
  int N = pb->N, P = pb->P, V = pb->V, Vp = pb->Vp, c = r->c, err = 0;
  uint32_t k0 = cfg->key0, k1 = cfg->key1, ch = cfg->chain, sw = r->sw;
  double *spatcoef = r->spatcoef, *phi = r->phi, bw = r->bw, nu = r->nu;
  double wmr = 0.0;
  for (int j = r->j0; j < r->j1; ++j) {
    int vox = pb->vox[c][j], v = pb->idx[vox], sc = pb->idxsc[vox];
    double bwm = bw * pb->wm[v];
    double b[16] = {0}, e[16], zs = 0.0, qw[256] = {0};
    uint32_t o[4];
    for (int i = 0; i < N; ++i) {
      if ((i & 3) == 0)
        philox((uint32_t)(i >> 2), (uint32_t)v, sw, (ch << 8) | ORC_TAG_Z, k0, k1, o);
      double mu = bwm;
      for (int p = 0; p < P; ++p)
        mu += spatcoef[(size_t)p * Vp + sc] * pb->covar[p * N + i];
      int y = pb->data[(size_t)i * V + v] == 1;
      /* t/logit links: (Z - mu) sqrt(phi) ~ N(0, 1) truncated */
      double ph = r->mix ? phi[(size_t)i * V + v] : 1.0, sq = sqrt(ph);
      double a = (y ? -mu : mu) * sq, t;
      if (a <= ORC_A_TAIL) {
        t = orc_tn_lower_inv(a, o[i & 3]);
      } else {
        uint32_t kp[2 * ORC_TAIL_MAX];
        for (int q = 0; q < ORC_TAIL_MAX / 2; ++q)
          philox((uint32_t)i * 8u + (uint32_t)q, (uint32_t)v, sw,
                 (ch << 8) | ORC_TAG_ZTAIL, k0, k1, kp + 4 * q);
        if (!orc_tn_lower_tail(a, kp, ORC_TAIL_MAX, &t)) err |= ORC_ERR_TN_CAP;
      }
      double rr = (y ? t : -t) / sq, z = mu + rr;
      zs += z;
      if (r->mix) {
        double g = mix_gamma(cfg, r->md, r->mc, (uint32_t)i, (uint32_t)v, sw, &err);
        double phn = 2.0 * g / (nu + rr * rr);
        phi[(size_t)i * V + v] = phn;
        for (int p = 0; p < P; ++p) {
          double xp = pb->covar[p * N + i];
          b[p] += xp * phn * (z - bwm);
          for (int q = 0; q < P; ++q) qw[q + p * P] += phn * xp * pb->covar[q * N + i];
        }
      } else {
        for (int p = 0; p < P; ++p) b[p] += pb->covar[p * N + i] * (z - bwm);
      }
    }
    for (int p = 0; p < P; p += 4) {
      philox((uint32_t)(p >> 2), (uint32_t)v, sw, (ch << 8) | ORC_TAG_BETA, k0, k1, o);
      for (int q = 0; q < 4 && p + q < P; ++q) e[p + q] = orc_normal_from_bits(o[q]);
    }
    if (!beta_voxel(pb, c, j, b, r->omega, e, 1, spatcoef, r->mix ? qw : NULL))
      err |= ORC_ERR_CHOL;
    double xb = 0.0;
    for (int p = 0; p < P; ++p) xb += r->xsum[p] * spatcoef[(size_t)p * Vp + sc];
    wmr += pb->wm[v] * (zs - xb);
  }
  r->wmr = wmr;
  r->err = err;
}

static void *chain_range_thread(void *arg) {
  chain_colour_range((chain_range *)arg);
  return NULL;
}

int orc_chain_run(const orc_problem *pb, const orc_chain_cfg *cfg, int64_t s0,
                  int64_t nsweeps, double *spatcoef, double *omega,
                  double *acc_sum, double *acc_sq, double *prb_sum,
                  int64_t *nkept, double *beta_wm, double *wm_sum,
                  double *phi) {
  int N = pb->N, P = pb->P, V = pb->V, Vp = pb->Vp, S = pb->S, err = 0;
  const int mix = cfg->model != 1 && phi;
  const double nu = cfg->t_df, md = 0.5 * (nu + 1.0) - 1.0 / 3.0;
  const double mc = 1.0 / sqrt(9.0 * md);
  double *prb = (double *)malloc(sizeof(double) * ((size_t)S * V + 1));
  double bw = beta_wm ? *beta_wm : cfg->beta_wm;
  double xsum[16] = {0}, wm2 = 0.0;
  const int nth = g_orc_threads;
  chain_range rg[256];
  pthread_t tid[256];
  for (int p = 0; p < P; ++p)
    for (int i = 0; i < N; ++i) xsum[p] += pb->covar[p * N + i];
  for (int v = 0; v < V; ++v) wm2 += (double)pb->wm[v] * pb->wm[v];
  for (int64_t s = s0; s < s0 + nsweeps; ++s) {
    uint32_t sw = (uint32_t)s;
    double wmr = 0.0; /* sum_v WM_v sum_i (Z_iv - x_i' beta_v), new beta */
    for (int c = 0; c < 2; ++c) {
      int n = pb->n[c], nt = nth < n ? nth : (n > 0 ? n : 1);
      for (int t = 0; t < nt; ++t) {
        chain_range *r = &rg[t];
        r->pb = pb;
        r->cfg = cfg;
        r->spatcoef = spatcoef;
        r->phi = phi;
        r->omega = omega;
        r->xsum = xsum;
        r->bw = bw;
        r->md = md;
        r->mc = mc;
        r->nu = nu;
        r->mix = mix;
        r->c = c;
        r->sw = sw;
        r->j0 = (int)((int64_t)n * t / nt);
        r->j1 = (int)((int64_t)n * (t + 1) / nt);
      }
      if (nt == 1) {
        chain_colour_range(&rg[0]);
      } else {
        int started = 0;
        for (int t = 1; t < nt; ++t, ++started)
          if (pthread_create(&tid[t], NULL, chain_range_thread, &rg[t]) != 0) break;
        chain_colour_range(&rg[0]);
        for (int t = 1; t <= started; ++t) pthread_join(tid[t], NULL);
        for (int t = started + 1; t < nt; ++t) chain_colour_range(&rg[t]);
      }
      for (int t = 0; t < nt; ++t) {
        wmr += rg[t].wmr;
        err |= rg[t].err;
      }
    }
    /* beta_WM | Z, beta (updateBetaGPU, covarGPU.cu:680-720): normal with
     * variance 1 / (N sum WM^2) and mean variance * wmr; the lesion
     * probabilities of this sweep use the beta_WM of its latent draws. */
    double bw_used = bw;
    if (cfg->wm_update) {
      uint32_t o[4];
      philox(0u, 0u, sw, (cfg->chain << 8) | ORC_TAG_WM, cfg->key0, cfg->key1, o);
      double var = 1.0 / ((double)N * wm2);
      bw = (double)(float)(var * wmr + sqrt(var) * orc_normal_from_bits(o[0]));
    }
    err |= chain_wishart(pb, cfg, sw, spatcoef, omega);
    int kept = (s > cfg->burnin) && (s % (cfg->thin > 0 ? cfg->thin : 1) == 0);
    if (kept && wm_sum) *wm_sum += bw;
    if (kept && acc_sum) { /* running sums of mcmc.cpp:637-645 */
      if (mix) /* ProbLogitGPU (covarGPU.cu:1695-1721) */
        for (int q = 0; q < pb->nsize; ++q) {
          if (!pb->msk[q]) continue;
          for (int g = 0; g < S; ++g)
            prb[(size_t)g * V + pb->idx[q]] =
                1.0 / (1.0 + exp(-spatcoef[(size_t)g * Vp + pb->idxsc[q]] * cfg->inv_lf));
        }
      else
        orc_compute_prb(pb, bw_used, spatcoef, prb);
      ++(*nkept);
      for (int p = 0; p < pb->nsize; ++p) {
        if (!pb->msk[p]) continue;
        int v = pb->idx[p], sc = pb->idxsc[p];
        for (int q = 0; q < P; ++q) {
          double x = spatcoef[(size_t)q * Vp + sc];
          acc_sum[(size_t)q * V + v] += x;
          acc_sq[(size_t)q * V + v] += x * x;
        }
        for (int g = 0; g < S; ++g) prb_sum[(size_t)g * V + v] += prb[(size_t)g * V + v];
      }
    }
  }
  free(prb);
  if (beta_wm) *beta_wm = bw;
  return err;
}

/* ============================================= CPU timing port (float) == */

struct orc_port {
  const orc_problem *pb;
  uint64_t s[3];
  int df_offset;
  float *beta;  /* [P][Vp] */
  float *omega; /* [P][P] */
  float *Z;     /* [N][V] */
};

/* KISS as used by the reference (randgen.cpp:9-23), 64-bit words and the
 * 2^-64 scale of PREC = 64 (main.cu:12,54). */
static inline double kiss64(uint64_t *s) {
  s[1] = s[1] ^ (s[1] << 17);
  s[2] = (s[2] ^ (s[2] << 18)) & 0x7FFFFFFFull;
  s[0] = 69069ull * s[0] + 23606797ull;
  s[1] ^= (s[1] >> 15);
  s[2] ^= (s[2] >> 13);
  return (double)(s[0] + s[1] + s[2]) * 5.421010862427522e-20;
}

static double port_snorm(uint64_t *s) { /* Marsaglia polar method */
  for (;;) {
    double v1 = 2.0 * kiss64(s) - 1.0, v2 = 2.0 * kiss64(s) - 1.0;
    double r = v1 * v1 + v2 * v2;
    if (r < 1.0 && r > 0.0) return v1 * sqrt(-2.0 * log(r) / r);
  }
}

/* Robert (1995) two-sided truncated normal, the scheme of the reference's
 * truncNorm2 (randgen.cpp:726-776). */
static double port_truncnorm(double mu, double lo, double hi, uint64_t *s) {
  double u = lo - mu, v = hi - mu, a, b, x;
  if (v < 0) {
    a = -v;
    b = -u;
  } else {
    a = u;
    b = v;
  }
  if (b > a + 3.0 * exp(-a * a - 1.0 / (a * a)) / (a + sqrt(a * a + 4.0))) {
    for (;;) {
      if (a < 0.0) {
        do x = port_snorm(s);
        while (!(x > a));
      } else {
        double as = 0.5 * (a + sqrt(a * a + 4.0));
        for (;;) {
          x = a - log(kiss64(s)) / as;
          if (log(kiss64(s)) < x * (as - 0.5 * x) - as * as * 0.5) break;
        }
      }
      if (x < b) break;
    }
  } else {
    double boo = 0.0;
    if (b < 0.0) boo = b * b;
    if (a > 0.0) boo = a * a;
    for (;;) {
      x = (b - a) * kiss64(s) + a;
      if (2.0 * log(kiss64(s)) < boo - x * x) break;
    }
  }
  if (v <= 0) x = -x;
  return x + mu;
}

static double port_gamma(double a, uint64_t *s) { /* Marsaglia-Tsang */
  double d = a - 1.0 / 3.0, c = 1.0 / sqrt(9.0 * d);
  for (;;) {
    double x = port_snorm(s), cx = c * x;
    if (cx <= -1.0) continue;
    double v3 = (1 + cx) * (1 + cx) * (1 + cx);
    if (log(kiss64(s)) < 0.5 * x * x + d * (1.0 - v3 + 3.0 * log1p(cx)))
      return d * v3;
  }
}

static int cholf(float *A, int n) { /* covar.cpp:38-57 scheme, float */
  for (int k = 0; k < n; ++k) {
    if (!(A[k + k * n] > 0)) return 0;
    A[k + k * n] = sqrtf(A[k + k * n]);
    for (int j = k + 1; j < n; ++j) A[k + j * n] /= A[k + k * n];
    for (int j = k + 1; j < n; ++j)
      for (int i = j; i < n; ++i) A[j + i * n] -= A[k + i * n] * A[k + j * n];
  }
  return 1;
}

static void cholf_inverse(float *H, int n) { /* covar.cpp:59-91 scheme */
  float inv[256], col[16];
  for (int k = 0; k < n; ++k) {
    for (int i = 0; i < n; ++i) col[i] = (i == k) ? 1.0f : 0.0f;
    for (int i = 0; i < n; ++i) {
      float s = col[i];
      for (int j = 0; j < i; ++j) s -= H[j + i * n] * col[j];
      col[i] = s / H[i + i * n];
    }
    for (int i = n - 1; i >= 0; --i) {
      float s = col[i];
      for (int j = i + 1; j < n; ++j) s -= H[i + j * n] * col[j];
      col[i] = s / H[i + i * n];
    }
    for (int i = 0; i < n; ++i) inv[k + i * n] = col[i];
  }
  memcpy(H, inv, sizeof(float) * n * n);
}

orc_port *orc_port_new(const orc_problem *pb, uint64_t seed, int df_offset) {
  orc_port *pt = (orc_port *)calloc(1, sizeof(orc_port));
  pt->pb = pb;
  pt->s[0] = seed | 1u;
  pt->s[1] = (seed >> 21) + 2u;
  pt->s[2] = (seed >> 42) + 3u;
  pt->df_offset = df_offset;
  pt->beta = (float *)calloc((size_t)pb->P * pb->Vp, sizeof(float));
  pt->omega = (float *)calloc((size_t)pb->P * pb->P, sizeof(float));
  for (int p = 0; p < pb->P; ++p) pt->omega[p + p * pb->P] = 1.0f;
  pt->Z = (float *)calloc((size_t)pb->N * pb->V, sizeof(float));
  return pt;
}

void orc_port_free(orc_port *pt) {
  if (!pt) return;
  free(pt->beta);
  free(pt->omega);
  free(pt->Z);
  free(pt);
}

int64_t orc_port_updates(const orc_port *pt, int nvox_limit) {
  int64_t nv = 0;
  for (int c = 0; c < 2; ++c)
    nv += (nvox_limit >= 0 && nvox_limit < pt->pb->n[c]) ? nvox_limit
                                                         : pt->pb->n[c];
  return nv * pt->pb->N;
}

/* One CPU sweep in the reference's order and precision (mcmc.cpp:395-434):
 * updateZ over both colours, then Spat_Coefff per colour (FP32, chol ->
 * invert -> chol), then the FP64 Wishart. */
void orc_port_sweep(orc_port *pt, int nvox_limit) {
  const orc_problem *pb = pt->pb;
  int N = pb->N, P = pb->P, V = pb->V, Vp = pb->Vp;
  for (int c = 0; c < 2; ++c) {
    int n = (nvox_limit >= 0 && nvox_limit < pb->n[c]) ? nvox_limit : pb->n[c];
    for (int j = 0; j < n; ++j) {
      int vox = pb->vox[c][j], v = pb->idx[vox], sc = pb->idxsc[vox];
      for (int i = 0; i < N; ++i) {
        float tmp = 0;
        for (int p = 0; p < P; ++p)
          tmp += pt->beta[(size_t)p * Vp + sc] * pb->covar[p * N + i];
        double mu = (double)tmp;
        pt->Z[(size_t)i * V + v] =
            pb->data[(size_t)i * V + v] == 1
                ? (float)port_truncnorm(mu, 0.0, 500.0, pt->s)
                : (float)port_truncnorm(mu, -500.0, -0.0, pt->s);
      }
    }
  }
  for (int c = 0; c < 2; ++c) {
    int n = (nvox_limit >= 0 && nvox_limit < pb->n[c]) ? nvox_limit : pb->n[c];
    for (int j = 0; j < n; ++j) {
      int vox = pb->vox[c][j], v = pb->idx[vox], sc = pb->idxsc[vox];
      float mean[16], sumV[16], var[256], m2[16], runiv[16];
      for (int p = 0; p < P; ++p) {
        float s = 0;
        for (int t = 0; t < 6; ++t)
          s += pt->beta[(size_t)p * Vp + pb->idxsc[NB(pb, vox, t)]];
        sumV[p] = s;
        mean[p] = 0;
      }
      for (int i = 0; i < N; ++i) {
        float zz = pt->Z[(size_t)i * V + v];
        for (int p = 0; p < P; ++p) mean[p] += pb->covar[p * N + i] * zz;
      }
      for (int a = 0; a < P; ++a)
        for (int q = 0; q < P; ++q) {
          mean[a] += pt->omega[q + a * P] * sumV[q];
          var[q + a * P] =
              pb->xtx[q + a * P] + pb->nbrs[c][j] * pt->omega[q + a * P];
        }
      cholf(var, P);
      cholf_inverse(var, P);
      for (int a = 0; a < P; ++a) {
        float s = 0;
        for (int q = 0; q < P; ++q) s += var[q + a * P] * mean[q];
        m2[a] = s;
      }
      if (!cholf(var, P)) continue;
      for (int a = 0; a < P; ++a) runiv[a] = (float)port_snorm(pt->s);
      for (int a = 0; a < P; ++a) {
        float s = 0;
        for (int q = 0; q <= a; ++q) s += var[q + a * P] * runiv[q];
        pt->beta[(size_t)a * Vp + sc] = s + m2[a];
      }
    }
  }
  double *b = (double *)malloc(sizeof(double) * (size_t)P * Vp);
  for (size_t i = 0; i < (size_t)P * Vp; ++i) b[i] = pt->beta[i];
  double S[256], chi2[16], wn[128], om[256];
  orc_spatcoef_prec_S(pb, b, S);
  free(b);
  double df = (double)V + pt->df_offset;
  for (int i = 0; i < P; ++i) {
    chi2[i] = 2.0 * port_gamma(0.5 * (df - i), pt->s);
    for (int j = 0; j < i; ++j) wn[i * (i - 1) / 2 + j] = port_snorm(pt->s);
  }
  if (orc_wishart_from_S(P, S, chi2, wn, om))
    for (int i = 0; i < P * P; ++i) pt->omega[i] = (float)om[i];
}
