// bsg_wishart.cuh -- the FP64 Omega | beta draw run by one warp at the end
// of a sweep: Marsaglia-Tsang gamma variates, warp-parallel Cholesky, and
// the Bartlett construction.
#pragma once

#include "bsg_device.cuh"

namespace bsg {

// ----------------------------------------------------- FP64 Wishart tail --
// Marsaglia & Tsang (2000) gamma(a, 1); a < 1 through the U^(1/a) boost.
// Attempt t of slot uses counter (slot*64 + t, 0, sweep, chain<<8|GAMMA).
// The squeeze u < 1 - 0.0331 x^4 lies inside the acceptance region, so it
// accepts exactly the attempts the log test would; it spares the two FP64
// logarithms in most attempts.  F64: the normal of each attempt in FP64
// (the FP64 chain) instead of the FP32 inversion.
template <bool F64 = false>
static __device__ double gamma_mt(double a, uint32_t slot, uint32_t sweep,
                                  uint32_t c3, uint32_t k0, uint32_t k1,
                                  int *err) {
  const bool boost = a < 1.0;
  const double aa = boost ? a + 1.0 : a;
  const double dd = aa - 1.0 / 3.0, c = 1.0 / sqrt(9.0 * dd);
  for (int t = 0; t < kGammaMax; ++t) {
    const uint4 r = philox1(make_uint4(slot * 64u + (uint32_t)t, 0u, sweep, c3),
                            k0, k1);
    const double x = F64 ? normal_of_d(r.x) : (double)normal_of(r.x);
    const double cx = c * x;
    if (!(cx > -1.0)) continue;
    const double v3 = (1.0 + cx) * (1.0 + cx) * (1.0 + cx);
    const double u = u_of_d(r.y), x2 = x * x;
    if (u < 1.0 - 0.0331 * x2 * x2 ||
        log(u) < 0.5 * x * x + dd * (1.0 - v3 + 3.0 * log1p(cx)))
      return dd * v3 * (boost ? pow(u_of_d(r.z), 1.0 / a) : 1.0);
  }
  *err |= kErrGammaCap;
  return dd;
}

// The Bartlett variates of a sweep, which do not depend on S: lane i < P
// draws sqrt(chi^2(df - i)) into wd[i], lane q < P(P-1)/2 the normal of
// the q-th strictly lower entry (row-major) into wd[kMaxP + q].  Run by the
// last colour-0 block, off the Omega draw's dependency chain.  Returns the
// lane's error bits.  F64: normals in FP64 (the FP64 chain).
template <bool F64 = false>
static __device__ int wishart_draws(const ChainDev &ch, const DatasetDev &d,
                                    long long sweep, int lane, double *wd) {
  const int P = d.P;
  const uint32_t cid = ch.chain_id << 8, sw = (uint32_t)sweep;
  int err = 0;
  const double df = (double)d.V + (double)ch.df_offset;
  if (lane < P)
    wd[lane] = sqrt(2.0 * gamma_mt<F64>(0.5 * (df - lane), (uint32_t)lane, sw,
                                        cid | kTagGamma, ch.key0, ch.key1, &err));
  if (lane < P * (P - 1) / 2) {
    const uint4 r = philox1(make_uint4((uint32_t)(lane >> 2), 0u, sw, cid | kTagWNorm),
                            ch.key0, ch.key1);
    wd[kMaxP + lane] = F64 ? normal_of_d(pick4(r, lane & 3))
                           : (double)normal_of(pick4(r, lane & 3));
  }
  return err;
}

// Omega | beta ~ Wishart(df, (S + I)^-1) by the Bartlett construction of
// rwishart2 (cholesky.cpp:245-286), FP64, one warp.  The reference forms
// chol((S + I)^-1) by chol -> invert -> chol (covar.cpp:286-291,
// covarGPU.cu:1099-1104); the same factor is reached here with a fraction
// of the dependent work: with the reverse (upper) Cholesky S + I = U U',
// the inverse is U^-T U^-1 and U^-T is lower triangular with a positive
// diagonal, so chol((S + I)^-1) = U^-T (the Cholesky factor is unique),
// and B = U^-T T comes from forward substitution without forming U^-T.
static __device__ void wishart_warp(const ChainDev &ch, const DatasetDev &d,
                                    const double *tot, long long sweep,
                                    bool kept, long long nk, int supplied,
                                    const Supplied &sup, int lane) {
  __shared__ double A[kMaxP][kMaxP], T[kMaxP][kMaxP], B[kMaxP][kMaxP], rd[kMaxP];
  const int P = d.P;
  const uint32_t cid = ch.chain_id << 8, sw = (uint32_t)sweep;
  int err = 0;
  // entry q of the packed lower triangle is (r, c), r >= c; the lanes take
  // the entries (one round up to P = 7), so that every stage below is a
  // few dependent FP64 operations deep (this part's FP64 pipe does two
  // lanes per clock per SM, so depth, not width, sets the time)
  auto rc_of = [](int q, int &r, int &c) {
    r = 0;
    while ((r + 1) * (r + 2) / 2 <= q) ++r;
    c = q - r * (r + 1) / 2;
  };
  const int NP = P * (P + 1) / 2;
  for (int q = lane; q < P * P; q += 32) {
    const int r = q / P, c = q - r * P;
    A[r][c] = (r >= c ? tot[tri(r, c)] : tot[tri(c, r)]) + (r == c ? 1.0 : 0.0);
    T[r][c] = 0.0;
  }
  __syncwarp();
  // S + I = U U' with U upper, last pivot first; U goes to the upper
  // triangle of A (diagonal included), the lower triangle holds the
  // remaining leading block, rd[k] = 1 / U[k][k].
  bool ok = true;
  for (int k = P - 1; k >= 0; --k) {
    const double dk = A[k][k];
    ok = ok && (dk > 0.0);
    const double rs = rsqrt(dk);
    __syncwarp();
    if (lane < k) A[lane][k] = A[k][lane] * rs;
    if (lane == k) {
      A[k][k] = dk * rs;
      rd[k] = rs;
    }
    __syncwarp();
    for (int q = lane; q < k * (k + 1) / 2; q += 32) {
      int i, j;
      rc_of(q, i, j);
      A[i][j] -= A[i][k] * A[j][k];
    }
    __syncwarp();
  }
  if (ok) {
    // T: the Bartlett factor, lower; sqrt(chi^2) on the diagonal and
    // normals below it (drawn by the last colour-0 block of this sweep,
    // or supplied)
    const int nw = P * (P - 1) / 2;
    if (lane < P) T[lane][lane] = supplied ? sqrt(sup.chi2[lane]) : __ldcg(ch.wdraw + lane);
    if (lane < nw) {
      int i = 1;
      while ((i + 1) * i / 2 <= lane) ++i;  // row i: lane in [i(i-1)/2, i(i+1)/2)
      const int j = lane - i * (i - 1) / 2;
      T[i][j] = supplied ? sup.wnorm[lane] : __ldcg(ch.wdraw + kMaxP + lane);
    }
    __syncwarp();
    // B = L T with L = U^-T, by forward substitution U' B = T (row i:
    // B[i][.] = (T[i][.] - sum_{k<i} U[k][i] B[k][.]) / U[i][i]), right-
    // looking so that each row costs two dependent FP64 operations; B is
    // lower triangular like T
    for (int q = lane; q < NP; q += 32) {
      int i, j;
      rc_of(q, i, j);
      B[i][j] = T[i][j];
    }
    __syncwarp();
    for (int i = 0; i < P; ++i) {
      if (lane <= i) B[i][lane] *= rd[i];
      __syncwarp();
      // rows r > i, columns j <= i: (P - 1 - i)(i + 1) <= 16 entries
      const int nr = P - 1 - i;
      if (lane < nr * (i + 1)) {
        const int r = i + 1 + lane / (i + 1), j = lane - (lane / (i + 1)) * (i + 1);
        B[r][j] -= A[i][r] * B[i][j];
      }
      __syncwarp();
    }
    __syncwarp();
    bool fin = true;
    for (int q = lane; q < NP; q += 32) {  // Omega = B B', both triangles
      int i, j;
      rc_of(q, i, j);
      double s = 0.0;
      for (int k = 0; k <= j; ++k) s += B[i][k] * B[j][k];
      A[i][j] = s;  // A is free again
      A[j][i] = s;
      fin = fin && isfinite(s);
    }
    fin = __all_sync(0xffffffffu, fin);
    __syncwarp();
    if (fin) {
      for (int q = lane; q < P * P; q += 32) {
        const int r = q / P, c = q - r * P;
        ch.omega_d[q] = A[r][c];
        ch.omega_f[q] = (float)A[r][c];
      }
    } else {
      err |= kErrNaN;
    }
  } else {
    err |= kErrWishart;
  }
  if (lane < P) ch.colmean[lane] = (float)(tot[kMaxPairs + lane] / (double)d.V);
  if (lane == 0) {
    // beta_WM | Z, beta ~ N(var * sum_v WM_v sum_i (Z_iv - x_i' beta_v),
    // var = 1 / (N sum_v WM_v^2)) (updateBetaGPU, covarGPU.cu:680-720)
    float bw = *ch.wm_beta;
    if (ch.wm_update && !supplied) {
      const double var = 1.0 / ((double)d.N * d.wm2);
      const uint4 r = philox1(make_uint4(0u, 0u, sw, cid | kTagWm), ch.key0, ch.key1);
      const double z = (double)normal_of(pick4(r, 0));
      const float nb = (float)(var * tot[kWmOff] + sqrt(var) * z);
      if (isfinite(nb)) {
        bw = nb;
        *ch.wm_beta = nb;
      } else {
        err |= kErrNaN;
      }
    }
    if (kept) *ch.wm_sum += (double)bw;  // MWM of mcmc.cpp:636
  }
  err = __reduce_or_sync(0xffffffffu, err);
  if (lane == 0) {
    if (err) {
      atomicOr(ch.status, err);
      atomicOr(ch.any_status, err);
    }
    ch.sweep[1] = sweep + 1;
    if (kept) *ch.nkept = nk + 1;
    ch.done[1] = 0u;
    __threadfence();
  }
}

}  // namespace bsg
