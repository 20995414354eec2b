// bsg_fp64.cu -- the colour kernel of FP64 chains: the whole sweep in double
// precision on the sampler's Philox counters (latent draws, X'Z, the
// conditional precision and its Cholesky, the coefficient draw, the Omega
// pair sums, the Bartlett variates and the posterior sums).  A chain in this
// mode is the GPU form of the FP64 oracle chain (the C restatement of
// covar.cpp:121-325 and mcmc.cpp:584-651 on the same counters), fast enough
// to run the long reference chains that the FP32 sampler's maps are
// measured against at the brain-sized studies, where the CPU would take
// days.  It is written for agreement, not speed: one thread per voxel,
// subjects in order, CUDA's double-precision normcdf / normcdfinv.
#include "bsg_wishart.cuh"

namespace bsg {
namespace {

constexpr int kF64Chunk = 512;  // subjects of the design staged per pass

// N(0,1) truncated to (a, +inf) by inversion of u(k), in FP64:
// t = Phi^-1(Phi(a) + u Q(a)).  For a >= 0 the argument is at least 1/2 and
// t = -Phi^-1(Q(a) (1 - u)); for a < 0 the small Phi(a) keeps its relative
// precision and Q(a) = 1 - Phi(a) is at least 1/2.  1 - u = u(~k).
__device__ double tn_lower_inv_d(double a, uint32_t k) {
  const double uc = u_of_d(~k);
  if (a >= 0.0) return -normcdfinv(normcdf(-a) * uc);
  const double pa = normcdf(a), qa = 1.0 - pa;
  const double pl = pa + u_of_d(k) * qa;
  return pl < 0.5 ? normcdfinv(pl) : -normcdfinv(qa * uc);
}

// a > kATail: the Robert (1995) exponential-proposal rejection of
// tn_lower_tail in FP64, on the same counters and attempt order.
__device__ __noinline__ double tn_lower_tail_d(double a, uint32_t i, uint32_t v,
                                               uint32_t sweep, uint32_t c3,
                                               uint32_t key0, uint32_t key1, int *ok) {
  const double as = 0.5 * (a + sqrt(a * a + 4.0));
  for (int q = 0; q < kTailMax / 2; ++q) {
    const uint4 r = philox1(make_uint4(i * 8u + (uint32_t)q, v, sweep, c3), key0, key1);
    double x = a - log(u_of_d(r.x)) / as, d = x - as;
    if (log(u_of_d(r.y)) < -0.5 * d * d) return x;
    x = a - log(u_of_d(r.z)) / as;
    d = x - as;
    if (log(u_of_d(r.w)) < -0.5 * d * d) return x;
  }
  *ok = 0;
  return a;
}

// Abramowitz & Stegun 26.2.17 in FP64, as the reference's CPU compute_prb
// evaluates it (covar.cpp:327-348).
__device__ double prob_sdnorm_d(double x) {
  const double b1 = 0.319381530, b2 = -0.356563782, b3 = 1.781477937;
  const double b4 = -1.821255978, b5 = 1.330274429, p = 0.2316419;
  const double c = 0.39894228;
  const double t = 1.0 / (1.0 + p * fabs(x));
  const double tail = c * exp(-x * x / 2.0) * t *
                      (t * (t * (t * (t * b5 + b4) + b3) + b2) + b1);
  return x >= 0.0 ? 1.0 - tail : tail;
}

// Sum of one value over the blocks' partials (value-major), in a fixed
// order: lane l takes the blocks l, l + 32, ...; then the lanes are
// combined.  One warp.
__device__ double sum_rows(const double *base, int nrow, int lane) {
  double s = 0.0;
  for (int r = lane; r < nrow; r += 32) s += __ldcg(base + r);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  return s;
}

template <int P>
__global__ void __launch_bounds__(kF64Threads)
    fp64_colour_kernel(const DatasetDev *__restrict__ dsv, ChainDev *__restrict__ chv,
                       const BlockMap *__restrict__ map, int colour) {
  constexpr int NT = P * (P + 1) / 2;
  __shared__ float Xs[kF64Chunk * P];
  __shared__ double Om[P * P], Xtx[P * P];
  __shared__ double red[kF64Threads / 32][kFusedVals];
  __shared__ double tot[kFusedVals];
  __shared__ int is_last;

  const BlockMap bm = map[blockIdx.x];
  ChainDev &ch = chv[bm.chain];
  const DatasetDev &d = dsv[ch.dataset];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nc = d.n[colour];
  const int j = bm.start + tid;
  const bool active = j < nc;
  const int N = d.N, Vp = d.Vp;
  const long long sweep_ll = ch.sweep[colour];
  const uint32_t sweep = (uint32_t)sweep_ll, cid = ch.chain_id << 8;
  const bool kept =
      sweep_ll > ch.burnin && (sweep_ll % (ch.thin > 0 ? ch.thin : 1)) == 0;
  const double *b64 = ch.beta64;

  double beta[P], acc[P], bwm = 0.0;
  int v = 0, sc = 0;
  if (active) {
    sc = d.nb[colour][j];
    v = d.vidx[colour][j];
    bwm = (double)*ch.wm_beta * (d.wm ? (double)d.wm[v] : 1.0);
  }
#pragma unroll
  for (int p = 0; p < P; ++p) {
    beta[p] = active ? b64[(size_t)p * Vp + sc] : 0.0;
    acc[p] = 0.0;
  }
  int ok = 1;
  const uint32_t *yb = d.ybits[colour];

  // ---- latent Z_iv for every subject, accumulated into X'(Z - b_WM WM)
  // (updateZ, covar.cpp:302-325, and the b of Spat_Coefff, covar.cpp:142-150)
  for (int i0 = 0; i0 < N; i0 += kF64Chunk) {
    const int cn = min(kF64Chunk, N - i0);
    __syncthreads();
    for (int t = tid; t < P * cn; t += blockDim.x) {
      const int p = t / cn, ii = t - p * cn;
      Xs[ii * P + p] = d.covar[(size_t)p * N + i0 + ii];
    }
    __syncthreads();
    if (!active) continue;
    uint4 r = make_uint4(0, 0, 0, 0);
    uint32_t yw = 0;
    for (int ii = 0; ii < cn; ++ii) {
      const int i = i0 + ii;  // i0 is a multiple of 32
      if ((i & 31) == 0) yw = __ldg(yb + (size_t)(i >> 5) * nc + j);
      if ((i & 3) == 0)
        r = philox1(make_uint4((uint32_t)(i >> 2), (uint32_t)v, sweep, cid | kTagZ),
                    ch.key0, ch.key1);
      double x[P], mu = bwm;
#pragma unroll
      for (int p = 0; p < P; ++p) {
        x[p] = (double)Xs[ii * P + p];
        mu += beta[p] * x[p];
      }
      const bool y = (yw >> (i & 31)) & 1u;
      const double a = y ? -mu : mu;
      const double t =
          a <= (double)kATail
              ? tn_lower_inv_d(a, pick4(r, i & 3))
              : tn_lower_tail_d(a, (uint32_t)i, (uint32_t)v, sweep, cid | kTagZTail,
                                ch.key0, ch.key1, &ok);
      const double zr = mu + (y ? t : -t) - bwm;  // Z - b_WM WM
#pragma unroll
      for (int p = 0; p < P; ++p) acc[p] += x[p] * zr;
    }
  }

  // ---- beta_v | rest (Spat_Coefff, covar.cpp:142-180), production form
  const long long nk = *ch.nkept;
  for (int t = tid; t < P * P; t += blockDim.x) {
    Om[t] = ch.omega_d[t];
    Xtx[t] = (double)d.xtx[t];
  }
  __syncthreads();
  int err = ok ? 0 : kErrTnCap;
  double bnew[P], pv[NT];
#pragma unroll
  for (int q = 0; q < NT; ++q) pv[q] = 0.0;
  if (active) {
    double sumV[P];
#pragma unroll
    for (int p = 0; p < P; ++p) sumV[p] = 0.0;
    for (int t = 1; t <= 6; ++t) {
      const int sn = d.nb[colour][(size_t)t * nc + j];
#pragma unroll
      for (int p = 0; p < P; ++p) sumV[p] += b64[(size_t)p * Vp + sn];
    }
    const unsigned nbm = d.nbm[colour][j];
    const double nnb = (double)__popc(nbm);
    double b[P], Q[NT], e[P];
#pragma unroll
    for (int a = 0; a < P; ++a) {
      double s = acc[a];
#pragma unroll
      for (int q = 0; q < P; ++q) s += Om[q + a * P] * sumV[q];
      b[a] = s;
#pragma unroll
      for (int q = 0; q <= a; ++q) Q[tri(a, q)] = Xtx[q + a * P] + nnb * Om[q + a * P];
    }
    const bool okc = chol_packed<P>(Q);
#pragma unroll
    for (int p0 = 0; p0 < P; p0 += 4) {
      const uint4 rb = philox1(
          make_uint4((uint32_t)(p0 >> 2), (uint32_t)v, sweep, cid | kTagBeta), ch.key0,
          ch.key1);
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (p0 + q < P) e[p0 + q] = normal_of_d(pick4(rb, q));
    }
    // Q = G G': beta = G^-T (G^-1 b + e), mean Q^-1 b and covariance Q^-1
    solve_lower<P>(Q, b);
#pragma unroll
    for (int p = 0; p < P; ++p) bnew[p] = b[p] + e[p];
    solve_upper<P>(Q, bnew);
    bool fin = true;
#pragma unroll
    for (int p = 0; p < P; ++p) fin = fin && isfinite(bnew[p]);
    if (okc && fin) {
#pragma unroll
      for (int p = 0; p < P; ++p) {
        ch.beta64[(size_t)p * Vp + sc] = bnew[p];
        ch.beta[(size_t)p * Vp + sc] = (float)bnew[p];
      }
    } else {
#pragma unroll
      for (int p = 0; p < P; ++p) bnew[p] = beta[p];
    }
    err |= (okc ? 0 : kErrChol) | ((okc && !fin) ? kErrNaN : 0);

    // ---- posterior running sums of the kept sweep (mcmc.cpp:637-645)
    if (kept) {
#pragma unroll
      for (int p = 0; p < P; ++p) {
        ch.acc_sum[(size_t)p * d.V + v] += bnew[p];
        ch.acc_sq[(size_t)p * d.V + v] += bnew[p] * bnew[p];
      }
#pragma unroll
      for (int g2 = 0; g2 < P; ++g2)
        if (g2 < d.S) ch.prb_sum[(size_t)g2 * d.V + v] += prob_sdnorm_d(bnew[g2] + bwm);
    }

    // ---- Omega pair products of the voxel's edges (colour 1 sees every
    // in-mask edge once), with the reference's indicator (covar.cpp:235-253)
    if (colour == 1) {
      for (int t = 0; t < 6; ++t) {
        const int sn = d.nb[1][(size_t)(t + 1) * nc + j];
        const bool fwd = t & 1;
        const bool nin = (nbm >> t) & 1u;
        double dd[P];
        bool ind[P];
#pragma unroll
        for (int p = 0; p < P; ++p) {
          const double bn = b64[(size_t)p * Vp + sn];
          dd[p] = bnew[p] - bn;
          ind[p] = fwd ? (bn != 0.0) : (nin && bnew[p] != 0.0);
        }
#pragma unroll
        for (int r2 = 0; r2 < P; ++r2)
          if (ind[r2]) {
#pragma unroll
            for (int c2 = 0; c2 <= r2; ++c2) pv[tri(r2, c2)] += dd[r2] * dd[c2];
          }
      }
    }
  } else {
#pragma unroll
    for (int p = 0; p < P; ++p) bnew[p] = 0.0;  // no column-sum share
  }
  if (err) {
    atomicOr(ch.status, err);
    atomicOr(ch.any_status, err);
  }

  // ---- block partials (FP64 warp trees), the last block of each colour
  // sums them in block order; colour 0's also draws the Bartlett variates,
  // colour 1's draws Omega
  constexpr int kColOff = kMaxPairs;
  constexpr int NV = NT + P;
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    if (colour == 0 && q < NT) continue;
    double val = q < NT ? pv[q] : bnew[q - NT];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) val += __shfl_xor_sync(0xffffffffu, val, o);
    if (lane == 0) red[warp][q < NT ? q : kColOff + (q - NT)] = val;
  }
  __syncthreads();
  const int nwarp = kF64Threads / 32;
  const int lb = bm.start / kF64Threads;
  const int nblk = max(1, (nc + kF64Threads - 1) / kF64Threads);
  if (colour == 0) {
    if (tid < P) {
      double s = 0.0;
      for (int w = 0; w < nwarp; ++w) s += red[w][kColOff + tid];
      ch.partials0[(size_t)tid * ch.pstride0 + lb] = s;
      __threadfence();
    }
    __syncthreads();
    if (tid == 0) is_last = atomicAdd(ch.done, 1u) == (unsigned)(nblk - 1);
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    for (int m = warp; m < P; m += nwarp) {
      const double s = sum_rows(ch.partials0 + (size_t)m * ch.pstride0, nblk, lane);
      if (lane == 0) ch.tot0[m] = s;
    }
    if (warp == nwarp - 1) {
      const int e = __reduce_or_sync(0xffffffffu,
                                     wishart_draws<true>(ch, d, sweep_ll, lane, ch.wdraw));
      if (e && lane == 0) {
        atomicOr(ch.status, e);
        atomicOr(ch.any_status, e);
      }
    }
    __syncthreads();
    if (tid == 0) {
      ch.sweep[0] = sweep_ll + 1;
      ch.done[0] = 0u;
      __threadfence();
    }
    return;
  }
  if (tid < NV) {
    const int q = tid < NT ? tid : kColOff + (tid - NT);
    double s = 0.0;
    for (int w = 0; w < nwarp; ++w) s += red[w][q];
    ch.partials1[(size_t)q * ch.pstride1 + lb] = s;
    __threadfence();
  }
  __syncthreads();
  if (tid == 0) is_last = atomicAdd(ch.done + 1, 1u) == (unsigned)(nblk - 1);
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  for (int m = warp; m < NV; m += nwarp) {
    const int q = m < NT ? m : kColOff + (m - NT);
    double s = sum_rows(ch.partials1 + (size_t)q * ch.pstride1, nblk, lane);
    if (q >= kColOff) s += __ldcg(ch.tot0 + (q - kColOff));
    if (lane == 0) tot[q] = s;
  }
  __syncthreads();
  if (warp == 0) wishart_warp(ch, d, tot, sweep_ll, kept, nk, 0, Supplied{}, lane);
}

}  // namespace

cudaError_t launch_fp64(int P, const DatasetDev *ds, ChainDev *ch, const BlockMap *map,
                        int nblocks, int colour, cudaStream_t st) {
  if (nblocks <= 0) return cudaSuccess;
  switch (P) {
#define BSG_F64(PP)                                                             \
  case PP:                                                                      \
    fp64_colour_kernel<PP><<<nblocks, kF64Threads, 0, st>>>(ds, ch, map, colour); \
    break;
    BSG_F64(1)
    BSG_F64(2)
    BSG_F64(3)
    BSG_F64(4)
    BSG_F64(5)
    BSG_F64(6)
    BSG_F64(7)
    BSG_F64(8)
#undef BSG_F64
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace bsg
