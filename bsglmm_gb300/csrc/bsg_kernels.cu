// bsg_kernels.cu -- the post-sweep pass (Omega neighbour-pair reduction,
// column sums, FP64 posterior accumulators, lesion probabilities and the
// Wishart tail), the lesion-probability map, outcome bit packing, and the
// dispatcher of the fused colour kernel.
#include "bsg_device.cuh"

namespace bsg {

cudaError_t launch_fused_l1(int, int, bool, const DatasetDev *, ChainDev *,
                            const BlockMap *, int, int, const Supplied &,
                            cudaStream_t);
cudaError_t launch_fused_l2(int, int, bool, const DatasetDev *, ChainDev *,
                            const BlockMap *, int, int, const Supplied &,
                            cudaStream_t);
cudaError_t launch_fused_l4(int, int, bool, const DatasetDev *, ChainDev *,
                            const BlockMap *, int, int, const Supplied &,
                            cudaStream_t);
cudaError_t launch_fused_l8(int, int, bool, const DatasetDev *, ChainDev *,
                            const BlockMap *, int, int, const Supplied &,
                            cudaStream_t);

bool fused_supported(int P, int lpv, int threads) {
  if (P < 1 || P > kMaxP) return false;
  if (lpv != 1 && lpv != 2 && lpv != 4 && lpv != 8) return false;
  if (threads != 64 && threads != 128 && threads != 256) return false;
  return true;
}

cudaError_t launch_fused(int P, int lpv, int threads, bool supplied,
                         const DatasetDev *ds, ChainDev *ch,
                         const BlockMap *map, int nblocks, int colour,
                         const Supplied &sup, cudaStream_t st) {
  switch (lpv) {
    case 1:
      return launch_fused_l1(P, threads, supplied, ds, ch, map, nblocks,
                             colour, sup, st);
    case 2:
      return launch_fused_l2(P, threads, supplied, ds, ch, map, nblocks,
                             colour, sup, st);
    case 4:
      return launch_fused_l4(P, threads, supplied, ds, ch, map, nblocks,
                             colour, sup, st);
    case 8:
      return launch_fused_l8(P, threads, supplied, ds, ch, map, nblocks,
                             colour, sup, st);
    default:
      return cudaErrorInvalidValue;
  }
}

// ----------------------------------------------------- FP64 Wishart tail --
// Dense helpers on element (r, c) at A[c + r*n] (cholesky.cpp layout).
__device__ static bool chol_full(double *A, int n) {
  for (int k = 0; k < n; ++k) {
    double dkk = A[k + k * n];
    if (!(dkk > 0.0)) return false;
    dkk = sqrt(dkk);
    A[k + k * n] = dkk;
    for (int j = k + 1; j < n; ++j) A[k + j * n] /= dkk;
    for (int j = k + 1; j < n; ++j)
      for (int i = j; i < n; ++i) A[j + i * n] -= A[k + i * n] * A[k + j * n];
  }
  return true;
}

// Inverse of G G' from the lower factor (cholesky.cpp:55-86 scheme).
__device__ static void chol_inverse(const double *G, int n, double *out) {
  double col[kMaxP];
  for (int k = 0; k < n; ++k) {
    for (int i = 0; i < n; ++i) col[i] = (i == k) ? 1.0 : 0.0;
    for (int i = 0; i < n; ++i) {
      double s = 0.0;
      for (int j = 0; j < i; ++j) s += G[j + i * n] * col[j];
      col[i] = (col[i] - s) / G[i + i * n];
    }
    for (int i = n - 1; i >= 0; --i) {
      double s = 0.0;
      for (int j = i + 1; j < n; ++j) s += G[i + j * n] * col[j];
      col[i] = (col[i] - s) / G[i + i * n];
    }
    for (int i = 0; i < n; ++i) out[k + i * n] = col[i];
  }
}

// Marsaglia & Tsang (2000) gamma(a, 1); a < 1 through the U^(1/a) boost.
// Attempt t of slot uses counter (slot*64 + t, 0, sweep, chain<<8|GAMMA).
__device__ static double gamma_mt(double a, uint32_t slot, uint32_t sweep,
                                  uint32_t c3, uint32_t k0, uint32_t k1,
                                  int *err) {
  const bool boost = a < 1.0;
  const double aa = boost ? a + 1.0 : a;
  const double dd = aa - 1.0 / 3.0, c = 1.0 / sqrt(9.0 * dd);
  for (int t = 0; t < kGammaMax; ++t) {
    const uint4 r = philox1(make_uint4(slot * 64u + (uint32_t)t, 0u, sweep, c3),
                            k0, k1);
    const double x = (double)normal_of(r.x);
    const double cx = c * x;
    if (!(cx > -1.0)) continue;
    const double v3 = (1.0 + cx) * (1.0 + cx) * (1.0 + cx);
    const double lhs = log(u_of_d(r.y));
    const double rhs = 0.5 * x * x + dd * (1.0 - v3 + 3.0 * log1p(cx));
    if (lhs < rhs) return dd * v3 * (boost ? pow(u_of_d(r.z), 1.0 / a) : 1.0);
  }
  *err |= kErrGammaCap;
  return dd;
}

// Omega | beta ~ Wishart(df, (S + I)^-1) by the Bartlett construction of
// rwishart2 (cholesky.cpp:245-286) after chol -> invert -> chol
// (covar.cpp:286-291, covarGPU.cu:1099-1104), all in FP64.
__device__ static void wishart_tail(ChainDev &ch, const DatasetDev &d,
                                    const double *tot, long long sweep,
                                    bool kept, long long nk, int supplied,
                                    const Supplied &sup) {
  const int P = d.P;
  double A[kMaxP * kMaxP], Ai[kMaxP * kMaxP], T[kMaxP * kMaxP];
  double B[kMaxP * kMaxP];
  int err = 0;
  for (int r = 0; r < P; ++r)
    for (int c = 0; c <= r; ++c)
      A[c + r * P] = A[r + c * P] = tot[tri(r, c)] + (r == c ? 1.0 : 0.0);
  bool ok = chol_full(A, P);
  if (ok) {
    chol_inverse(A, P, Ai);
    ok = chol_full(Ai, P);
  }
  if (ok) {
    const double df = (double)d.V + (double)ch.df_offset;
    const uint32_t cid = ch.chain_id << 8, sw = (uint32_t)sweep;
    for (int i = 0; i < P * P; ++i) T[i] = 0.0;
    for (int i = 0; i < P; ++i) {
      const double c2 = supplied ? sup.chi2[i]
                                 : 2.0 * gamma_mt(0.5 * (df - i), (uint32_t)i,
                                                  sw, cid | kTagGamma, ch.key0,
                                                  ch.key1, &err);
      T[i + i * P] = sqrt(c2);
      for (int j = 0; j < i; ++j) {
        const int m = i * (i - 1) / 2 + j;
        double z;
        if (supplied) {
          z = sup.wnorm[m];
        } else {
          const uint4 r = philox1(make_uint4((uint32_t)(m >> 2), 0u, sw,
                                             cid | kTagWNorm),
                                  ch.key0, ch.key1);
          z = (double)normal_of(pick4(r, m & 3));
        }
        T[j + i * P] = z;
      }
    }
    for (int i = 0; i < P; ++i)
      for (int j = 0; j <= i; ++j) {
        double s = 0.0;
        for (int k = j; k <= i; ++k) s += Ai[k + i * P] * T[j + k * P];
        B[j + i * P] = s;
      }
    bool fin = true;
    for (int i = 0; i < P; ++i)
      for (int j = 0; j < P; ++j) {
        const int K = i < j ? i : j;
        double s = 0.0;
        for (int k = 0; k <= K; ++k) s += B[k + i * P] * B[k + j * P];
        A[j + i * P] = s;
        fin = fin && isfinite(s);
      }
    if (fin) {
      for (int i = 0; i < P * P; ++i) {
        ch.omega_d[i] = A[i];
        ch.omega_f[i] = (float)A[i];
      }
    } else {
      err |= kErrNaN;
    }
  } else {
    err |= kErrWishart;
  }
  for (int p = 0; p < P; ++p)
    ch.colmean[p] = (float)(tot[kMaxPairs + p] / (double)d.V);
  if (err) atomicOr(ch.status, err);
  *ch.sweep = sweep + 1;
  if (kept) *ch.nkept = nk + 1;
  *ch.done = 0u;
  __threadfence();
}

// ------------------------------------------------------ post-sweep pass --
// One pass over every in-mask voxel after both colours: the pair sums of
// Spat_Coef_Prec (covarGPU.cu:953-1013, covar.cpp:220-262; the indicator
// tests the row coefficient of the forward neighbour), the column sums of
// covarGPU.cu:563-583, and on kept sweeps the FP64 Welford accumulators of
// beta and of the lesion probability (mcmc.cpp:627-649).  Block partials
// are summed in block order by the last block to arrive, which then draws
// Omega: the result is bitwise reproducible.
__global__ void __launch_bounds__(kPostThreads)
    post_sweep_kernel(const DatasetDev *__restrict__ dsv,
                      ChainDev *__restrict__ chv,
                      const BlockMap *__restrict__ map, int supplied,
                      Supplied sup) {
  __shared__ double red[kPostThreads / 32][kPostVals];
  __shared__ double tot[kPostVals];
  __shared__ int is_last;

  const BlockMap bm = map[blockIdx.x];
  ChainDev &ch = chv[bm.chain];
  const DatasetDev &d = dsv[ch.dataset];
  const int P = d.P, S = d.S, V = d.V, Vp = d.Vp;
  const int n0 = d.n[0], ntot = n0 + d.n[1];
  const long long sweep = *ch.sweep, nk = *ch.nkept;
  const int thin = ch.thin > 0 ? ch.thin : 1;
  const bool kept = sweep > ch.burnin && (sweep % thin) == 0;
  const double inv_n = 1.0 / (double)(nk + 1);
  const int npairs = P * (P + 1) / 2;

  double accp[kMaxPairs], cs[kMaxP];
#pragma unroll
  for (int q = 0; q < kMaxPairs; ++q) accp[q] = 0.0;
#pragma unroll
  for (int p = 0; p < kMaxP; ++p) cs[p] = 0.0;

  for (int t = 0; t < kPostPerThread; ++t) {
    const int pos = bm.start + threadIdx.x + t * kPostThreads;
    if (pos >= ntot) break;
    const int c = pos < n0 ? 0 : 1;
    const int j = c ? pos - n0 : pos;
    const int nc = d.n[c];
    const int32_t *nbp = d.nb[c];
    const int sc = nbp[j];
    float bs[kMaxP];
#pragma unroll
    for (int p = 0; p < kMaxP; ++p) {
      bs[p] = p < P ? ch.beta[(size_t)p * Vp + sc] : 0.f;
      cs[p] += (double)bs[p];
    }
    float pv[kMaxPairs];
#pragma unroll
    for (int q = 0; q < kMaxPairs; ++q) pv[q] = 0.f;
#pragma unroll
    for (int f = 0; f < 3; ++f) {  // forward neighbours +x, +y, +z
      const int sn = nbp[(size_t)(2 + 2 * f) * nc + j];
      float dd[kMaxP];
      bool ind[kMaxP];
#pragma unroll
      for (int p = 0; p < kMaxP; ++p) {
        const float bn = p < P ? ch.beta[(size_t)p * Vp + sn] : 0.f;
        dd[p] = bs[p] - bn;
        ind[p] = bn != 0.f;
      }
#pragma unroll
      for (int r = 0; r < kMaxP; ++r)
        if (r < P && ind[r]) {
#pragma unroll
          for (int c2 = 0; c2 <= r; ++c2) pv[tri(r, c2)] += dd[r] * dd[c2];
        }
    }
#pragma unroll
    for (int q = 0; q < kMaxPairs; ++q)
      if (q < npairs) accp[q] += (double)pv[q];

    if (kept) {
      const int v = d.vidx[c][j];
#pragma unroll
      for (int p = 0; p < kMaxP; ++p)
        if (p < P) {
          const double x = (double)bs[p];
          double *mp = ch.acc_mean + (size_t)p * V + v;
          double mn = *mp;
          const double dl = x - mn;
          mn += dl * inv_n;
          *mp = mn;
          ch.acc_m2[(size_t)p * V + v] += dl * (x - mn);
        }
      const float bwm = ch.beta_wm * (d.wm ? d.wm[v] : 1.f);
#pragma unroll
      for (int g = 0; g < kMaxP; ++g)
        if (g < S) {
          const double pr = (double)prob_sdnorm(bs[g] + bwm);
          double *pp = ch.acc_prb + (size_t)g * V + v;
          *pp += (pr - *pp) * inv_n;
        }
    }
  }

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < kPostVals; ++q) {
    const bool live = q < kMaxPairs ? q < npairs : (q - kMaxPairs) < P;
    if (!live) continue;
    double val = q < kMaxPairs ? accp[q] : cs[q - kMaxPairs];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) val += __shfl_xor_sync(0xffffffffu, val, o);
    if (lane == 0) red[warp][q] = val;
  }
  __syncthreads();
  const int lb = bm.start / (kPostThreads * kPostPerThread);
  if (threadIdx.x < kPostVals) {
    const int q = threadIdx.x;
    const bool live = q < kMaxPairs ? q < npairs : (q - kMaxPairs) < P;
    double s = 0.0;
    if (live)
      for (int w = 0; w < kPostThreads / 32; ++w) s += red[w][q];
    ch.partials[(size_t)lb * kPostVals + q] = s;
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned prev = atomicAdd(ch.done, 1u);
    is_last = prev == (unsigned)(ch.post_blocks - 1);
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  if (threadIdx.x < kPostVals) {
    double s = 0.0;
    for (int b = 0; b < ch.post_blocks; ++b)
      s += __ldcg(ch.partials + (size_t)b * kPostVals + threadIdx.x);
    tot[threadIdx.x] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) wishart_tail(ch, d, tot, sweep, kept, nk, supplied, sup);
}

cudaError_t launch_post(const DatasetDev *ds, ChainDev *ch,
                        const BlockMap *map, int nblocks, bool supplied,
                        const Supplied &sup, cudaStream_t st) {
  if (nblocks <= 0) return cudaSuccess;
  post_sweep_kernel<<<nblocks, kPostThreads, 0, st>>>(ds, ch, map,
                                                      supplied ? 1 : 0, sup);
  return cudaGetLastError();
}

// ------------------------------------------------- lesion probability --
// compute_prbGPU / ProbSDNormGPU (covarGPU.cu:1723-1747, 1814-1824).
__global__ void prb_kernel(const DatasetDev *__restrict__ dsv,
                           const ChainDev *__restrict__ chv, int chain,
                           float *__restrict__ prb) {
  const ChainDev &ch = chv[chain];
  const DatasetDev &d = dsv[ch.dataset];
  const int n0 = d.n[0], ntot = n0 + d.n[1];
  for (int pos = blockIdx.x * blockDim.x + threadIdx.x; pos < ntot;
       pos += gridDim.x * blockDim.x) {
    const int c = pos < n0 ? 0 : 1;
    const int j = c ? pos - n0 : pos;
    const int sc = d.nb[c][j], v = d.vidx[c][j];
    const float bwm = ch.beta_wm * (d.wm ? d.wm[v] : 1.f);
    for (int g = 0; g < d.S; ++g)
      prb[(size_t)g * d.V + v] = prob_sdnorm(ch.beta[(size_t)g * d.Vp + sc] + bwm);
  }
}

cudaError_t launch_prb(const DatasetDev *ds, const ChainDev *ch, int chain,
                       const DatasetDev &dh, float *prb, cudaStream_t st) {
  const int ntot = dh.n[0] + dh.n[1];
  if (ntot <= 0) return cudaSuccess;
  const int blocks = (ntot + 255) / 256;
  prb_kernel<<<blocks, 256, 0, st>>>(ds, ch, chain, prb);
  return cudaGetLastError();
}

// --------------------------------------------------- outcome bit packing --
// data[i*V + v] bytes -> ybits[w*nc + j], bit b = subject 32w + b of the
// voxel at colour position j.  Values other than 0/1 raise kErrInput.
__global__ void pack_kernel(const uint8_t *__restrict__ bytes, int N, int V,
                            int nc, const int32_t *__restrict__ vidx,
                            uint32_t *__restrict__ ybits, int *status) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int w = blockIdx.y;
  if (j >= nc) return;
  const int v = vidx[j];
  uint32_t word = 0;
  int bad = 0;
  for (int b = 0; b < 32; ++b) {
    const int i = 32 * w + b;
    if (i < N) {
      const uint8_t y = bytes[(size_t)i * V + v];
      word |= (uint32_t)(y == 1) << b;
      bad |= y > 1;
    }
  }
  ybits[(size_t)w * nc + j] = word;
  if (bad) atomicOr(status, kErrInput);
}

cudaError_t launch_pack(const uint8_t *bytes, int N, int V, int nc,
                        const int32_t *vidx, uint32_t *ybits, int *status,
                        cudaStream_t st) {
  if (nc <= 0 || N <= 0) return cudaSuccess;
  const int W = (N + 31) / 32;
  dim3 grid((nc + 255) / 256, W);
  pack_kernel<<<grid, 256, 0, st>>>(bytes, N, V, nc, vidx, ybits, status);
  return cudaGetLastError();
}

}  // namespace bsg
