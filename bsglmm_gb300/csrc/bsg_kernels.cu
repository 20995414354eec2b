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

// In-place Cholesky of the lower triangle of the P x P matrix A (row-major
// A[r*kMaxP + c]) by one warp, rows across lanes (the outer-product scheme
// of cholesky.cpp:13-33).  Returns false (warp-uniform) on a non-positive
// pivot.
__device__ static bool chol_warp(double (*A)[kMaxP], int P, int lane) {
  bool ok = true;
  for (int k = 0; k < P; ++k) {
    const double d = A[k][k];
    ok = ok && (d > 0.0);
    const double s = sqrt(d);
    __syncwarp();
    if (lane == k) A[k][k] = s;
    if (lane > k && lane < P) A[lane][k] /= s;
    __syncwarp();
    if (lane > k && lane < P)
      for (int j = k + 1; j <= lane; ++j) A[lane][j] -= A[lane][k] * A[j][k];
    __syncwarp();
  }
  return ok;
}

// Omega | beta ~ Wishart(df, (S + I)^-1) by the Bartlett construction of
// rwishart2 (cholesky.cpp:245-286) after chol -> invert -> chol
// (covar.cpp:286-291, covarGPU.cu:1099-1104), FP64, one warp.
__device__ static void wishart_warp(ChainDev &ch, const DatasetDev &d,
                                    const double *tot, long long sweep,
                                    bool kept, long long nk, int supplied,
                                    const Supplied &sup, int lane) {
  __shared__ double A[kMaxP][kMaxP], Ai[kMaxP][kMaxP], T[kMaxP][kMaxP],
      B[kMaxP][kMaxP];
  const int P = d.P;
  int err = 0;
  if (lane < P)
    for (int c = 0; c < P; ++c) {
      const int r = lane;
      A[r][c] = (r >= c ? tot[tri(r, c)] : tot[tri(c, r)]) + (r == c ? 1.0 : 0.0);
      T[r][c] = 0.0;
    }
  __syncwarp();
  bool ok = chol_warp(A, P, lane);
  if (ok) {
    // column `lane` of (G G')^-1 by forward then back substitution
    if (lane < P) {
      double col[kMaxP];
      for (int i = 0; i < P; ++i) col[i] = (i == lane) ? 1.0 : 0.0;
      for (int i = 0; i < P; ++i) {
        double s = 0.0;
        for (int j = 0; j < i; ++j) s += A[i][j] * col[j];
        col[i] = (col[i] - s) / A[i][i];
      }
      for (int i = P - 1; i >= 0; --i) {
        double s = 0.0;
        for (int j = i + 1; j < P; ++j) s += A[j][i] * col[j];
        col[i] = (col[i] - s) / A[i][i];
      }
      for (int i = 0; i < P; ++i) Ai[lane][i] = col[i];  // row `lane` of Ai
    }
    __syncwarp();
    ok = chol_warp(Ai, P, lane);
  }
  if (ok) {
    const double df = (double)d.V + (double)ch.df_offset;
    const uint32_t cid = ch.chain_id << 8, sw = (uint32_t)sweep;
    if (lane < P) {
      const double c2 = supplied ? sup.chi2[lane]
                                 : 2.0 * gamma_mt(0.5 * (df - lane), (uint32_t)lane,
                                                  sw, cid | kTagGamma, ch.key0,
                                                  ch.key1, &err);
      T[lane][lane] = sqrt(c2);
    }
    const int nw = P * (P - 1) / 2;
    if (lane < nw) {
      int i = 1;
      while ((i + 1) * i / 2 <= lane) ++i;  // row i: lane in [i(i-1)/2, i(i+1)/2)
      const int j = lane - i * (i - 1) / 2;
      double z;
      if (supplied) {
        z = sup.wnorm[lane];
      } else {
        const uint4 r = philox1(make_uint4((uint32_t)(lane >> 2), 0u, sw,
                                           cid | kTagWNorm),
                                ch.key0, ch.key1);
        z = (double)normal_of(pick4(r, lane & 3));
      }
      T[i][j] = z;
    }
    __syncwarp();
    if (lane < P) {  // row `lane` of B = L T (L lower from Ai)
      const int i = lane;
      for (int j = 0; j < P; ++j) {
        double s = 0.0;
        for (int k = j; k <= i; ++k) s += Ai[i][k] * T[k][j];
        B[i][j] = j <= i ? s : 0.0;
      }
    }
    __syncwarp();
    bool fin = true;
    if (lane < P) {
      const int i = lane;
      for (int j = 0; j < P; ++j) {
        const int K = i < j ? i : j;
        double s = 0.0;
        for (int k = 0; k <= K; ++k) s += B[i][k] * B[j][k];
        A[i][j] = s;  // A is free again
        fin = fin && isfinite(s);
      }
    }
    fin = __all_sync(0xffffffffu, fin);
    __syncwarp();
    if (fin) {
      if (lane < P)
        for (int j = 0; j < P; ++j) {
          ch.omega_d[lane * P + j] = A[lane][j];
          ch.omega_f[lane * P + j] = (float)A[lane][j];
        }
    } else {
      err |= kErrNaN;
    }
  } else {
    err |= kErrWishart;
  }
  if (lane < P) ch.colmean[lane] = (float)(tot[kMaxPairs + lane] / (double)d.V);
  err = __reduce_or_sync(0xffffffffu, err);
  if (lane == 0) {
    if (err) atomicOr(ch.status, err);
    *ch.sweep = sweep + 1;
    if (kept) *ch.nkept = nk + 1;
    *ch.done = 0u;
    __threadfence();
  }
}

// ------------------------------------------------------ post-sweep pass --
// One pass over every in-mask voxel after both colours: the pair sums of
// Spat_Coef_Prec (covarGPU.cu:953-1013, covar.cpp:220-262; the indicator
// tests the row coefficient of the forward neighbour), the column sums of
// covarGPU.cu:563-583, and on kept sweeps the FP64 running sums of beta,
// beta^2 and the lesion probability (mcmc.cpp:627-649).  Each thread sums
// the products of its (at most four) voxels in FP32 and adds them to FP64
// accumulators; block partials are summed in a fixed order by the last
// block to arrive, whose first warp then draws Omega: the result is
// bitwise reproducible.
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
  const int npairs = P * (P + 1) / 2;

  float pv[kMaxPairs], csf[kMaxP];
#pragma unroll
  for (int q = 0; q < kMaxPairs; ++q) pv[q] = 0.f;
#pragma unroll
  for (int p = 0; p < kMaxP; ++p) csf[p] = 0.f;

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
      csf[p] += bs[p];
    }
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
    if (kept) {  // running sums of mcmc.cpp:637-645, FP64
      const int v = d.vidx[c][j];
#pragma unroll
      for (int p = 0; p < kMaxP; ++p)
        if (p < P) {
          const double x = (double)bs[p];
          ch.acc_sum[(size_t)p * V + v] += x;
          ch.acc_sq[(size_t)p * V + v] += x * x;
        }
      const float bwm = ch.beta_wm * (d.wm ? d.wm[v] : 1.f);
#pragma unroll
      for (int g = 0; g < kMaxP; ++g)
        if (g < S) ch.prb_sum[(size_t)g * V + v] += (double)prob_sdnorm(bs[g] + bwm);
    }
  }

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < kPostVals; ++q) {
    const bool live = q < kMaxPairs ? q < npairs : (q - kMaxPairs) < P;
    if (!live) continue;
    double val = q < kMaxPairs ? (double)pv[q] : (double)csf[q - kMaxPairs];
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
  // Warp w sums values q = w, w + 8, ...: lanes stride over the blocks,
  // then a fixed shuffle tree -- same order on every run.
  for (int q = warp; q < kPostVals; q += kPostThreads / 32) {
    const bool live = q < kMaxPairs ? q < npairs : (q - kMaxPairs) < P;
    double s = 0.0;
    if (live)
      for (int b = lane; b < ch.post_blocks; b += 32)
        s += __ldcg(ch.partials + (size_t)b * kPostVals + q);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) tot[q] = s;
  }
  __syncthreads();
  if (warp == 0) wishart_warp(ch, d, tot, sweep, kept, nk, supplied, sup, lane);
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
