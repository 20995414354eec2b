// bsg_predict.cu -- the DIC / Qhat predictive pass.
//
// Replaces compute_predictGPU (covarGPU.cu:1866-1957) with its kernels
// ProbSDNormGPU_prediction (covarGPU.cu:1783-1812) and reduce_for_Mpredict
// (covarGPU.cu:1826-1864), and the DE sum of compute_prb_DIC
// (covar.cpp:442-486).  For subject i and group column g the pass forms
//   Mpredict[i][g] = sum over in-mask v of log P(Y_iv | eta_igv),
//   eta_igv = beta_vg + beta_WM WM_v + sum_{p >= S} beta_vp X_pi,
// with P(Y = 1) = PhiAS(eta), the A&S 26.2.17 form of the reference.  The
// reference launches 2 + S kernels and a blocking copy per subject; here one
// launch covers every subject and voxel and a second reduces the tiles.
//
// predict_kernel: a block takes 128 subjects (one per thread, the design
// row in registers) and a tile of 1024 voxels staged 128 at a time in shared
// memory (coefficients as float4 pairs, beta_WM WM_v, and each warp's
// 32-subject outcome word per voxel).  Per-thread sums are FP32 over 32
// voxels, then FP64; each block writes its [subjects][columns] partials.
//
// predict_finish_kernel: one warp per subject sums the tile partials in a
// fixed order (lane l takes tiles l, l + 32, ...; xor-shuffle tree), so the
// result does not depend on scheduling; lane 0 updates Qhat
// (covarGPU.cu:1937-1953) and stores the subject's own-group term; the last
// block to arrive adds them, in subject order, to the ED sum.
//
// Log probabilities: PhiAS(-x) = 1 - PhiAS(x) holds exactly for the A&S
// form, so the observed outcome's probability is taken on its own side: on
// the tail side log(c t poly(t)) - eta^2 / 2 (no exp, no underflow), on the
// other side log(1 - c t poly(t) exp(-eta^2 / 2)).  The reference's FP32
// y log(p + 1e-35) + (1 - y) log(1 - p + 1e-35) is the same quantity where
// its 1 - p does not cancel (|eta| below about 5).
#include "bsg_device.cuh"

namespace bsg {

namespace {

constexpr int kPredSub = 128;  // voxels staged per pass (one per thread)
static_assert(kPredSub == kPredThreads, "staging uses one voxel per thread");

// ln P(Y = y | eta) under A&S 26.2.17, FP32.
__device__ __forceinline__ float loglik_as(float eta, uint32_t y) {
  const float b1 = 0.319381530f, b2 = -0.356563782f, b3 = 1.781477937f;
  const float b4 = -1.821255978f, b5 = 1.330274429f, p = 0.2316419f;
  const float c = 0.39894228f;
  const float ax = fabsf(eta);
  const float t = rcp_approx(fmaf(p, ax, 1.0f));
  const float r = c * t * fmaf(t, fmaf(t, fmaf(t, fmaf(t, b5, b4), b3), b2), b1);
  const float h = 0.5f * eta * eta;
  // tail side: Y = 1 with eta < 0, or Y = 0 with eta >= 0
  const bool tail = y ? (eta < 0.f) : (eta >= 0.f);
  const float e = ex2_approx(h * -1.44269504f);
  const float u = tail ? r : fmaf(-r, e, 1.0f);
  return fmaf(lg2_approx(u), 0.693147181f, tail ? -h : 0.f);
}

__device__ __forceinline__ bool predict_gate(const ChainDev &ch, int mode) {
  if (mode != kPredKept) return true;
  const long long s = ch.sweep[1] - 1;  // the sweep that just completed
  return s > ch.burnin && (s % (ch.thin > 0 ? ch.thin : 1)) == 0;
}

template <int P>
__global__ void __launch_bounds__(kPredThreads)
    predict_kernel(const DatasetDev *__restrict__ dsv, ChainDev *__restrict__ chv,
                   const BlockMap *__restrict__ map, int chain, int mode) {
  // Coefficients of this sweep are final once the previous kernel is done.
  cudaGridDependencySynchronize();
  cudaTriggerProgrammaticLaunchCompletion();
  const int cidx = map ? map[blockIdx.x].chain : chain;
  const int tile = map ? map[blockIdx.x].start : (int)blockIdx.x;
  const ChainDev &ch = chv[cidx];
  const DatasetDev &d = dsv[ch.dataset];
  const int N = d.N, S = d.S, Vp = d.Vp, V = d.V;
  const int i0 = blockIdx.y * kPredThreads;
  if (i0 >= N || !predict_gate(ch, mode)) return;  // uniform per block
  const int G = mode == kPredDE ? 1 : S;
  const int n0 = d.n[0], ntot = n0 + d.n[1];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int i = i0 + tid;
  const int word = i0 / 32 + warp;  // this warp's 32-subject outcome word

  __shared__ float4 Bs[kPredSub][2];
  __shared__ float Bw[kPredSub];
  __shared__ uint32_t Ys[kPredThreads / 32][kPredSub];

  float x[P];
#pragma unroll
  for (int p = 0; p < P; ++p) x[p] = i < N ? d.covar[(size_t)p * N + i] : 0.f;
  double acc[P];
#pragma unroll
  for (int g = 0; g < P; ++g) acc[g] = 0.0;
  const double inv_nk =
      mode == kPredDE ? 1.0 / (double)(*ch.nkept > 0 ? *ch.nkept : 1) : 0.0;

  const int t0 = tile * kPredTile, t1 = min(t0 + kPredTile, ntot);
  for (int q0 = t0; q0 < t1; q0 += kPredSub) {
    const int nsub = min(kPredSub, t1 - q0);
    __syncthreads();
    if (tid < nsub) {
      const int pos = q0 + tid;
      const int c = pos < n0 ? 0 : 1, j = c ? pos - n0 : pos;
      const int sc = d.nb[c][j], v = d.vidx[c][j];
      float b[8];
#pragma unroll
      for (int p = 0; p < 8; ++p) {
        if (p >= P)
          b[p] = 0.f;
        else if (mode == kPredDE)
          b[p] = (float)(ch.acc_sum[(size_t)p * V + v] * inv_nk);
        else
          b[p] = ch.beta[(size_t)p * Vp + sc];
      }
      Bs[tid][0] = make_float4(b[0], b[1], b[2], b[3]);
      Bs[tid][1] = make_float4(b[4], b[5], b[6], b[7]);
      Bw[tid] = ch.beta_wm * (d.wm ? d.wm[v] : 1.f);
    }
    if (word < d.W) {
      for (int k = lane; k < nsub; k += 32) {
        const int pos = q0 + k;
        const int c = pos < n0 ? 0 : 1, j = c ? pos - n0 : pos;
        Ys[warp][k] = d.ybits[c][(size_t)word * d.n[c] + j];
      }
    }
    __syncthreads();
    if (i < N) {
      for (int k0 = 0; k0 < nsub; k0 += 32) {
        const int k1 = min(k0 + 32, nsub);
        float s32[P];
#pragma unroll
        for (int g = 0; g < P; ++g) s32[g] = 0.f;
        for (int k = k0; k < k1; ++k) {
          const float4 u0 = Bs[k][0], u1 = Bs[k][1];
          const float b[8] = {u0.x, u0.y, u0.z, u0.w, u1.x, u1.y, u1.z, u1.w};
          const uint32_t y = (Ys[warp][k] >> lane) & 1u;
          if (mode == kPredDE) {
            float eta = Bw[k];
#pragma unroll
            for (int p = 0; p < P; ++p) eta = fmaf(b[p], x[p], eta);
            s32[0] += loglik_as(eta, y);
          } else {
            float rest = Bw[k];
#pragma unroll
            for (int p = 0; p < P; ++p)
              if (p >= S) rest = fmaf(b[p], x[p], rest);
#pragma unroll
            for (int g = 0; g < P; ++g)
              if (g < S) s32[g] += loglik_as(b[g] + rest, y);
          }
        }
#pragma unroll
        for (int g = 0; g < P; ++g) acc[g] += (double)s32[g];
      }
    }
  }
  if (i < N) {
    double *out = ch.pred_part + ((size_t)tile * N + i) * G;
#pragma unroll
    for (int g = 0; g < P; ++g)
      if (g < G) out[g] = acc[g];
  }
}

__global__ void __launch_bounds__(kPredWarps * 32)
    predict_finish_kernel(const DatasetDev *__restrict__ dsv,
                          ChainDev *__restrict__ chv,
                          const BlockMap *__restrict__ map, int chain, int mode) {
  cudaGridDependencySynchronize();
  cudaTriggerProgrammaticLaunchCompletion();
  const int cidx = map ? map[blockIdx.x].chain : chain;
  const int sblk = map ? map[blockIdx.x].start : (int)blockIdx.x;
  ChainDev &ch = chv[cidx];
  const DatasetDev &d = dsv[ch.dataset];
  if (!predict_gate(ch, mode)) return;  // uniform per chain
  const int N = d.N, S = d.S;
  const int G = mode == kPredDE ? 1 : S;
  const int T = ch.pred_tiles;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int i = sblk * kPredWarps + warp;
  const bool first = *ch.npred == 0;

  if (i < N) {
    double m[kMaxP];
#pragma unroll
    for (int g = 0; g < kMaxP; ++g) {
      double s = 0.0;
      if (g < G)
        for (int t = lane; t < T; t += 32) s += ch.pred_part[((size_t)t * N + i) * G + g];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      m[g] = s;
    }
    if (lane == 0) {
      if (mode == kPredDE) {
        ch.pred_subj[i] = m[0];
      } else {
        // the subject's own group: the first nonzero group column
        // (covarGPU.cu:1929-1935)
        int sub = 0;
        for (int g = S - 1; g >= 0; --g)
          if (d.covar[(size_t)g * N + i] != 0.f) sub = g;
        double own = m[0];
#pragma unroll
        for (int g = 0; g < kMaxP; ++g)
          if (g == sub) own = m[g];
#pragma unroll
        for (int g = 0; g < kMaxP; ++g)
          if (g < S) ch.mpred[(size_t)i * S + g] = m[g];
        if (mode == kPredKept) {
          ch.pred_subj[i] = own;
          // Qhat (covarGPU.cu:1937-1953): log-sum over kept sweeps of
          // Mpredict[g] - Mpredict[own]; on the first kept sweep column 0
          // is set and the others are log-added onto 0.
#pragma unroll
          for (int g = 0; g < kMaxP; ++g) {
            if (g >= S) continue;
            double *q = ch.qhat + (size_t)i * S + g;
            const double dg = m[g] - own;
            if (first && g == 0) {
              *q = dg;
            } else {
              const double mx = fmax(dg, *q);
              *q = log(exp(*q - mx) + exp(dg - mx)) + mx;
            }
          }
        }
      }
    }
  }
  if (mode == kPredNow) return;

  // The last block of this chain adds the subjects' terms in subject order.
  __shared__ bool last;
  __shared__ double red[kPredWarps * 32];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned nblk = (unsigned)((N + kPredWarps - 1) / kPredWarps);
    last = atomicAdd(ch.pred_done, 1u) == nblk - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double s = 0.0;
  for (int k = threadIdx.x; k < N; k += blockDim.x)
    s += *(volatile double *)(ch.pred_subj + k);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (mode == kPredKept) {
      ch.pred_sums[0] += red[0];
      *ch.npred += 1;
    } else {
      ch.pred_sums[1] = -2.0 * red[0];
    }
    *ch.pred_done = 0;
  }
}

template <int P>
cudaError_t launch_predict_p(const DatasetDev *ds, ChainDev *ch, const BlockMap *map,
                             int nblocks, int chunks, int chain, int mode,
                             cudaStream_t st, bool pdl) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(nblocks, chunks);
  cfg.blockDim = dim3(kPredThreads);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, predict_kernel<P>, ds, ch, map, chain, mode);
}

}  // namespace

cudaError_t launch_predict(int P, const DatasetDev *ds, ChainDev *ch,
                           const BlockMap *map, int nblocks, int chunks, int chain,
                           int mode, cudaStream_t st, bool pdl) {
  if (nblocks <= 0 || chunks <= 0) return cudaSuccess;
  switch (P) {
    case 1: return launch_predict_p<1>(ds, ch, map, nblocks, chunks, chain, mode, st, pdl);
    case 2: return launch_predict_p<2>(ds, ch, map, nblocks, chunks, chain, mode, st, pdl);
    case 3: return launch_predict_p<3>(ds, ch, map, nblocks, chunks, chain, mode, st, pdl);
    case 4: return launch_predict_p<4>(ds, ch, map, nblocks, chunks, chain, mode, st, pdl);
    case 5: return launch_predict_p<5>(ds, ch, map, nblocks, chunks, chain, mode, st, pdl);
    case 6: return launch_predict_p<6>(ds, ch, map, nblocks, chunks, chain, mode, st, pdl);
    case 7: return launch_predict_p<7>(ds, ch, map, nblocks, chunks, chain, mode, st, pdl);
    case 8: return launch_predict_p<8>(ds, ch, map, nblocks, chunks, chain, mode, st, pdl);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_predict_finish(const DatasetDev *ds, ChainDev *ch,
                                  const BlockMap *map, int nblocks, int chain,
                                  int mode, cudaStream_t st, bool pdl) {
  if (nblocks <= 0) return cudaSuccess;
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(nblocks);
  cfg.blockDim = dim3(kPredWarps * 32);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, predict_finish_kernel, ds, ch, map, chain, mode);
}

}  // namespace bsg
