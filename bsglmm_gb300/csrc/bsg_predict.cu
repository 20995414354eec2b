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
// predict_kernel<P, S>: a block takes 128 subjects (one per thread, the
// design row in registers) and a tile of voxels, sized on the host so that
// the grid is one wave, staged 128 at a time in shared memory (the voxel's
// coefficients and beta_WM WM_v as float4s, and each warp's 32-subject
// outcome word).  The outcome enters as a sign flip of eta.  Per-thread
// sums are FP32 (log2 units) over 32 voxels, then FP64; each block writes
// its [subjects][columns] partials.
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

// A&S 26.2.17 with 1/sqrt(2 pi) folded in: c * (b1 t + ... + b5 t^5).
constexpr float kA1 = 0.39894228f * 0.319381530f;
constexpr float kA2 = 0.39894228f * -0.356563782f;
constexpr float kA3 = 0.39894228f * 1.781477937f;
constexpr float kA4 = 0.39894228f * -1.821255978f;
constexpr float kA5 = 0.39894228f * 1.330274429f;

// log2 P(Y | eta) under A&S 26.2.17, FP32, for a = eta with its sign bit
// flipped when Y = 0: the observed outcome lies on the tail side iff a < 0.
// Tail side: log2(c t poly(t)) - eta^2 / (2 ln 2); other side:
// log2(1 - c t poly(t) exp(-eta^2 / 2)).
__device__ __forceinline__ float log2lik_as(float a) {
  const float t = rcp_approx(fmaf(0.2316419f, fabsf(a), 1.0f));
  const float r = t * fmaf(t, fmaf(t, fmaf(t, fmaf(t, kA5, kA4), kA3), kA2), kA1);
  const float w = (a * -0.721347520f) * a;  // -eta^2 / 2 in log2 units
  const bool tail = a < 0.f;
  const float u = tail ? r : fmaf(-r, ex2_approx(w), 1.0f);
  return lg2_approx(u) + (tail ? w : 0.f);
}

// log2 P(Y | eta) for the t/logit links, P(Y = 1) = 1 / (1 + exp(-z)) with
// z = eta / lf (ProbLogitGPU_prediction, covarGPU.cu:1750-1781), for a = z
// with its sign flipped when Y = 0: -log2(1 + exp(-a)).
__device__ __forceinline__ float log2lik_logit(float a) {
  const float e = ex2_approx(fabsf(a) * -1.44269504f);
  return -(lg2_approx(1.f + e) + fmaxf(-a, 0.f) * 1.44269504f);
}

__device__ __forceinline__ bool predict_gate(const ChainDev &ch, int mode) {
  if (mode != kPredKept) return true;
  const long long s = ch.sweep[1] - 1;  // the sweep that just completed
  return s > ch.burnin && (s % (ch.thin > 0 ? ch.thin : 1)) == 0;
}

// P covariates, the first S of them group columns.  Shared row per voxel:
// P coefficients then beta_WM WM_v, padded to float4s.
template <int P, int S>
__global__ void __launch_bounds__(kPredThreads)
    predict_kernel(const DatasetDev *__restrict__ dsv, ChainDev *__restrict__ chv,
                   const BlockMap *__restrict__ map, int chain, int mode) {
  constexpr int Q = (P + 1 + 3) / 4;  // float4s per staged voxel
  // Coefficients of this sweep are final once the previous kernel is done.
  cudaGridDependencySynchronize();
  cudaTriggerProgrammaticLaunchCompletion();
  const int cidx = map ? map[blockIdx.x].chain : chain;
  const int tile = map ? map[blockIdx.x].start : (int)blockIdx.x;
  const ChainDev &ch = chv[cidx];
  const DatasetDev &d = dsv[ch.dataset];
  const int N = d.N, Vp = d.Vp, V = d.V;
  const int i0 = blockIdx.y * kPredThreads;
  if (i0 >= N || !predict_gate(ch, mode)) return;  // uniform per block
  const bool de = mode == kPredDE;
  const int n0 = d.n[0], ntot = n0 + d.n[1];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int i = i0 + tid;
  const int word = i0 / 32 + warp;  // this warp's 32-subject outcome word
  const int tw = ch.pred_tile;      // voxels per tile

  __shared__ float4 Bs[kPredSub][Q];
  __shared__ uint32_t Ys[kPredThreads / 32][kPredSub];

  float x[P];
#pragma unroll
  for (int p = 0; p < P; ++p) x[p] = i < N ? d.covar[(size_t)p * N + i] : 0.f;
  double acc[S];
#pragma unroll
  for (int g = 0; g < S; ++g) acc[g] = 0.0;
  const double inv_nk = de ? 1.0 / (double)(*ch.nkept > 0 ? *ch.nkept : 1) : 0.0;
  // beta_WM: the current value, or its mean over kept sweeps for DE (MWM)
  const float bwc = de ? (float)(*ch.wm_sum * inv_nk) : *ch.wm_beta;
  // t/logit links: logistic of eta / lf; the DE of compute_prb_DIC
  // (covar.cpp:457-465) takes exp(eta) / (1 + exp(eta)), without lf
  const bool logit = ch.model != 1;
  const float ilf = de ? 1.f : ch.inv_lf;

  const int t0 = tile * tw, t1 = min(t0 + tw, ntot);
  for (int q0 = t0; q0 < t1; q0 += kPredSub) {
    const int nsub = min(kPredSub, t1 - q0);
    __syncthreads();
    if (tid < nsub) {
      const int pos = q0 + tid;
      const int c = pos < n0 ? 0 : 1, j = c ? pos - n0 : pos;
      const int sc = d.nb[c][j], v = d.vidx[c][j];
      float b[4 * Q];
#pragma unroll
      for (int p = 0; p < 4 * Q; ++p) {
        if (p < P)
          b[p] = de ? (float)(ch.acc_sum[(size_t)p * V + v] * inv_nk)
                    : ch.beta[(size_t)p * Vp + sc];
        else
          b[p] = 0.f;
      }
      b[P] = bwc * (d.wm ? d.wm[v] : 1.f);
#pragma unroll
      for (int u = 0; u < Q; ++u)
        Bs[tid][u] = make_float4(b[4 * u], b[4 * u + 1], b[4 * u + 2], b[4 * u + 3]);
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
      const int sh = 31 - lane;  // brings this subject's bit to the sign
      for (int k0 = 0; k0 < nsub; k0 += 32) {
        const int k1 = min(k0 + 32, nsub);
        float s32[S];
#pragma unroll
        for (int g = 0; g < S; ++g) s32[g] = 0.f;
#pragma unroll 2
        for (int k = k0; k < k1; ++k) {
          float b[4 * Q];
#pragma unroll
          for (int u = 0; u < Q; ++u) {
            const float4 f = Bs[k][u];
            b[4 * u] = f.x, b[4 * u + 1] = f.y, b[4 * u + 2] = f.z, b[4 * u + 3] = f.w;
          }
          // sign mask: flips eta's sign when Y = 0
          const uint32_t ymask = ~(Ys[warp][k] << sh) & 0x80000000u;
          if (de) {
            float eta = b[P];
#pragma unroll
            for (int p = 0; p < P; ++p) eta = fmaf(b[p], x[p], eta);
            const float a = __uint_as_float(__float_as_uint(eta) ^ ymask);
            s32[0] += logit ? log2lik_logit(a) : log2lik_as(a);
          } else {
            float rest = b[P];
#pragma unroll
            for (int p = S; p < P; ++p) rest = fmaf(b[p], x[p], rest);
#pragma unroll
            for (int g = 0; g < S; ++g) {
              const float a = __uint_as_float(__float_as_uint(b[g] + rest) ^ ymask);
              s32[g] += logit ? log2lik_logit(a * ilf) : log2lik_as(a);
            }
          }
        }
#pragma unroll
        for (int g = 0; g < S; ++g) acc[g] = fma((double)s32[g], 0.6931471805599453, acc[g]);
      }
    }
  }
  if (i < N) {
    const int G = de ? 1 : S;
    double *out = ch.pred_part + ((size_t)tile * N + i) * G;
#pragma unroll
    for (int g = 0; g < S; ++g)
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

template <int P, int S>
cudaError_t launch_predict_ps(const DatasetDev *ds, ChainDev *ch, const BlockMap *map,
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
  return cudaLaunchKernelEx(&cfg, predict_kernel<P, S>, ds, ch, map, chain, mode);
}

template <int P, int S>
int predict_blocks_per_sm_ps() {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, predict_kernel<P, S>,
                                                    kPredThreads, 0) != cudaSuccess)
    return 1;
  return n > 0 ? n : 1;
}

// Dispatch on (P, S), 1 <= S <= P <= 8.
template <template <int, int> class F, typename... A>
auto dispatch_ps(int P, int S, A... a) -> decltype(F<1, 1>::f(a...)) {
  switch (P * 16 + S) {
#define BSG_C(P_, S_) \
  case P_ * 16 + S_:  \
    return F<P_, S_>::f(a...);
    BSG_C(1, 1)
    BSG_C(2, 1) BSG_C(2, 2)
    BSG_C(3, 1) BSG_C(3, 2) BSG_C(3, 3)
    BSG_C(4, 1) BSG_C(4, 2) BSG_C(4, 3) BSG_C(4, 4)
    BSG_C(5, 1) BSG_C(5, 2) BSG_C(5, 3) BSG_C(5, 4) BSG_C(5, 5)
    BSG_C(6, 1) BSG_C(6, 2) BSG_C(6, 3) BSG_C(6, 4) BSG_C(6, 5) BSG_C(6, 6)
    BSG_C(7, 1) BSG_C(7, 2) BSG_C(7, 3) BSG_C(7, 4) BSG_C(7, 5) BSG_C(7, 6) BSG_C(7, 7)
    BSG_C(8, 1) BSG_C(8, 2) BSG_C(8, 3) BSG_C(8, 4) BSG_C(8, 5) BSG_C(8, 6) BSG_C(8, 7)
    BSG_C(8, 8)
#undef BSG_C
    default:
      return F<1, 1>::fail();
  }
}

template <int P, int S>
struct LaunchF {
  static cudaError_t f(const DatasetDev *ds, ChainDev *ch, const BlockMap *map,
                       int nblocks, int chunks, int chain, int mode, cudaStream_t st,
                       bool pdl) {
    return launch_predict_ps<P, S>(ds, ch, map, nblocks, chunks, chain, mode, st, pdl);
  }
  static cudaError_t fail() { return cudaErrorInvalidValue; }
};

template <int P, int S>
struct OccF {
  static int f(int) { return predict_blocks_per_sm_ps<P, S>(); }
  static int fail() { return 1; }
};

}  // namespace

cudaError_t launch_predict(int P, int S, const DatasetDev *ds, ChainDev *ch,
                           const BlockMap *map, int nblocks, int chunks, int chain,
                           int mode, cudaStream_t st, bool pdl) {
  if (nblocks <= 0 || chunks <= 0) return cudaSuccess;
  return dispatch_ps<LaunchF>(P, S, ds, ch, map, nblocks, chunks, chain, mode, st, pdl);
}

int predict_blocks_per_sm(int P, int S) { return dispatch_ps<OccF>(P, S, 0); }
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
