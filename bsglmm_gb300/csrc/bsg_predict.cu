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
// result does not depend on scheduling; lanes 0..S-1 update Qhat
// (covarGPU.cu:1937-1953), lane 0 stores the subject's own-group term; the last
// block to arrive adds them, in subject order, to the ED sum.
//
// Log probabilities: PhiAS(-x) = 1 - PhiAS(x) holds exactly for the A&S
// form, so the observed outcome's probability is taken on its own side: on
// the tail side log(c t poly(t)) - eta^2 / 2 (no exp, no underflow), on the
// other side log(1 - c t poly(t) exp(-eta^2 / 2)).  The reference's FP32
// y log(p + 1e-35) + (1 - y) log(1 - p + 1e-35) is the same quantity where
// its 1 - p does not cancel (|eta| below about 5).
#include "../../include/bsglmm_gb300.h"
#include "bsg_device.cuh"

namespace bsg {

namespace {

constexpr int kPredSub = 128;  // voxels staged per pass (one per thread)
// Resident blocks per SM asked of ptxas: 12 (40 registers, full occupancy;
// measured faster than the 52-register schedule at 9 blocks) while the
// design row and the group sums fit, fewer for larger P and S.
template <int P, int S>
constexpr int pred_min_blocks() {
  return (P <= 5 && S <= 2) ? 12 : (P + S <= 8 ? 10 : 8);
}
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
// Products and sums carry explicit rounding, so the f32x2 forms below give
// exactly the scalar values per component.
__device__ __forceinline__ float log2lik_as(float a) {
  const float t = rcp_approx(fmaf(0.2316419f, fabsf(a), 1.0f));
  const float r =
      __fmul_rn(t, fmaf(t, fmaf(t, fmaf(t, fmaf(t, kA5, kA4), kA3), kA2), kA1));
  const float w = __fmul_rn(__fmul_rn(a, -0.721347520f), a);  // -eta^2/2, log2 units
  const bool tail = a < 0.f;
  const float u = tail ? r : fmaf(-r, ex2_approx(w), 1.0f);
  return __fadd_rn(lg2_approx(u), tail ? w : 0.f);
}

__device__ __forceinline__ float2 log2lik_as2(float2 a) {
  const float2 h = fma2(splat2(0.2316419f), make_float2(fabsf(a.x), fabsf(a.y)), splat2(1.0f));
  const float2 t = make_float2(rcp_approx(h.x), rcp_approx(h.y));
  const float2 r = mul2(t, fma2(t, fma2(t, fma2(t, fma2(t, splat2(kA5), splat2(kA4)),
                                                splat2(kA3)), splat2(kA2)), splat2(kA1)));
  const float2 w = mul2(mul2(a, splat2(-0.721347520f)), a);
  const float2 fm = fma2(mul2(r, splat2(-1.f)),
                         make_float2(ex2_approx(w.x), ex2_approx(w.y)), splat2(1.0f));
  const bool t0 = a.x < 0.f, t1 = a.y < 0.f;
  return add2(make_float2(lg2_approx(t0 ? r.x : fm.x), lg2_approx(t1 ? r.y : fm.y)),
              make_float2(t0 ? w.x : 0.f, t1 ? w.y : 0.f));
}

// -log2 P(Y | eta) for the t/logit links, P(Y = 1) = 1 / (1 + exp(-z)) with
// z = eta / lf (ProbLogitGPU_prediction, covarGPU.cu:1750-1781), for a = z
// with its sign flipped when Y = 0: log2(1 + exp(-a)) (the sums subtract it).
__device__ __forceinline__ float nlog2lik_logit(float a) {
  const float e = ex2_approx(__fmul_rn(fabsf(a), -1.44269504f));
  return fmaf(fmaxf(-a, 0.f), 1.44269504f, lg2_approx(__fadd_rn(1.f, e)));
}

__device__ __forceinline__ float2 nlog2lik_logit2(float2 a) {
  const float2 s = mul2(make_float2(fabsf(a.x), fabsf(a.y)), splat2(-1.44269504f));
  const float2 e1 = add2(splat2(1.f), make_float2(ex2_approx(s.x), ex2_approx(s.y)));
  return fma2(make_float2(fmaxf(-a.x, 0.f), fmaxf(-a.y, 0.f)), splat2(1.44269504f),
              make_float2(lg2_approx(e1.x), lg2_approx(e1.y)));
}

__device__ __forceinline__ float2 sign_flip2(float2 a, uint32_t m0, uint32_t m1) {
  return make_float2(__uint_as_float(__float_as_uint(a.x) ^ m0),
                     __uint_as_float(__float_as_uint(a.y) ^ m1));
}

__device__ __forceinline__ bool predict_gate(const ChainDev &ch, int mode) {
  if (mode != kPredKept) return true;
  const long long s = ch.sweep[1] - 1;  // the sweep that just completed
  return s > ch.burnin && (s % (ch.thin > 0 ? ch.thin : 1)) == 0;
}

// P covariates, the first S of them group columns.  Voxels are staged in
// pairs: pair row u holds (b_2u,p, b_2u+1,p) for p = 0..P (the P
// coefficients, then beta_WM WM_v), padded to float4s, so that each thread
// evaluates two voxels per f32x2 operation.
template <int P, int S>
__global__ void __launch_bounds__(kPredThreads, pred_min_blocks<P, S>())
    predict_kernel(const DatasetDev *__restrict__ dsv, ChainDev *__restrict__ chv,
                   const BlockMap *__restrict__ map, int chain, int mode) {
  constexpr int R2 = (2 * (P + 1) + 3) / 4;  // float4s per staged voxel pair
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

  __shared__ float4 Bs2[kPredSub / 2][R2];
  __shared__ uint32_t Ys[kPredThreads / 32][kPredSub];

  float2 xx[P];  // the subject's design row, duplicated for f32x2 operands
#pragma unroll
  for (int p = 0; p < P; ++p) {
    const float xv = i < N ? d.covar[(size_t)p * N + i] : 0.f;
    xx[p] = make_float2(xv, xv);
  }
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
      float *row = reinterpret_cast<float *>(&Bs2[tid >> 1][0]) + (tid & 1);
#pragma unroll
      for (int p = 0; p < P; ++p)
        row[2 * p] = de ? (float)(ch.acc_sum[(size_t)p * V + v] * inv_nk)
                        : ch.beta[(size_t)p * Vp + sc];
      row[2 * P] = bwc * (d.wm ? d.wm[v] : 1.f);
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
        float2 s2[S];  // FP32 sums of the even (.x) and odd (.y) voxels
#pragma unroll
        for (int g = 0; g < S; ++g) s2[g] = make_float2(0.f, 0.f);
        // voxels k, k + 1 of one pair row, then an odd last voxel alone from
        // the .x halves
        int k = k0;
#pragma unroll 1
        for (; k + 1 < k1; k += 2) {  // (measured: unroll 1 < 4 < 2 in time)
          float2 bp[2 * R2];
#pragma unroll
          for (int u = 0; u < R2; ++u) {
            const float4 f = Bs2[k >> 1][u];
            bp[2 * u] = make_float2(f.x, f.y);
            bp[2 * u + 1] = make_float2(f.z, f.w);
          }
          const uint2 yy = *reinterpret_cast<const uint2 *>(&Ys[warp][k]);
          // sign masks: flip eta's sign when Y = 0
          const uint32_t m0 = ~(yy.x << sh) & 0x80000000u, m1 = ~(yy.y << sh) & 0x80000000u;
          if (de) {
            float2 eta = bp[P];
#pragma unroll
            for (int p = 0; p < P; ++p) eta = fma2(bp[p], xx[p], eta);
            const float2 a = sign_flip2(eta, m0, m1);
            s2[0] = logit ? sub2(s2[0], nlog2lik_logit2(a)) : add2(s2[0], log2lik_as2(a));
          } else {
            float2 rest = bp[P];
#pragma unroll
            for (int p = S; p < P; ++p) rest = fma2(bp[p], xx[p], rest);
#pragma unroll
            for (int g = 0; g < S; ++g) {
              const float2 a = sign_flip2(add2(bp[g], rest), m0, m1);
              s2[g] = logit ? sub2(s2[g], nlog2lik_logit2(mul2(a, splat2(ilf))))
                            : add2(s2[g], log2lik_as2(a));
            }
          }
        }
        if (k < k1) {
          const float *br = reinterpret_cast<const float *>(&Bs2[k >> 1][0]);
          const uint32_t m0 = ~(Ys[warp][k] << sh) & 0x80000000u;
          if (de) {
            float eta = br[2 * P];
#pragma unroll
            for (int p = 0; p < P; ++p) eta = fmaf(br[2 * p], xx[p].x, eta);
            const float a = __uint_as_float(__float_as_uint(eta) ^ m0);
            s2[0].x = logit ? __fsub_rn(s2[0].x, nlog2lik_logit(a))
                            : __fadd_rn(s2[0].x, log2lik_as(a));
          } else {
            float rest = br[2 * P];
#pragma unroll
            for (int p = S; p < P; ++p) rest = fmaf(br[2 * p], xx[p].x, rest);
#pragma unroll
            for (int g = 0; g < S; ++g) {
              const float a = __uint_as_float(__float_as_uint(__fadd_rn(br[2 * g], rest)) ^ m0);
              s2[g].x = logit ? __fsub_rn(s2[g].x, nlog2lik_logit(__fmul_rn(a, ilf)))
                              : __fadd_rn(s2[g].x, log2lik_as(a));
            }
          }
        }
#pragma unroll
        for (int g = 0; g < S; ++g)
          acc[g] = fma((double)(s2[g].x + s2[g].y), 0.6931471805599453, acc[g]);
      }
    }
  }
  if (i < N) {
    // [subject][column][tile]: the finishing warp of a subject then reads
    // its tiles from consecutive addresses
    const int G = de ? 1 : S;
    double *out = ch.pred_part + (size_t)i * G * ch.pred_tiles + tile;
#pragma unroll
    for (int g = 0; g < S; ++g)
      if (g < G) out[(size_t)g * ch.pred_tiles] = acc[g];
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
      if (g < G) {
        // consecutive tiles across the lanes, four loads in flight per lane;
        // the sum keeps tile order
        const double *src = ch.pred_part + ((size_t)i * G + g) * T;
#pragma unroll 4
        for (int t = lane; t < T; t += 32) s += __ldcg(src + t);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      m[g] = s;
    }
    if (mode == kPredDE) {
      if (lane == 0) ch.pred_subj[i] = m[0];
    } else {
      // the subject's own group: the first nonzero group column
      // (covarGPU.cu:1929-1935)
      int sub = 0;
      for (int g = S - 1; g >= 0; --g)
        if (d.covar[(size_t)g * N + i] != 0.f) sub = g;
      double own = m[0], mg = m[0];
#pragma unroll
      for (int g = 0; g < kMaxP; ++g) {
        if (g == sub) own = m[g];
        if (g == lane) mg = m[g];
      }
      if (lane == 0 && mode == kPredKept) ch.pred_subj[i] = own;
      // lane g < S stores column g and updates its Qhat entry
      // (covarGPU.cu:1937-1953): log-sum over kept sweeps of Mpredict[g] -
      // Mpredict[own]; on the first kept sweep column 0 is set and the
      // others are log-added onto 0
      if (lane < S) {
        ch.mpred[(size_t)i * S + lane] = mg;
        if (mode == kPredKept) {
          double *q = ch.qhat + (size_t)i * S + lane;
          const double dg = mg - own;
          if (first && lane == 0) {
            *q = dg;
          } else {
            // log(exp(q - mx) + exp(dg - mx)) + mx with mx = max(q, dg): one
            // of the two terms is exp(0) = 1 exactly
            const double mx = fmax(dg, *q), lo = fmin(dg, *q);
            *q = log(1.0 + exp(lo - mx)) + mx;
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

// Self-check of the f32x2 forms: for n random inputs, each paired helper
// against two calls of its scalar form, compared bit for bit (and the
// Marsaglia-Tsang acceptance decisions); mismatches are counted.
__global__ void pairs_selftest_kernel(int64_t n, uint32_t k0, uint32_t k1,
                                      unsigned long long *bad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint4 r = philox1(make_uint4((uint32_t)i, (uint32_t)(i >> 32), 0u, 0xA5u), k0, k1);
  const uint4 q = philox1(make_uint4((uint32_t)i, (uint32_t)(i >> 32), 1u, 0xA5u), k0, k1);
  auto ne = [](float x, float y) { return __float_as_uint(x) != __float_as_uint(y); };
  // arguments over [-8, 8): both inversion branches, the clamp and both
  // log-likelihood sides
  const float a0 = fmaf(u_of(r.x), 16.f, -8.f), a1 = fmaf(u_of(r.y), 16.f, -8.f);
  unsigned m = 0;
  const float c0 = fminf(a0, kATail), c1 = fminf(a1, kATail);
  const float2 t = tn_lower_inv2(make_float2(c0, c1), r.z, r.w);
  m += ne(t.x, tn_lower_inv(c0, r.z)) + ne(t.y, tn_lower_inv(c1, r.w));
  const float2 z = normal_of2(q.x, q.y);
  m += ne(z.x, normal_of(q.x)) + ne(z.y, normal_of(q.y));
  // Gamma(4.5): the t_8 weights of the logistic link
  const float dd = 4.5f - 1.f / 3.f, cc = rsqrtf(9.f * dd);
  float2 g;
  bool o0, o1;
  gamma_mt_try2(dd, cc, q.x, q.z, q.y, q.w, &g, &o0, &o1);
  float g0, g1;
  const bool s0 = gamma_mt_try(dd, cc, q.x, q.y, &g0);
  const bool s1 = gamma_mt_try(dd, cc, q.z, q.w, &g1);
  m += ne(g.x, g0) + ne(g.y, g1) + (o0 != s0) + (o1 != s1);
  const float2 la = log2lik_as2(make_float2(a0, a1));
  m += ne(la.x, log2lik_as(a0)) + ne(la.y, log2lik_as(a1));
  const float2 ll = nlog2lik_logit2(make_float2(a0, a1));
  m += ne(ll.x, nlog2lik_logit(a0)) + ne(ll.y, nlog2lik_logit(a1));
  if (m) atomicAdd(bad, (unsigned long long)m);
}

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

extern "C" bsg_status bsg_selftest_pairs(int32_t device, int64_t n, uint64_t seed,
                                         int64_t *mismatches) {
  if (!mismatches || n < 0) return BSG_ERR_INVALID;
  int nd = 0;
  if (cudaGetDeviceCount(&nd) != cudaSuccess || nd == 0) return BSG_ERR_NO_DEVICE;
  if (cudaSetDevice(device) != cudaSuccess) return BSG_ERR_INVALID;
  unsigned long long *bad = nullptr;
  if (cudaMalloc(&bad, sizeof(*bad)) != cudaSuccess) return BSG_ERR_CUDA;
  unsigned long long h = 0;
  cudaError_t e = cudaMemset(bad, 0, sizeof(*bad));
  if (e == cudaSuccess && n > 0) {
    const int threads = 256;
    bsg::pairs_selftest_kernel<<<(unsigned)((n + threads - 1) / threads), threads>>>(
        n, (uint32_t)seed, (uint32_t)(seed >> 32), bad);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(&h, bad, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(bad);
  if (e != cudaSuccess) return BSG_ERR_CUDA;
  *mismatches = (int64_t)h;
  return BSG_OK;
}
