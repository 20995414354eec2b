// bsg_noalloc.cu -- bsg_omega_update_noalloc: the Omega | beta draw of one
// chain for callers that must not allocate device memory.
//
// Who needs it: code that calls the sampler from inside a host framework
// that owns every device allocation (an inference/graph runtime's plugin,
// a custom call of a compiler runtime, a real-time pipeline that
// pre-allocates everything at start-up).  cudaMalloc there is either
// forbidden, or it synchronises the whole device and breaks the caller's
// stream ordering and its memory accounting.  Such a caller owns the beta
// field, the lattice maps and the output, and passes device pointers; the
// only extra memory the reduction needs -- one partial-sum row per block
// and an arrival counter -- comes from a fixed array compiled into this
// library.
//
// The array is a file-scope __device__ variable: every GPU that loads the
// library holds it (1.4 MB) until the process exits, and every call on a
// device shares it.  Calls that may overlap on the GPU (different streams,
// no ordering between them) race on it and must be serialised by the
// caller.  The kernel keeps its small FP64 matrices in shared memory, so a
// launch needs no per-thread local-memory frame beyond a few spilled words.
//
// The first call in a process (and the first after a device reset) looks
// the array's device address up; because this library's kernels are loaded
// lazily, that first call also loads this file's module onto the device.
// Callers should therefore make one call at start-up, before any stream
// capture and before their own memory budget is fixed.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/bsglmm_gb300.h"
#include "bsg_device.cuh"

namespace bsg {
namespace {

constexpr int kNaVoxPerBlock = kPostThreads * kPostPerThread;  // 1024
constexpr int kNaMaxBlocks = BSG_NOALLOC_MAX_VOXELS / kNaVoxPerBlock;
constexpr int kNaPartialOffset = 32;  // words; keeps the rows 256-B aligned
constexpr size_t kNaWords = kNaPartialOffset + (size_t)kNaMaxBlocks * kPostVals;
static_assert(BSG_NOALLOC_MAX_VOXELS % kNaVoxPerBlock == 0, "block multiple");

// word 0: arrival counter; words 32..: block partials (doubles as bits).
static __device__ __align__(256) unsigned long long g_omega_scratch[kNaWords];

struct NaArgs {
  const float *beta;
  const int32_t *vox, *idxsc;
  int V, Vp, P, sy, sz, nblocks;
  double df;
  const double *chi2, *wnorm;
  uint32_t key0, key1, chain_id, sweep;
  double *omega;
  int32_t *status;
};

__device__ bool na_chol(double *A, int n) {
  for (int k = 0; k < n; ++k) {
    double d = A[k + k * n];
    if (!(d > 0.0)) return false;
    d = sqrt(d);
    A[k + k * n] = d;
    for (int j = k + 1; j < n; ++j) A[k + j * n] /= d;
    for (int j = k + 1; j < n; ++j)
      for (int i = j; i < n; ++i) A[j + i * n] -= A[k + i * n] * A[k + j * n];
  }
  return true;
}

// Inverse of G G' from the lower factor G, column by column (the scheme of
// cholesky.cpp:55-86); col is a work column of n doubles.
__device__ void na_inverse(const double *G, int n, double *out, double *col) {
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

// Gamma(a) by Marsaglia-Tsang on the sampler's gamma counters, so the draw
// equals the one bsg_run makes for the same (seed, chain, sweep).
__device__ double na_gamma(double a, uint32_t slot, const NaArgs &g, int *err) {
  const bool boost = a < 1.0;
  const double aa = boost ? a + 1.0 : a;
  const double dd = aa - 1.0 / 3.0, c = 1.0 / sqrt(9.0 * dd);
  for (int t = 0; t < kGammaMax; ++t) {
    const uint4 r = philox1(make_uint4(slot * 64u + (uint32_t)t, 0u, g.sweep,
                                       (g.chain_id << 8) | kTagGamma),
                            g.key0, g.key1);
    const double x = (double)normal_of(r.x), cx = c * x;
    if (!(cx > -1.0)) continue;
    const double v3 = (1.0 + cx) * (1.0 + cx) * (1.0 + cx);
    const double u = u_of_d(r.y), x2 = x * x;
    if (u < 1.0 - 0.0331 * x2 * x2 ||  // the squeeze, as the sampler's draw
        log(u) < 0.5 * x * x + dd * (1.0 - v3 + 3.0 * log1p(cx)))
      return dd * v3 * (boost ? pow(u_of_d(r.z), 1.0 / a) : 1.0);
  }
  *err |= kErrGammaCap;
  return dd;
}

// Bartlett draw after chol -> invert -> chol of S + I (the reference's
// covar.cpp:286-295 with cholesky.cpp:245-286), FP64, one thread.  The
// sampler's own draw (the last colour-1 block of bsg_run) reaches the same
// factor chol((S + I)^-1) by a reverse Cholesky instead: the factor is
// unique, so the two differ only by rounding.  wk holds the four P x P
// work matrices (shared memory of the calling block).
__device__ void na_wishart(const NaArgs &g, const double *tot, double *wk) {
  const int P = g.P;
  double *A = wk, *Ai = wk + kMaxP * kMaxP, *T = wk + 2 * kMaxP * kMaxP;
  double *B = wk + 3 * kMaxP * kMaxP;
  int err = 0;
  for (int r = 0; r < P; ++r)
    for (int c = 0; c <= r; ++c)
      A[c + r * P] = A[r + c * P] = tot[tri(r, c)] + (r == c ? 1.0 : 0.0);
  bool ok = na_chol(A, P);
  if (ok) {
    na_inverse(A, P, Ai, B);  // B is free until the Bartlett product
    ok = na_chol(Ai, P);
  }
  if (ok) {
    for (int i = 0; i < P * P; ++i) T[i] = 0.0;
    for (int i = 0; i < P; ++i) {
      const double c2 = g.chi2 ? g.chi2[i]
                               : 2.0 * na_gamma(0.5 * (g.df - i), (uint32_t)i, g, &err);
      T[i + i * P] = sqrt(c2);
      for (int j = 0; j < i; ++j) {
        const int m = i * (i - 1) / 2 + j;
        double z;
        if (g.wnorm) {
          z = g.wnorm[m];
        } else {
          const uint4 r = philox1(make_uint4((uint32_t)(m >> 2), 0u, g.sweep,
                                             (g.chain_id << 8) | kTagWNorm),
                                  g.key0, g.key1);
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
    if (fin)
      for (int i = 0; i < P * P; ++i) g.omega[i] = A[i];
    else
      err |= kErrNaN;
  } else {
    err |= kErrWishart;
  }
  if (g.status) *g.status = err;
}

// S = sum over in-mask voxels and their forward neighbours (+x, +y, +z) of
// the pair products, with the reference's indicator (the neighbour's row
// coefficient is nonzero, covar.cpp:235-253): the same edges and
// indicator as the sampler, which counts each edge from its colour-1 end
// over all six neighbours.  Here each thread sums its voxels' FP32 products
// in FP64, the block partials go to the scratch array, and the last block
// to arrive sums them in block order and draws Omega.  The sampler sums in
// FP32 warp trees first, so the two Omegas agree to rounding (about 1e-6
// relative), not bit for bit.
__global__ void __launch_bounds__(kPostThreads)
    omega_noalloc_kernel(NaArgs g, unsigned long long *scratch) {
  __shared__ double red[kPostThreads / 32][kMaxPairs];
  __shared__ double tot[kMaxPairs];
  __shared__ double wk[4 * kMaxP * kMaxP];
  __shared__ int is_last;
  const int P = g.P, npairs = P * (P + 1) / 2;
  double accp[kMaxPairs];
#pragma unroll
  for (int q = 0; q < kMaxPairs; ++q) accp[q] = 0.0;
  for (int t = 0; t < kPostPerThread; ++t) {
    const int pos = blockIdx.x * kNaVoxPerBlock + threadIdx.x + t * kPostThreads;
    if (pos >= g.V) break;
    const int p0 = g.vox[pos];
    const int sc = g.idxsc[p0];
    float bs[kMaxP];
#pragma unroll
    for (int p = 0; p < kMaxP; ++p) bs[p] = p < P ? g.beta[(size_t)p * g.Vp + sc] : 0.f;
    float pv[kMaxPairs];
#pragma unroll
    for (int q = 0; q < kMaxPairs; ++q) pv[q] = 0.f;
    const int off[3] = {1, g.sy, g.sz};
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      const int sn = g.idxsc[p0 + off[f]];
      float dd[kMaxP];
      bool ind[kMaxP];
#pragma unroll
      for (int p = 0; p < kMaxP; ++p) {
        const float bn = p < P ? g.beta[(size_t)p * g.Vp + sn] : 0.f;
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
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < kMaxPairs; ++q) {
    if (q >= npairs) continue;
    double v = accp[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp][q] = v;
  }
  __syncthreads();
  double *partials = reinterpret_cast<double *>(scratch + kNaPartialOffset);
  if (threadIdx.x < kMaxPairs) {
    double s = 0.0;
    if (threadIdx.x < npairs)
      for (int w = 0; w < kPostThreads / 32; ++w) s += red[w][threadIdx.x];
    partials[(size_t)blockIdx.x * kPostVals + threadIdx.x] = s;
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned long long prev = atomicAdd(scratch, 1ull);
    is_last = prev == (unsigned long long)(g.nblocks - 1);
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  if (threadIdx.x < kMaxPairs) {
    double s = 0.0;
    for (int b = 0; b < g.nblocks; ++b)
      s += __ldcg(partials + (size_t)b * kPostVals + threadIdx.x);
    tot[threadIdx.x] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    na_wishart(g, tot, wk);
    scratch[0] = 0ull;  // leave the counter cleared for the next call
  }
}

// Device address of the scratch array, looked up once per device and
// context.  The runtime's host-side symbol is only a stand-in: the address
// on the device comes from cudaGetSymbolAddress with the device current.
// A cudaDeviceReset destroys the context and the module with it, so the
// cache is keyed on the current driver context (cuCtxGetCurrent, reached
// through the runtime's driver entry point, so the library does not link
// libcuda itself) and looked up again when that changes.
typedef int (*CtxGetCurrentFn)(void **);

struct NaSlot {
  void *ctx = nullptr;
  unsigned long long *ptr = nullptr;
};
std::mutex g_na_mutex;
NaSlot g_na_slot[256];
CtxGetCurrentFn g_ctx_get = nullptr;
bool g_ctx_tried = false;

cudaError_t scratch_for_current_device(unsigned long long **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 256) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_na_mutex);
  if (!g_ctx_tried) {
    g_ctx_tried = true;
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_ctx_get = reinterpret_cast<CtxGetCurrentFn>(fn);
  }
  // (before the device's first runtime call no context is current yet:
  // the lookup below creates it, and the next call caches it)
  void *ctx = nullptr;
  if (g_ctx_get && g_ctx_get(&ctx) != 0) ctx = nullptr;
  NaSlot &slot = g_na_slot[dev];
  // without the driver entry point every call looks the address up again
  if (!slot.ptr || !ctx || slot.ctx != ctx) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_omega_scratch);
    if (e != cudaSuccess) return e;
    slot.ptr = static_cast<unsigned long long *>(p);
    slot.ctx = ctx;
  }
  *out = slot.ptr;
  return cudaSuccess;
}

}  // namespace
}  // namespace bsg

extern "C" bsg_status bsg_omega_update_noalloc(
    const float *spatcoef, const int32_t *vox, const int32_t *idxsc,
    int32_t nrow, int32_t ncol, int32_t V, int32_t Vp, int32_t P,
    int32_t df_offset, const double *chi2, const double *wnorm, uint64_t seed,
    uint32_t chain_id, int64_t sweep, double *omega, int32_t *status,
    void *stream) {
  using namespace bsg;
  if (!spatcoef || !vox || !idxsc || !omega) return BSG_ERR_INVALID;
  if (nrow < 1 || ncol < 1 || V < 1 || Vp < V || (chi2 == nullptr) != (wnorm == nullptr))
    return BSG_ERR_INVALID;
  if (P < 1 || P > kMaxP || V > BSG_NOALLOC_MAX_VOXELS) return BSG_ERR_UNSUPPORTED;
  if ((double)V + df_offset < P) return BSG_ERR_INVALID;
  unsigned long long *scratch = nullptr;
  if (scratch_for_current_device(&scratch) != cudaSuccess) return BSG_ERR_CUDA;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // The counter must start at zero even if an earlier call was cut short.
  if (cudaMemsetAsync(scratch, 0, sizeof(unsigned long long), st) != cudaSuccess)
    return BSG_ERR_CUDA;
  NaArgs g{};
  g.beta = spatcoef;
  g.vox = vox;
  g.idxsc = idxsc;
  g.V = V;
  g.Vp = Vp;
  g.P = P;
  g.sy = nrow + 2;
  g.sz = (nrow + 2) * (ncol + 2);
  g.nblocks = (V + kNaVoxPerBlock - 1) / kNaVoxPerBlock;
  g.df = (double)V + (double)df_offset;
  g.chi2 = chi2;
  g.wnorm = wnorm;
  g.key0 = (uint32_t)(seed & 0xFFFFFFFFu);
  g.key1 = (uint32_t)(seed >> 32);
  g.chain_id = chain_id;
  g.sweep = (uint32_t)sweep;
  g.omega = omega;
  g.status = status;
  omega_noalloc_kernel<<<g.nblocks, kPostThreads, 0, st>>>(g, scratch);
  return cudaGetLastError() == cudaSuccess ? BSG_OK : BSG_ERR_CUDA;
}
