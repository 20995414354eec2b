// bsg_kernels.cu -- dispatcher of the fused colour kernel, the
// lesion-probability map and outcome bit packing.
#include <algorithm>

#include "bsg_device.cuh"

namespace bsg {

cudaError_t launch_fused_l1(int, int, bool, const DatasetDev *, ChainDev *,
                            const BlockMap *, int, int, const Supplied &,
                            cudaStream_t, bool);
cudaError_t launch_fused_l2(int, int, bool, const DatasetDev *, ChainDev *,
                            const BlockMap *, int, int, const Supplied &,
                            cudaStream_t, bool);
cudaError_t launch_fused_l4(int, int, bool, const DatasetDev *, ChainDev *,
                            const BlockMap *, int, int, const Supplied &,
                            cudaStream_t, bool);
cudaError_t launch_fused_l8(int, int, bool, const DatasetDev *, ChainDev *,
                            const BlockMap *, int, int, const Supplied &,
                            cudaStream_t, bool);

bool fused_supported(int P, int lpv, int threads) {
  if (P < 1 || P > kMaxP) return false;
  if (lpv != 1 && lpv != 2 && lpv != 4 && lpv != 8) return false;
  if (threads != 64 && threads != 128 && threads != 256) return false;
  return true;
}

cudaError_t launch_fused(int P, int lpv, int threads, bool supplied,
                         const DatasetDev *ds, ChainDev *ch,
                         const BlockMap *map, int nblocks, int colour,
                         const Supplied &sup, cudaStream_t st, bool pdl) {
  switch (lpv) {
    case 1:
      return launch_fused_l1(P, threads, supplied, ds, ch, map, nblocks,
                             colour, sup, st, pdl);
    case 2:
      return launch_fused_l2(P, threads, supplied, ds, ch, map, nblocks,
                             colour, sup, st, pdl);
    case 4:
      return launch_fused_l4(P, threads, supplied, ds, ch, map, nblocks,
                             colour, sup, st, pdl);
    case 8:
      return launch_fused_l8(P, threads, supplied, ds, ch, map, nblocks,
                             colour, sup, st, pdl);
    default:
      return cudaErrorInvalidValue;
  }
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
    const float bwm = *ch.wm_beta * (d.wm ? d.wm[v] : 1.f);
    for (int g = 0; g < d.S; ++g) {
      const float b = ch.beta[(size_t)g * d.Vp + sc];
      // t/logit links: ProbLogitGPU (covarGPU.cu:1695-1721), without WM
      prb[(size_t)g * d.V + v] = ch.model != 1 ? prob_logit(b, ch.inv_lf)
                                               : prob_sdnorm(b + bwm);
    }
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

// ----------------------------------------------------------------- fill --
__global__ void fill_kernel(float *p, size_t n, float value) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    p[i] = value;
}

cudaError_t launch_fill(float *p, size_t n, float value, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const size_t blocks = std::min<size_t>((n + 255) / 256, 8192);
  fill_kernel<<<(unsigned)blocks, 256, 0, st>>>(p, n, value);
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
