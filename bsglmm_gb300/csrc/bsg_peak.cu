// bsg_peak.cu -- FP32 FMA throughput microbenchmark: the denominator of the
// fused kernel's roofline (no FP32 SIMT peak is published for GB300).
#include <cuda_runtime.h>

#include "../../include/bsglmm_gb300.h"

namespace {

// Eight independent FMA chains per thread, unrolled so the scheduler
// always has ready FFMA instructions; the result is stored so nothing is
// dead code.
__global__ void __launch_bounds__(256) fma_peak_kernel(float *out, int iters,
                                                       float a, float b) {
  float x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = (float)(threadIdx.x + k) * 1e-3f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u)
#pragma unroll
      for (int k = 0; k < 8; ++k) x[k] = fmaf(x[k], a, b);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" bsg_status bsg_fp32_peak(int32_t device, double *tflops) {
  if (!tflops) return BSG_ERR_INVALID;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return BSG_ERR_NO_DEVICE;
  if (cudaSetDevice(device) != cudaSuccess) return BSG_ERR_INVALID;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return BSG_ERR_CUDA;
  const int threads = 256, blocks = prop.multiProcessorCount * 8;
  const int iters = 4096;
  float *out = nullptr;
  if (cudaMalloc(&out, sizeof(float) * blocks * threads) != cudaSuccess)
    return BSG_ERR_CUDA;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_peak_kernel<<<blocks, threads>>>(out, 64, 0.999f, 1e-4f);  // warm-up
  float best = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {
    cudaEventRecord(e0);
    fma_peak_kernel<<<blocks, threads>>>(out, iters, 0.999f, 1e-4f);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return BSG_ERR_CUDA;
  const double flops = 2.0 * 8.0 * 16.0 * (double)iters * blocks * threads;
  *tflops = flops / (best * 1e-3) / 1e12;
  return BSG_OK;
}
