// bsg_mma.cuh -- the warp-level BF16x3 tensor-core form of the colour
// kernel's X'(Z - b_WM WM) contraction (the reference's loop at
// covarGPU.cu:327-351, fused_colour_kernel<..., TC = true>).
//
// One warp owns 32 voxels.  Every 16 subjects (a K slice) each voxel-thread
// stores its 16 latent values, split z = hi + lo into two BF16 parts, as
// two rows of the warp's Z tile in shared memory; the design slice, split
// the same way, is staged once per subject chunk for the whole block.  One
// m16n8k16 MMA per 8-voxel tile then adds [X_hi ; X_lo]' Z_hi (rows 0-7 and
// 8-15 of the accumulator) and a second adds [X_hi ; 0]' Z_lo, so that
// rows p and p + 8 sum to X_hi'Z_hi + X_hi'Z_lo + X_lo'Z_hi, the BF16x3
// split product accumulated in FP32 (the dropped X_lo'Z_lo term and the
// rounding of the lo parts leave about 2^-16 relative per product).
//
// Layouts (bytes):
//   design slice s   XA + s * 64P:  [quad q][covariate p < P][8 BF16], quad
//                    0: hi, subjects 0-7; 1: lo, 0-7; 2: hi, 8-15;
//                    3: lo, 8-15 (the four 8x8 matrices of one ldmatrix.x4,
//                    in the order of the m16n8k16 A fragment); rows p >= P
//                    point at a zero row
//   Z tile (per warp) [part (hi, lo)][half (subjects 0-7, 8-15)][voxel][8 BF16]
//                    (16-byte rows, so ldmatrix reads are conflict-free)
#pragma once

#include <cuda_bf16.h>

#include <cstdint>

#include "bsg_internal.h"

namespace bsg {

constexpr int kTcSliceBytesPerCov = 64;         // 4 quads x 16 bytes
constexpr int kTcSlices = kChunk / 16;          // K slices per subject chunk
constexpr int kTcZTileBytes = 2 * 2 * 32 * 16;  // per warp

// Dynamic shared memory of the TC kernel: the chunk's design slices, one
// zero row, and one Z tile per warp.
__host__ __device__ constexpr int tc_smem_bytes(int P, int threads) {
  return kTcSlices * kTcSliceBytesPerCov * P + 16 + (threads / 32) * kTcZTileBytes;
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void ldmatrix_x4(uint32_t addr, uint32_t &r0, uint32_t &r1,
                                            uint32_t &r2, uint32_t &r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}

// D (16x8 FP32) += A (16x16 BF16, row) * B (16x8 BF16, col).
__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], uint32_t a0, uint32_t a1,
                                               uint32_t a2, uint32_t a3, uint32_t b0,
                                               uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, "
      "{%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// The BF16 split of a pair of values: hi = bf16(z), lo = bf16(z - hi).
__device__ __forceinline__ void split_bf16x2(float2 z, uint32_t &hi, uint32_t &lo) {
  const __nv_bfloat162 h = __float22bfloat162_rn(z);
  const float2 hf = __bfloat1622float2(h);
  const __nv_bfloat162 l = __float22bfloat162_rn(make_float2(z.x - hf.x, z.y - hf.y));
  hi = *reinterpret_cast<const uint32_t *>(&h);
  lo = *reinterpret_cast<const uint32_t *>(&l);
}

__device__ __forceinline__ uint16_t bf16_bits(float x) {
  const __nv_bfloat16 b = __float2bfloat16_rn(x);
  return *reinterpret_cast<const uint16_t *>(&b);
}

// Stages the design of one subject chunk as BF16 hi/lo slices (all threads
// of the block; x beyond the chunk's cn subjects is 0).  Writes the zero row.
template <int P>
__device__ __forceinline__ void tc_stage_design(unsigned char *xa, const float *covar, int N,
                                                int i0, int cn, int tid, int nthreads) {
  uint16_t *xs = reinterpret_cast<uint16_t *>(xa);
  for (int t = tid; t < P * kChunk; t += nthreads) {
    const int p = t / kChunk, ii = t - p * kChunk;
    const float x = ii < cn ? covar[(size_t)p * N + i0 + ii] : 0.f;
    const uint16_t hi = bf16_bits(x);
    const float hf = __bfloat162float(*reinterpret_cast<const __nv_bfloat16 *>(&hi));
    const uint16_t lo = bf16_bits(x - hf);
    const int s = ii >> 4, k = ii & 15, q = (k >> 3) * 2;
    uint16_t *row = xs + (size_t)s * (kTcSliceBytesPerCov / 2) * P;
    row[(q * P + p) * 8 + (k & 7)] = hi;
    row[((q + 1) * P + p) * 8 + (k & 7)] = lo;
  }
  if (tid < 8) xs[(size_t)kTcSlices * (kTcSliceBytesPerCov / 2) * P + tid] = 0;
}

// Stores the warp-lane's 8 latent values (4 pairs, subjects 8*half + 0..7
// of the current K slice) as BF16 hi and lo rows of its voxel in the warp's
// Z tile.
__device__ __forceinline__ void tc_store_z(unsigned char *zt, int lane, int half,
                                           const float2 (&z)[4]) {
  uint32_t hw[4], lw[4];
#pragma unroll
  for (int h = 0; h < 4; ++h) split_bf16x2(z[h], hw[h], lw[h]);
  *reinterpret_cast<uint4 *>(zt + (0 * 2 + half) * 512 + lane * 16) =
      make_uint4(hw[0], hw[1], hw[2], hw[3]);
  *reinterpret_cast<uint4 *>(zt + (1 * 2 + half) * 512 + lane * 16) =
      make_uint4(lw[0], lw[1], lw[2], lw[3]);
}

// Adds one K slice to the warp's four 8-voxel accumulator tiles d[j]: 8
// MMAs (X_hi/X_lo against Z_hi, X_hi against Z_lo per tile).
template <int P>
__device__ __forceinline__ void tc_slice(const unsigned char *xa, int s, const unsigned char *zt,
                                         int lane, float (&d)[4][4]) {
  const int m = lane >> 3, r = lane & 7;
  const uint32_t arow =
      r < P ? smem_u32(xa + (size_t)s * kTcSliceBytesPerCov * P + (m * P + r) * 16)
            : smem_u32(xa + (size_t)kTcSlices * kTcSliceBytesPerCov * P);
  uint32_t a0, a1, a2, a3;
  ldmatrix_x4(arow, a0, a1, a2, a3);
#pragma unroll
  for (int part = 0; part < 2; ++part) {
#pragma unroll
    for (int jp = 0; jp < 2; ++jp) {
      // matrices: (half 0, tile 2jp), (half 1, tile 2jp), (half 0, tile
      // 2jp+1), (half 1, tile 2jp+1); lane's row = voxel 8 tile + r
      const int half = m & 1, tile = 2 * jp + (m >> 1);
      uint32_t b0, b1, b2, b3;
      ldmatrix_x4(smem_u32(zt + (part * 2 + half) * 512 + (8 * tile + r) * 16), b0, b1, b2,
                  b3);
      if (part == 0) {
        mma_bf16_16816(d[2 * jp], a0, a1, a2, a3, b0, b1);
        mma_bf16_16816(d[2 * jp + 1], a0, a1, a2, a3, b2, b3);
      } else {
        mma_bf16_16816(d[2 * jp], a0, 0u, a2, 0u, b0, b1);
        mma_bf16_16816(d[2 * jp + 1], a0, 0u, a2, 0u, b2, b3);
      }
    }
  }
}

// acc[p] of the lane's voxel from the four accumulator tiles: rows p and
// p + 8 summed, transposed through the warp's Z tile (free after the last
// slice).
template <int P>
__device__ __forceinline__ void tc_finish(unsigned char *zt, int lane, const float (&d)[4][4],
                                          float (&acc)[P]) {
  float *t = reinterpret_cast<float *>(zt);  // [32 voxels][8 covariates]
  const int g = lane >> 2, c = lane & 3;
  __syncwarp();
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    t[(8 * j + 2 * c) * 8 + g] = d[j][0] + d[j][2];
    t[(8 * j + 2 * c + 1) * 8 + g] = d[j][1] + d[j][3];
  }
  __syncwarp();
#pragma unroll
  for (int p = 0; p < P; ++p) acc[p] = t[lane * 8 + p];
  __syncwarp();
}

}  // namespace bsg
