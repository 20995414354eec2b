// bsg_fused.cuh -- the fused colour kernel: for every voxel of one
// checkerboard colour it draws the Albert-Chib latent Z_iv for all
// subjects from the packed outcome bits, accumulates X'(Z - b_WM WM) in
// registers (Z never reaches memory), forms the conditional precision
// Q = X'X + n_v Omega and mean vector, factors Q in registers and draws
// beta_v.
//
// Replaces Z_GPU1 (covarGPU.cu:1368-1428) + Spat_Coef_Probit
// (covarGPU.cu:293-396) and the CPU updateZ / Spat_Coefff
// (covar.cpp:302-325, 121-187).  Drawing Z_v immediately before beta_v is
// the same Gibbs transition as "all Z, then beta colour 0, then beta
// colour 1": Z_v depends only on (beta_v, Y_v) and beta_v's conditional
// only on (Z_v, the other colour's beta).
//
// Work mapping: LPV lanes per voxel; each lane takes whole 32-subject
// outcome words (w = k, k+LPV, ...) of a subject chunk staged in shared
// memory, so one Philox call serves four consecutive subjects of one lane.
#pragma once

#include "bsg_device.cuh"

namespace bsg {

// Resident 256-thread blocks per SM asked of ptxas: three (85 registers) up
// to P = 5, two (128 registers) above, measured fastest on the brain-sized
// study; BSG_FUSED_MIN_BLOCKS overrides it for tuning builds.
template <int P>
constexpr int fused_min_blocks() {
#ifdef BSG_FUSED_MIN_BLOCKS
  return BSG_FUSED_MIN_BLOCKS;
#else
  return P <= 5 ? 3 : 2;
#endif
}

template <int P, int LPV, bool SUPP>
__global__ void __launch_bounds__(256, fused_min_blocks<P>())
    fused_colour_kernel(const DatasetDev *__restrict__ dsv,
                        ChainDev *__restrict__ chv,
                        const BlockMap *__restrict__ map, int colour,
                        Supplied sup) {
  constexpr int NT = P * (P + 1) / 2;
  __shared__ float Xs[P][kChunkPad];
  __shared__ float Om[P * P], Xtx[P * P];

  const BlockMap bm = map[blockIdx.x];
  const ChainDev &ch = chv[bm.chain];
  const DatasetDev &d = dsv[ch.dataset];
  const int tid = threadIdx.x;
  const int g = tid / LPV, k = tid % LPV;
  const int nc = d.n[colour];
  const int j = bm.start + g;
  const bool active = j < nc;
  const int N = d.N, Vp = d.Vp;
  const uint32_t sweep = (uint32_t)(*ch.sweep);
  const uint32_t cid = ch.chain_id << 8;

  for (int t = tid; t < P * P; t += blockDim.x) {
    Om[t] = ch.omega_f[t];
    Xtx[t] = d.xtx[t];
  }

  float beta[P], acc[P];
  int v = 0, sc = 0;
  float bwm = 0.f;
  if (active) {
    sc = d.nb[colour][j];
    v = d.vidx[colour][j];
    bwm = ch.beta_wm * (d.wm ? d.wm[v] : 1.f);
#pragma unroll
    for (int p = 0; p < P; ++p) beta[p] = ch.beta[(size_t)p * Vp + sc];
  } else {
#pragma unroll
    for (int p = 0; p < P; ++p) beta[p] = 0.f;
  }
#pragma unroll
  for (int p = 0; p < P; ++p) acc[p] = 0.f;

  PhiloxKey key;
  if (!SUPP) key.init(ch.key0, ch.key1);
  int ok = 1;
  const uint32_t *yb = d.ybits[colour];

  for (int i0 = 0; i0 < N; i0 += kChunk) {
    const int cn = min(kChunk, N - i0);
    __syncthreads();
    for (int t = tid; t < P * kChunk; t += blockDim.x) {
      const int p = t / kChunk, ii = t - p * kChunk;
      Xs[p][ii + (ii >> 5)] = ii < cn ? d.covar[(size_t)p * N + i0 + ii] : 0.f;
    }
    __syncthreads();
    if (active) {
      // One subject: mu = bwm + x'beta; a = -mu if Y = 1 else mu (sign-bit
      // flip by ymask = Y << 31); t ~ N(0,1) on (a, inf);
      // Z - bwm = x'beta + (Y ? t : -t); acc += x (Z - bwm).
      auto subject = [&](int col, uint32_t ymask, uint32_t kk, uint32_t isub) {
        float x[P];
        float m0 = 0.f;
#pragma unroll
        for (int p = 0; p < P; ++p) {
          x[p] = Xs[p][col];
          m0 = fmaf(beta[p], x[p], m0);
        }
        const float a = __uint_as_float(__float_as_uint(m0 + bwm) ^ ymask);
        float t;
        if (SUPP || a <= kATail) {
          t = tn_lower_inv(a, kk);
        } else {
          t = tn_lower_tail(a, isub, (uint32_t)v, sweep, cid | kTagZTail,
                            ch.key0, ch.key1, &ok);
        }
        const float zr = m0 + __uint_as_float(__float_as_uint(t) ^ ymask ^ 0x80000000u);
#pragma unroll
        for (int p = 0; p < P; ++p) acc[p] = fmaf(x[p], zr, acc[p]);
      };
      auto variate = [&](uint4 r, int q, uint32_t isub) -> uint32_t {
        if (SUPP) return __ldg(sup.ubits + (size_t)isub * d.V + v);
        return pick4(r, q);
      };
      const int nw = (cn + 31) >> 5;
      for (int wl = k; wl < nw; wl += LPV) {
        const int w = (i0 >> 5) + wl;
        uint32_t yw = __ldg(yb + (size_t)w * nc + j);
        const int nbits = min(32, cn - (wl << 5));
        const int xo = (wl << 5) + wl;  // padded offset of bit 0
        const uint32_t i00 = (uint32_t)(i0 + (wl << 5));
        if (nbits == 32) {
#pragma unroll 1
          for (int b = 0; b < 32; b += 4) {
            const uint32_t i = i00 + (uint32_t)b;
            uint4 r = make_uint4(0, 0, 0, 0);
            if (!SUPP) r = philox(make_uint4(i >> 2, (uint32_t)v, sweep, cid | kTagZ), key);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              subject(xo + b + q, yw << 31, variate(r, q, i + q), i + q);
              yw >>= 1;
            }
          }
        } else {
          for (int b = 0; b < nbits; b += 4) {
            const uint32_t i = i00 + (uint32_t)b;
            uint4 r = make_uint4(0, 0, 0, 0);
            if (!SUPP) r = philox(make_uint4(i >> 2, (uint32_t)v, sweep, cid | kTagZ), key);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              if (b + q < nbits) subject(xo + b + q, yw << 31, variate(r, q, i + q), i + q);
              yw >>= 1;
            }
          }
        }
      }
    }
  }

  if (LPV > 1) {
#pragma unroll
    for (int p = 0; p < P; ++p)
#pragma unroll
      for (int o = LPV / 2; o > 0; o >>= 1)
        acc[p] += __shfl_xor_sync(0xffffffffu, acc[p], o);
  }
  if (!active || k != 0) {
    if (!ok) atomicOr(ch.status, kErrTnCap);
    return;
  }

  // ---- beta_v | rest  (Spat_Coefff, covar.cpp:142-180) -----------------
  float sumV[P];
#pragma unroll
  for (int p = 0; p < P; ++p) sumV[p] = 0.f;
#pragma unroll
  for (int t = 1; t <= 6; ++t) {
    const int sn = d.nb[colour][(size_t)t * nc + j];
#pragma unroll
    for (int p = 0; p < P; ++p) sumV[p] += ch.beta[(size_t)p * Vp + sn];
  }
  const float nnb = (float)d.nnb[colour][j];
  float b[P], Q[NT];
#pragma unroll
  for (int a = 0; a < P; ++a) {
    float s = acc[a];
#pragma unroll
    for (int q = 0; q < P; ++q) s += Om[q + a * P] * sumV[q];
    b[a] = s;
#pragma unroll
    for (int q = 0; q <= a; ++q) Q[tri(a, q)] = Xtx[q + a * P] + nnb * Om[q + a * P];
  }
  bool okc = chol_packed<P>(Q);

  float e[P];
  if (SUPP) {
#pragma unroll
    for (int p = 0; p < P; ++p) e[p] = __ldg(sup.normals + (size_t)v * P + p);
  } else {
#pragma unroll
    for (int p0 = 0; p0 < P; p0 += 4) {
      const uint4 r = philox(make_uint4((uint32_t)(p0 >> 2), (uint32_t)v, sweep,
                                        cid | kTagBeta), key);
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (p0 + q < P) e[p0 + q] = normal_of(pick4(r, q));
    }
  }

  float out[P];
  if (!SUPP || sup.form == 1) {
    // Q = G G':  m = G^-T G^-1 b,  beta = m + G^-T e = G^-T (G^-1 b + e)
    solve_lower<P>(Q, b);
#pragma unroll
    for (int p = 0; p < P; ++p) out[p] = b[p] + e[p];
    solve_upper<P>(Q, out);
  } else {
    // Reference draw (covar.cpp:168-177): V = Q^-1 by columns
    // (cholesky_invert_float), m = V b, L = chol(V), beta = m + L e.
    float Vc[P][P];  // Vc[k][q] = entry q of column k of Q^-1
#pragma unroll
    for (int kk = 0; kk < P; ++kk) {
      float x[P];
#pragma unroll
      for (int q = 0; q < P; ++q) x[q] = (q == kk) ? 1.f : 0.f;
      solve_lower<P>(Q, x);
      solve_upper<P>(Q, x);
#pragma unroll
      for (int q = 0; q < P; ++q) Vc[kk][q] = x[q];
    }
    float m[P], L[NT];
#pragma unroll
    for (int a = 0; a < P; ++a) {
      float s = 0.f;
#pragma unroll
      for (int q = 0; q < P; ++q) s += Vc[a][q] * b[q];
      m[a] = s;
#pragma unroll
      for (int q = 0; q <= a; ++q) L[tri(a, q)] = Vc[a][q];
    }
    okc = chol_packed<P>(L) && okc;
#pragma unroll
    for (int a = 0; a < P; ++a) {
      float s = 0.f;
#pragma unroll
      for (int q = 0; q <= a; ++q) s += L[tri(a, q)] * e[q];
      out[a] = s + m[a];
    }
  }

  bool fin = true;
#pragma unroll
  for (int p = 0; p < P; ++p) fin = fin && isfinite(out[p]);
  if (okc && fin) {
#pragma unroll
    for (int p = 0; p < P; ++p) ch.beta[(size_t)p * Vp + sc] = out[p];
  }
  const int err = (ok ? 0 : kErrTnCap) | (okc ? 0 : kErrChol) |
                  ((okc && !fin) ? kErrNaN : 0);
  if (err) atomicOr(ch.status, err);
}

// Instantiation helper used by bsg_fused_l*.cu.
template <int LPV>
cudaError_t launch_fused_lpv(int P, int threads, bool supplied,
                             const DatasetDev *ds, ChainDev *ch,
                             const BlockMap *map, int nblocks, int colour,
                             const Supplied &sup, cudaStream_t st) {
  if (nblocks <= 0) return cudaSuccess;
#define BSG_CASE(PP)                                                        \
  case PP:                                                                  \
    if (supplied) {                                                         \
      if constexpr (LPV == 1)                                               \
        fused_colour_kernel<PP, LPV, true>                                  \
            <<<nblocks, threads, 0, st>>>(ds, ch, map, colour, sup);        \
      else                                                                  \
        return cudaErrorInvalidValue;                                       \
    } else {                                                                \
      fused_colour_kernel<PP, LPV, false>                                   \
          <<<nblocks, threads, 0, st>>>(ds, ch, map, colour, sup);          \
    }                                                                       \
    break;
  switch (P) {
    BSG_CASE(1)
    BSG_CASE(2)
    BSG_CASE(3)
    BSG_CASE(4)
    BSG_CASE(5)
    BSG_CASE(6)
    BSG_CASE(7)
    BSG_CASE(8)
    default:
      return cudaErrorInvalidValue;
  }
#undef BSG_CASE
  return cudaGetLastError();
}

}  // namespace bsg
