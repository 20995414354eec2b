// bsg_device.cuh -- device building blocks of the sampler: the Philox
// counter-based generator, the canonical uniform / normal / truncated-normal
// maps, register-resident Cholesky for P <= 8, and the A&S normal CDF.
#pragma once

#include <cstdint>

#include "bsg_internal.h"
#include "bsg_math.cuh"

namespace bsg {

// ------------------------------------------------------------- Philox ----
// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): ten rounds of
// (hi, lo) = M * x with M = 0xD2511F53 / 0xCD9E8D57 and Weyl key steps
// 0x9E3779B9 / 0xBB67AE85.  Stateless: every variate of the sampler is a
// pure function of (counter, key), so results do not depend on the launch
// shape and resuming from a checkpoint is exact.
#ifndef BSG_PHILOX_ROUND_KEYS
#define BSG_PHILOX_ROUND_KEYS 0  // 1: keep the 10 round keys in registers
#endif

struct PhiloxKey {
#if BSG_PHILOX_ROUND_KEYS
  uint32_t k0[10], k1[10];  // round keys, precomputed once per thread
  __device__ __forceinline__ void init(uint32_t a, uint32_t b) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
      k0[r] = a + (uint32_t)r * 0x9E3779B9u;
      k1[r] = b + (uint32_t)r * 0xBB67AE85u;
    }
  }
  __device__ __forceinline__ uint32_t r0(int r) const { return k0[r]; }
  __device__ __forceinline__ uint32_t r1(int r) const { return k1[r]; }
#else
  uint32_t a0, a1;  // round keys formed on the fly
  __device__ __forceinline__ void init(uint32_t a, uint32_t b) {
    a0 = a;
    a1 = b;
  }
  __device__ __forceinline__ uint32_t r0(int r) const {
    return a0 + (uint32_t)r * 0x9E3779B9u;
  }
  __device__ __forceinline__ uint32_t r1(int r) const {
    return a1 + (uint32_t)r * 0xBB67AE85u;
  }
#endif
};

__device__ __forceinline__ uint4 philox(uint4 c, const PhiloxKey &k) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.r0(r), lo1, hi0 ^ c.w ^ k.r1(r), lo0);
  }
  return c;
}

__device__ __forceinline__ uint4 philox1(uint4 c, uint32_t a, uint32_t b) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ a, lo1, hi0 ^ c.w ^ b, lo0);
    a += 0x9E3779B9u;
    b += 0xBB67AE85u;
  }
  return c;
}

__device__ __forceinline__ uint32_t pick4(uint4 r, int q) {
  return q == 0 ? r.x : q == 1 ? r.y : q == 2 ? r.z : r.w;
}

// ------------------------------------------------ canonical variate maps --
// u(k) = (k + 1/2) 2^-32 and 1 - u(k) = u(~k) are both formed from the
// integer, so each tail keeps full relative precision.
__device__ __forceinline__ float u_of(uint32_t k) {
  return fmaf((float)k, 0x1p-32f, 0x1p-33f);
}
__device__ __forceinline__ double u_of_d(uint32_t k) {
  return ((double)k + 0.5) * 0x1p-32;
}

// Standard normal by inversion with exact tails, in FP64 (CUDA's
// normcdfinv): the variates of the FP64 chain.
__device__ __forceinline__ double normal_of_d(uint32_t k) {
  const bool lo = k < 0x80000000u;
  const double t = normcdfinv(u_of_d(lo ? k : ~k));
  return lo ? t : -t;
}

// Standard normal by inversion with exact tails.
__device__ __forceinline__ float normal_of(uint32_t k) {
  const bool lo = k < 0x80000000u;
  const float t = ndtri_lower(u_of(lo ? k : ~k));
  return lo ? t : -t;
}

// N(0,1) truncated to (a, +inf) by inversion of u(k):
//   t = Phi^-1(Phi(a) + u Q(a)).  With T = Q(|a|):
//   a >= 0:  the argument is >= 1/2, so t = -Phi^-1(T (1-u));
//   a <  0:  the argument is u + T (1-u); below 1/2 t = Phi^-1 of it, else
//            t = -Phi^-1((1-T)(1-u)).
// Both tails keep relative precision; 1 - u = u(~k) comes from the integer.
// CLAMP guards the argument against underflow when a is unbounded (the
// supplied-variate path); the sampler clamps a at the 5-sigma switch.
template <bool CLAMP = false>
__device__ __forceinline__ float tn_lower_inv(float a, uint32_t k) {
  const float T = phi_tail(fabsf(a));
  const float uc = u_of(~k);
  const float tuc = __fmul_rn(T, uc);
  const float q1 = fmaf(T, uc, u_of(k));
  const bool neg = a < 0.f;
  const bool lo = neg && q1 < 0.5f;
  float arg = lo ? q1 : (neg ? __fsub_rn(uc, tuc) : tuc);
  if (CLAMP) arg = fmaxf(arg, 1.17549435e-38f);
  const float t = ndtri_lower(arg);
  return lo ? t : -t;
}

// Two draws of tn_lower_inv (CLAMP off) with the paired f32x2 arithmetic:
// exactly (tn_lower_inv(a.x, k0), tn_lower_inv(a.y, k1)) in half the FP32
// instructions.
__device__ __forceinline__ float2 u_of2(uint32_t k0, uint32_t k1) {
  return fma2(make_float2((float)k0, (float)k1), splat2(0x1p-32f), splat2(0x1p-33f));
}
__device__ __forceinline__ float2 tn_lower_inv2(float2 a, uint32_t k0, uint32_t k1) {
  const float2 T = phi_tail2(make_float2(fabsf(a.x), fabsf(a.y)));
  const float2 uc = u_of2(~k0, ~k1);
  const float2 tuc = mul2(T, uc);
  const float2 q1 = fma2(T, uc, u_of2(k0, k1));
  const float2 dd = sub2(uc, tuc);
  const bool n0 = a.x < 0.f, n1 = a.y < 0.f;
  const bool lo0 = n0 && q1.x < 0.5f, lo1 = n1 && q1.y < 0.5f;
  const float2 t = ndtri_lower2(make_float2(lo0 ? q1.x : (n0 ? dd.x : tuc.x),
                                            lo1 ? q1.y : (n1 ? dd.y : tuc.y)));
  return make_float2(lo0 ? t.x : -t.x, lo1 ? t.y : -t.y);
}

// Far tail a > kATail: Robert (1995) exponential proposal with rate
// alpha* = (a + sqrt(a^2+4))/2, accept with prob exp(-(x - alpha*)^2/2).
// Attempt t uses the pair (2(t&1), 2(t&1)+1) of the counter
// (i*8 + t/2, v, sweep, chain<<8 | ZTAIL).  Bounded: on the cap it returns
// a and clears *ok.
static __device__ __noinline__ float tn_lower_tail(float a, uint32_t i, uint32_t v,
                                            uint32_t sweep, uint32_t c3,
                                            uint32_t key0, uint32_t key1,
                                            int *ok) {
  const float as = 0.5f * (a + sqrtf(fmaf(a, a, 4.f)));
  for (int q = 0; q < kTailMax / 2; ++q) {
    const uint4 r = philox1(make_uint4(i * 8u + (uint32_t)q, v, sweep, c3),
                            key0, key1);
    float x = a - logf(u_of(r.x)) / as, d = x - as;
    if (logf(u_of(r.y)) < -0.5f * d * d) return x;
    x = a - logf(u_of(r.z)) / as;
    d = x - as;
    if (logf(u_of(r.w)) < -0.5f * d * d) return x;
  }
  *ok = 0;
  return a;
}

// ------------------------------------------------ scale-mixture latent ----
// One Marsaglia & Tsang (2000) attempt at Gamma(alpha, 1), alpha >= 1, with
// d = alpha - 1/3 and c = 1/sqrt(9 d) from a normal (bits kn) and a uniform
// (bits ku): g = d v^3 with v = 1 + c x, accepted by the squeeze
// u < 1 - 0.0331 x^4 or by log u < x^2/2 + d (1 - v^3 + log v^3).
// Products and sums are stated with explicit rounding (no contraction), so
// gamma_mt_try2 below decides exactly as two calls of this function.
__device__ __forceinline__ bool gamma_mt_try(float d, float c, uint32_t kn,
                                             uint32_t ku, float *g) {
  const float x = normal_of(kn);
  const float v = fmaf(c, x, 1.f);
  const float v3 = __fmul_rn(__fmul_rn(v, v), v);
  *g = __fmul_rn(d, v3);
  if (!(v > 0.f)) return false;
  const float u = u_of(ku), x2 = __fmul_rn(x, x);
  if (u < fmaf(__fmul_rn(-0.0331f, x2), x2, 1.f)) return true;
  return __fmul_rn(lg2_approx(u), kLn2) <
         fmaf(0.5f, x2, __fmul_rn(d, fmaf(lg2_approx(v3), kLn2, __fsub_rn(1.f, v3))));
}

// Standard normals of two words by inversion: exactly (normal_of(k0),
// normal_of(k1)).
__device__ __forceinline__ float2 normal_of2(uint32_t k0, uint32_t k1) {
  const bool l0 = k0 < 0x80000000u, l1 = k1 < 0x80000000u;
  const float2 t = ndtri_lower2(u_of2(l0 ? k0 : ~k0, l1 ? k1 : ~k1));
  return make_float2(l0 ? t.x : -t.x, l1 ? t.y : -t.y);
}

// Two first attempts of gamma_mt_try in f32x2 pairs, without control flow:
// g = (d v0^3, d v1^3) and the two acceptance decisions, exactly as two
// scalar calls.
__device__ __forceinline__ void gamma_mt_try2(float d, float c, uint32_t kn0, uint32_t kn1,
                                              uint32_t ku0, uint32_t ku1, float2 *g,
                                              bool *ok0, bool *ok1) {
  const float2 x = normal_of2(kn0, kn1);
  const float2 v = fma2(splat2(c), x, splat2(1.f));
  const float2 v3 = mul2(mul2(v, v), v);
  *g = mul2(splat2(d), v3);
  const float2 u = u_of2(ku0, ku1), x2 = mul2(x, x);
  const float2 sq = fma2(mul2(splat2(-0.0331f), x2), x2, splat2(1.f));
  const float2 lu = mul2(make_float2(lg2_approx(u.x), lg2_approx(u.y)), splat2(kLn2));
  const float2 rhs =
      fma2(splat2(0.5f), x2,
           mul2(splat2(d), fma2(make_float2(lg2_approx(v3.x), lg2_approx(v3.y)),
                                splat2(kLn2), sub2(splat2(1.f), v3))));
  *ok0 = v.x > 0.f && (u.x < sq.x || lu.x < rhs.x);
  *ok1 = v.y > 0.f && (u.y < sq.y || lu.y < rhs.y);
}

// Further attempts after a rejected first one: attempt pairs from counters
// (i * 32 + q, v, sweep, c3), at most kGammaMax attempts in all; sets
// *ok = 0 and returns d (the mode) if none is accepted.
static __device__ __noinline__ float gamma_mt_more(float d, float c, uint32_t i,
                                                   uint32_t v, uint32_t sweep,
                                                   uint32_t c3, uint32_t key0,
                                                   uint32_t key1, int *ok) {
  float g = d;
  for (int q = 0; q < (kGammaMax - 1) / 2; ++q) {
    const uint4 r = philox1(make_uint4(i * 32u + (uint32_t)q, v, sweep, c3), key0, key1);
    if (gamma_mt_try(d, c, r.x, r.y, &g)) return g;
    if (gamma_mt_try(d, c, r.z, r.w, &g)) return g;
  }
  *ok = 0;
  return d;
}

// Logistic lesion probability of the t/logit links (ProbLogitGPU,
// covarGPU.cu:1695-1721): exp(x / lf) / (1 + exp(x / lf)), written so that
// it cannot overflow.
__device__ __forceinline__ float prob_logit(float x, float inv_lf) {
  return 1.f / (1.f + expf(-x * inv_lf));
}

// Abramowitz & Stegun 26.2.17 normal CDF (covarGPU.cu:1672-1693 uses the
// same published polynomial).
__device__ __forceinline__ float prob_sdnorm(float x) {
  const float b1 = 0.319381530f, b2 = -0.356563782f, b3 = 1.781477937f;
  const float b4 = -1.821255978f, b5 = 1.330274429f, p = 0.2316419f;
  const float c = 0.39894228f;
  const float ax = fabsf(x);
  const float t = 1.0f / (1.0f + p * ax);
  const float tail =
      c * expf(-x * x / 2.0f) * t *
      (t * (t * (t * (t * b5 + b4) + b3) + b2) + b1);
  return x >= 0.0f ? 1.0f - tail : tail;
}

// ----------------------------------------- packed lower-triangular algebra
__host__ __device__ constexpr int tri(int r, int c) { return r * (r + 1) / 2 + c; }

// Outer-product Cholesky in place on packed lower storage (the scheme of
// cholesky.cpp:13-33, with divisions as there).  Returns false if a pivot
// is not positive.
template <int P, typename T>
__device__ __forceinline__ bool chol_packed(T (&A)[P * (P + 1) / 2]) {
  bool ok = true;
#pragma unroll
  for (int k = 0; k < P; ++k) {
    T d = A[tri(k, k)];
    ok = ok && (d > T(0));
    d = sqrt(d);
    A[tri(k, k)] = d;
#pragma unroll
    for (int j = k + 1; j < P; ++j) A[tri(j, k)] = A[tri(j, k)] / d;
#pragma unroll
    for (int j = k + 1; j < P; ++j)
#pragma unroll
      for (int i = j; i < P; ++i) A[tri(i, j)] -= A[tri(i, k)] * A[tri(j, k)];
  }
  return ok;
}

// x := G^-1 x (forward substitution).
template <int P, typename T>
__device__ __forceinline__ void solve_lower(const T (&G)[P * (P + 1) / 2],
                                            T (&x)[P]) {
#pragma unroll
  for (int a = 0; a < P; ++a) {
    T s = T(0);
#pragma unroll
    for (int q = 0; q < a; ++q) s += G[tri(a, q)] * x[q];
    x[a] = (x[a] - s) / G[tri(a, a)];
  }
}

// x := G^-T x (back substitution).
template <int P, typename T>
__device__ __forceinline__ void solve_upper(const T (&G)[P * (P + 1) / 2],
                                            T (&x)[P]) {
#pragma unroll
  for (int a = P - 1; a >= 0; --a) {
    T s = T(0);
#pragma unroll
    for (int q = a + 1; q < P; ++q) s += G[tri(q, a)] * x[q];
    x[a] = (x[a] - s) / G[tri(a, a)];
  }
}

}  // namespace bsg
