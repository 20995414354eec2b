// bsg_math.cuh -- FP32 normal tail probability and inverse normal CDF used
// by the latent draws, written for instruction count (the latent draw runs
// N*V times per sweep).
//
//   phi_tail(x)    Q(x) = 1 - Phi(x) for x >= 0, relative error < 1.2e-6.
//                  Q = phi(x) R(x) with the Mills ratio R = Q / phi fitted
//                  for this library as a degree-(3,4) rational in x on
//                  [0, 9] (Sanathanan-Koerner least squares on relative
//                  error against 40-digit values; fit error 6.8e-7).  All
//                  coefficients are positive, so the rational stays finite
//                  and decays like 1/x beyond the fit range, as R does.
//                  1/sqrt(2 pi) is folded into the numerator.
//   ndtri_lower(p) Phi^-1(p) for 0 < p <= 1/2 as one degree-(5,4) rational
//                  in rho = sqrt(-log2 p), fitted for this library by least
//                  squares on [1e-38, 1/2] (absolute error 4e-8; in float32
//                  with the MUFU approximations, absolute error < 1e-6 near
//                  p = 1/2 and relative error < 1e-6 beyond).  One branch-
//                  free evaluation replaces the two regions of Wichura's
//                  AS 241.
//
// The coefficient lines below are also read by tests/test_math_approx.py,
// which checks both functions in float32 against scipy.
#pragma once

namespace bsg {

// BEGIN-COEFFICIENTS
constexpr float kMillsN0 = 4.9999965914e-01f;
constexpr float kMillsN1 = 3.5229928749e-01f;
constexpr float kMillsN2 = 1.1418309070e-01f;
constexpr float kMillsN3 = 1.5839596273e-02f;
constexpr float kMillsD1 = 1.5024640812e+00f;
constexpr float kMillsD2 = 9.2728669120e-01f;
constexpr float kMillsD3 = 2.8589874975e-01f;
constexpr float kMillsD4 = 3.9713598231e-02f;
constexpr float kNdtN0 = 3.2486578541e+00f;
constexpr float kNdtN1 = 1.1044934586e+01f;
constexpr float kNdtN2 = -2.8432280551e+00f;
constexpr float kNdtN3 = -8.8573652006e+00f;
constexpr float kNdtN4 = -2.4531834439e+00f;
constexpr float kNdtN5 = -1.3981649743e-01f;
constexpr float kNdtD1 = 7.1093794929e+00f;
constexpr float kNdtD2 = 7.9459598930e+00f;
constexpr float kNdtD3 = 2.0855841983e+00f;
constexpr float kNdtD4 = 1.1873321670e-01f;
// END-COEFFICIENTS
constexpr float kLog2eHalfNeg = -0.72134752044448170f;  // -log2(e) / 2
constexpr float kLn2 = 0.693147181f;

// MUFU approximations through documented PTX (ex2 / lg2 / rcp / rsqrt
// .approx, flush-to-zero): one instruction each, errors of a few ulp.
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float lg2_approx(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rsqrt_approx(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Q(x) for x >= 0.  The rounding of x*x costs at most 7.5e-7 relative at
// the 5-sigma switch of the latent sampler (the only range where Q's
// relative precision matters).
__device__ __forceinline__ float phi_tail(float x) {
  const float e = ex2_approx(__fmul_rn(x, __fmul_rn(x, kLog2eHalfNeg)));
  const float n = fmaf(fmaf(fmaf(kMillsN3, x, kMillsN2), x, kMillsN1), x, kMillsN0);
  const float d = fmaf(fmaf(fmaf(fmaf(kMillsD4, x, kMillsD3), x, kMillsD2), x,
                            kMillsD1), x, 1.0f);
  return __fmul_rn(__fmul_rn(e, n), rcp_approx(d));
}

// Phi^-1(p), 0 < p <= 1/2; p must be a normal float (callers clamp where
// it could underflow).
__device__ __forceinline__ float ndtri_lower(float p) {
  const float l = -lg2_approx(p);  // >= 1
  const float rho = __fmul_rn(l, rsqrt_approx(l));
  const float n = fmaf(fmaf(fmaf(fmaf(fmaf(kNdtN5, rho, kNdtN4), rho, kNdtN3),
                                 rho, kNdtN2), rho, kNdtN1), rho, kNdtN0);
  const float d = fmaf(fmaf(fmaf(fmaf(kNdtD4, rho, kNdtD3), rho, kNdtD2), rho,
                            kNdtD1), rho, 1.0f);
  return __fmul_rn(n, rcp_approx(d));
}

// ------------------------------------------------- two lanes at a time ----
// The f32x2 forms of fma / mul / add / sub (sm_100 and later) evaluate two
// independent FP32 operations in one instruction, with the rounding of the
// scalar __fmaf_rn / __fmul_rn / __fadd_rn / __fsub_rn per component.  The
// scalar functions above state their products and sums with those
// intrinsics (no contraction), so phi_tail2 / ndtri_lower2 return exactly
// (phi_tail(x.x), phi_tail(x.y)) and (ndtri_lower(p.x), ndtri_lower(p.y)).
__device__ __forceinline__ float2 splat2(float c) { return make_float2(c, c); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
  return __ffma2_rn(a, b, c);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\t"
      "mov.b64 rb, {%4, %5};\n\t"
      "sub.rn.f32x2 rd, ra, rb;\n\t"
      "mov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}

__device__ __forceinline__ float2 phi_tail2(float2 x) {
  const float2 s = mul2(x, mul2(x, splat2(kLog2eHalfNeg)));
  const float2 e = make_float2(ex2_approx(s.x), ex2_approx(s.y));
  const float2 n = fma2(fma2(fma2(splat2(kMillsN3), x, splat2(kMillsN2)), x,
                             splat2(kMillsN1)), x, splat2(kMillsN0));
  const float2 d = fma2(fma2(fma2(fma2(splat2(kMillsD4), x, splat2(kMillsD3)), x,
                                  splat2(kMillsD2)), x, splat2(kMillsD1)), x,
                        splat2(1.0f));
  return mul2(mul2(e, n), make_float2(rcp_approx(d.x), rcp_approx(d.y)));
}

__device__ __forceinline__ float2 ndtri_lower2(float2 p) {
  const float2 l = make_float2(-lg2_approx(p.x), -lg2_approx(p.y));
  const float2 rho = mul2(l, make_float2(rsqrt_approx(l.x), rsqrt_approx(l.y)));
  const float2 n = fma2(fma2(fma2(fma2(fma2(splat2(kNdtN5), rho, splat2(kNdtN4)), rho,
                                       splat2(kNdtN3)), rho, splat2(kNdtN2)), rho,
                             splat2(kNdtN1)), rho, splat2(kNdtN0));
  const float2 d = fma2(fma2(fma2(fma2(splat2(kNdtD4), rho, splat2(kNdtD3)), rho,
                                  splat2(kNdtD2)), rho, splat2(kNdtD1)), rho,
                        splat2(1.0f));
  return mul2(n, make_float2(rcp_approx(d.x), rcp_approx(d.y)));
}

}  // namespace bsg
