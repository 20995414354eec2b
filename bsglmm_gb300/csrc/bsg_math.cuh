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
  const float e = ex2_approx(x * (x * -0.72134752044448170f));
  const float n = fmaf(fmaf(fmaf(kMillsN3, x, kMillsN2), x, kMillsN1), x, kMillsN0);
  const float d = fmaf(fmaf(fmaf(fmaf(kMillsD4, x, kMillsD3), x, kMillsD2), x,
                            kMillsD1), x, 1.0f);
  return e * n * rcp_approx(d);
}

// Phi^-1(p), 0 < p <= 1/2; p must be a normal float (callers clamp where
// it could underflow).
__device__ __forceinline__ float ndtri_lower(float p) {
  const float l = -lg2_approx(p);  // >= 1
  const float rho = l * rsqrt_approx(l);
  const float n = fmaf(fmaf(fmaf(fmaf(fmaf(kNdtN5, rho, kNdtN4), rho, kNdtN3),
                                 rho, kNdtN2), rho, kNdtN1), rho, kNdtN0);
  const float d = fmaf(fmaf(fmaf(fmaf(kNdtD4, rho, kNdtD3), rho, kNdtD2), rho,
                            kNdtD1), rho, 1.0f);
  return n * rcp_approx(d);
}

}  // namespace bsg
