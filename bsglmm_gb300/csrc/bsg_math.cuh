// bsg_math.cuh -- FP32 normal tail probability and inverse normal CDF used
// by the latent draws, written for instruction count (the latent draw runs
// N*V times per sweep).
//
//   phi_tail(x)    Q(x) = 1 - Phi(x) for x >= 0, relative error < 5e-7.
//                  Q = phi(x) R(x) with the Mills ratio R = Q / phi fitted
//                  for this library as a degree-(4,5) rational in x on
//                  [0, 9] (Sanathanan-Koerner least squares on relative
//                  error against 40-digit values; fit error 8e-9).  All
//                  coefficients are positive, so the rational stays finite
//                  and decays like 1/x beyond the fit range, as R does.
//                  1/sqrt(2 pi) is folded into the numerator.
//   ndtri_lower(p) Phi^-1(p) for 0 < p <= 1/2: Wichura (1988), Algorithm
//                  AS 241, PPND7 (relative error about 1e-7).
//
// The coefficient lines below are also read by tests/test_math_approx.py,
// which checks both functions in float32 against scipy.
#pragma once

namespace bsg {

// BEGIN-COEFFICIENTS
constexpr float kMillsN0 = 5.0000000402e-01f;
constexpr float kMillsN1 = 4.2497986971e-01f;
constexpr float kMillsN2 = 1.7361015356e-01f;
constexpr float kMillsN3 = 3.7449412193e-02f;
constexpr float kMillsN4 = 3.6586313638e-03f;
constexpr float kMillsD1 = 1.6478446270e+00f;
constexpr float kMillsD2 = 1.1620069222e+00f;
constexpr float kMillsD3 = 4.4409883918e-01f;
constexpr float kMillsD4 = 9.3884636633e-02f;
constexpr float kMillsD5 = 9.1705278204e-03f;
// AS 241 PPND7
constexpr float kPpA0 = 3.3871327179e+00f, kPpA1 = 5.0434271938e+01f;
constexpr float kPpA2 = 1.5929113202e+02f, kPpA3 = 5.9109374720e+01f;
constexpr float kPpB1 = 1.7895169469e+01f, kPpB2 = 7.8757757664e+01f;
constexpr float kPpB3 = 6.7187563600e+01f;
constexpr float kPpC0 = 1.4234372777e+00f, kPpC1 = 2.7568153900e+00f;
constexpr float kPpC2 = 1.3067284816e+00f, kPpC3 = 1.7023821103e-01f;
constexpr float kPpD1 = 7.3700164250e-01f, kPpD2 = 1.2021132975e-01f;
constexpr float kPpE0 = 6.6579051150e+00f, kPpE1 = 3.0812263860e+00f;
constexpr float kPpE2 = 4.2868294337e-01f, kPpE3 = 1.7337203997e-02f;
constexpr float kPpF1 = 2.4197894225e-01f, kPpF2 = 1.2258202635e-02f;
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

// Q(x) for x >= 0.  x*x is split into hi + lo so the exponent keeps full
// precision up to the 5-sigma switch of the latent sampler:
// exp(-x^2/2) = 2^(-hi log2(e)/2) (1 - lo/2).
__device__ __forceinline__ float phi_tail(float x) {
  const float hi = x * x;
  const float lo = fmaf(x, x, -hi);
  float e = ex2_approx(hi * -0.72134752044448170f);
  e = fmaf(e * lo, -0.5f, e);
  const float n = fmaf(fmaf(fmaf(fmaf(kMillsN4, x, kMillsN3), x, kMillsN2), x,
                            kMillsN1), x, kMillsN0);
  const float d = fmaf(fmaf(fmaf(fmaf(fmaf(kMillsD5, x, kMillsD4), x, kMillsD3),
                                 x, kMillsD2), x, kMillsD1), x, 1.0f);
  return e * n * rcp_approx(d);
}

// Phi^-1(p), 0 < p <= 1/2 (clamped below at the smallest normal float).
// The central and r <= 5 tail rationals share one reciprocal; r > 5
// (p < 1.4e-11) takes a separate, rarely executed branch.
__device__ __forceinline__ float ndtri_lower(float p) {
  p = fmaxf(p, 1.17549435e-38f);
  const float q = p - 0.5f;
  const float r = fmaf(-q, q, 0.180625f);
  const float nc = q * fmaf(fmaf(fmaf(kPpA3, r, kPpA2), r, kPpA1), r, kPpA0);
  const float dc = fmaf(fmaf(fmaf(kPpB3, r, kPpB2), r, kPpB1), r, 1.0f);
  const float nl = lg2_approx(p) * -0.69314718055994531f;  // -ln p > 0
  const float s = nl * rsqrt_approx(nl);
  float t = s - 1.6f;
  float nt = -fmaf(fmaf(fmaf(kPpC3, t, kPpC2), t, kPpC1), t, kPpC0);
  float dt = fmaf(fmaf(kPpD2, t, kPpD1), t, 1.0f);
  if (s > 5.0f) {
    t = s - 5.0f;
    nt = -fmaf(fmaf(fmaf(kPpE3, t, kPpE2), t, kPpE1), t, kPpE0);
    dt = fmaf(fmaf(kPpF2, t, kPpF1), t, 1.0f);
  }
  const bool central = q >= -0.425f;
  return (central ? nc : nt) * rcp_approx(central ? dc : dt);
}

}  // namespace bsg
