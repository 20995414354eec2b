// bsg_fused.cuh -- the fused colour kernel: for every voxel of one
// checkerboard colour it draws the Albert-Chib latent Z_iv for all
// subjects from the packed outcome bits, accumulates X'(Z - b_WM WM) in
// registers (Z never reaches memory), forms the conditional precision
// Q = X'X + n_v Omega and mean vector, factors Q in registers and draws
// beta_v.  With the new beta_v it also adds the kept sweep's FP64 running
// sums and the column sums, and (colour 1) the voxel's Omega pair products;
// the last colour-1 block of a chain draws Omega.  A sweep is two launches.
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
// memory, so one Philox call serves four consecutive subjects of one lane
// (the probit kernel takes two or four calls, 8 or 16 subjects, per step,
// and does its FP32 arithmetic on pairs of subjects with the f32x2
// instructions).
#pragma once

#include <type_traits>

#include "bsg_mma.cuh"
#include "bsg_wishart.cuh"

namespace bsg {

// Resident 256-thread blocks per SM asked of ptxas.  The probit kernel
// comes in two forms of its whole-word step (below): WIDE draws 16 subjects
// from four Philox calls at two blocks of 128 registers; the narrow form
// draws 8 from two calls at three blocks of 80 registers up to P = 5 (two
// above).  On the brain-sized study (N = 1000, P = 5) WIDE is 6.5 % faster
// per sweep; on 64 chains of a 50-subject study in one launch the narrow
// form's extra resident warps win by 27 %.  BSG_FUSED_MIN_BLOCKS overrides
// it for tuning builds.
template <int P, bool MIX = false, bool WIDE = false>
constexpr int fused_min_blocks() {
#ifdef BSG_FUSED_MIN_BLOCKS
  return BSG_FUSED_MIN_BLOCKS;
#else
  // the t/logit kernel also keeps the voxel's X' Phi X in registers
  return MIX ? (P <= 5 ? 2 : 1) : ((WIDE || P > 5) ? 2 : 3);
#endif
}

// MIX: the t/logit links (the reference's MODEL 0 and 2, Z_GPU2 and
// Phi_GPU, covarGPU.cu:1430-1563, and the weighted Spat_Coef,
// covarGPU.cu:398-513): Z_iv ~ N(mu, 1/phi_iv) truncated by Y, then
// phi_iv | Z, beta ~ Gamma((nu + 1) / 2, rate (nu + (Z - mu)^2) / 2), and the
// coefficient draw uses X' Phi X and X' Phi (Z - b_WM WM).
// WMU: chains that draw beta_WM (one lane per voxel) also carry each voxel's
// term of its conditional mean through the block partials.
// TC: the probit kernel's X'(Z - b_WM WM) on the tensor cores as a BF16x3
// split product (bsg_mma.cuh), one lane per voxel; the rest is unchanged.
// WIDE: the 16-subject whole-word step (identical results).
template <int P, int LPV, bool SUPP, bool MIX = false, bool WMU = false, bool TC = false,
          bool WIDE = false>
__global__ void __launch_bounds__(256, fused_min_blocks<P, MIX, WIDE>())
    fused_colour_kernel(const DatasetDev *__restrict__ dsv,
                        ChainDev *__restrict__ chv,
                        const BlockMap *__restrict__ map, int colour,
                        Supplied sup) {
  static_assert(!TC || (!SUPP && !MIX && !WMU && LPV == 1),
                "the tensor-core X'Z serves the probit production kernel");
  static_assert(!WIDE || (!SUPP && !MIX && !TC && LPV == 1),
                "the 16-subject step serves the probit production kernels");
  constexpr int NT = P * (P + 1) / 2;
  constexpr int PP = P <= 4 ? 4 : 8;  // design row padded to float4s
  // The probit kernel stages the design as subject pairs: pair row m holds
  // (x_2m,p, x_2m+1,p) for p = 0..P-1, so one f32x2 operation serves two
  // subjects; a pad of 4 floats after every 16 pair rows keeps the lanes of
  // a voxel (32 subjects = 16 pair rows apart) on distinct banks.  The
  // other kernels keep one padded row per subject (a pad row per 32).
  constexpr bool PAIRX = !MIX && !SUPP;
  constexpr int RW = 2 * ((P + 1) & ~1);  // floats per pair row
  constexpr int XS_FLOATS = PAIRX ? (kChunk / 2) * RW + (kChunk / 32) * 4 : kChunkPad * PP;
  __shared__ __align__(16) float Xs[XS_FLOATS];
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
  // This colour's own sweep counter: the previous launch of this colour
  // finished before this one started (see the dependency protocol below).
  const long long sweep_ll = ch.sweep[colour];
  const uint32_t sweep = (uint32_t)sweep_ll;
  const uint32_t cid = ch.chain_id << 8;
  const bool kept =
      sweep_ll > ch.burnin && (sweep_ll % (ch.thin > 0 ? ch.thin : 1)) == 0;

  float beta[P], acc[P];
  int v = 0, sc = 0;
  float bwm = 0.f, wmv = 0.f;
  if (active) {
    sc = d.nb[colour][j];
    v = d.vidx[colour][j];
    wmv = d.wm ? d.wm[v] : 1.f;
    // beta_WM is final since the previous colour-1 launch: with its update
    // on, colour-0 launches do not start early (no programmatic launch)
    bwm = *ch.wm_beta * wmv;
#pragma unroll
    for (int p = 0; p < P; ++p) beta[p] = ch.beta[(size_t)p * Vp + sc];
  } else {
#pragma unroll
    for (int p = 0; p < P; ++p) beta[p] = 0.f;
  }
#pragma unroll
  for (int p = 0; p < P; ++p) acc[p] = 0.f;
  // PAIRX: the coefficients duplicated into both halves of an f32x2 operand,
  // and X'(Z - b_WM WM) of the even (.x) and odd (.y) subjects
  float2 bb[PAIRX ? P : 1], acc2[PAIRX ? P : 1];
#pragma unroll
  for (int p = 0; p < (PAIRX ? P : 1); ++p) {
    bb[p] = make_float2(beta[p], beta[p]);
    acc2[p] = make_float2(0.f, 0.f);
  }
  constexpr int NQ = MIX ? NT : 1;
  float qw[NQ];  // MIX: this voxel's X' Phi X, packed lower
#pragma unroll
  for (int q = 0; q < NQ; ++q) qw[q] = 0.f;

  PhiloxKey key;
  if (!SUPP) key.init(ch.key0, ch.key1);
  int ok = 1;
  const uint32_t *yb = d.ybits[colour];
  // TC: the chunk's design slices and this warp's Z tile (dynamic shared
  // memory), the warp's four 8-voxel accumulator tiles, and whether any lane
  // of the warp has a voxel (the MMAs need the whole warp: lanes without one
  // contribute zeros)
  extern __shared__ __align__(16) unsigned char tc_smem[];
  unsigned char *tc_zt = TC ? tc_smem + kTcSlices * kTcSliceBytesPerCov * P + 16 +
                                  (tid >> 5) * kTcZTileBytes
                            : nullptr;
  float tcd[TC ? 4 : 1][4];
#pragma unroll
  for (int jt = 0; jt < (TC ? 4 : 1); ++jt)
#pragma unroll
    for (int q = 0; q < 4; ++q) tcd[jt][q] = 0.f;
  const bool run = TC ? __any_sync(0xffffffffu, active) : active;

  for (int i0 = 0; i0 < N; i0 += kChunk) {
    const int cn = min(kChunk, N - i0);
    __syncthreads();
    for (int t = tid; t < P * kChunk; t += blockDim.x) {
      const int p = t / kChunk, ii = t - p * kChunk;
      const float xv = ii < cn ? d.covar[(size_t)p * N + i0 + ii] : 0.f;
      if constexpr (PAIRX) {
        const int m = ii >> 1;
        Xs[m * RW + (m >> 4) * 4 + 2 * p + (ii & 1)] = xv;
      } else {
        Xs[(ii + (ii >> 5)) * PP + p] = xv;
      }
    }
    if constexpr (TC) tc_stage_design<P>(tc_smem, d.covar, N, i0, cn, tid, blockDim.x);
    __syncthreads();
    if (run) {
      // One subject: mu = bwm + x'beta; a = -mu if Y = 1 else mu (sign-bit
      // flip by ymask = Y << 31); t ~ N(0,1) on (a, inf);
      // Z - bwm = x'beta + (Y ? t : -t); acc += x (Z - bwm).
      auto subject = [&](int col, uint32_t ymask, uint32_t kk, uint32_t isub,
                         uint32_t gn, uint32_t gu, float ph) {
        float x[P];
        if constexpr (PAIRX) {
          const int ii = col - col / 33, m = ii >> 1;  // col = ii + ii / 32
          const float *xr = &Xs[m * RW + (m >> 4) * 4 + (ii & 1)];
#pragma unroll
          for (int p = 0; p < P; ++p) x[p] = xr[2 * p];
        } else {
          const float4 v0 = *reinterpret_cast<const float4 *>(&Xs[col * PP]);
          x[0] = v0.x;
          if (P > 1) x[1] = v0.y;
          if (P > 2) x[2] = v0.z;
          if (P > 3) x[3] = v0.w;
          if (P > 4) {
            const float4 v1 = *reinterpret_cast<const float4 *>(&Xs[col * PP + 4]);
            x[4] = v1.x;
            if (P > 5) x[5] = v1.y;
            if (P > 6) x[6] = v1.z;
            if (P > 7) x[7] = v1.w;
          }
        }
        float m0 = 0.f;
#pragma unroll
        for (int p = 0; p < P; ++p) m0 = fmaf(beta[p], x[p], m0);
        if constexpr (MIX) {
          // standardised: (Z - mu) sqrt(phi) ~ N(0, 1) on (a, inf) after the
          // outcome's sign flip, a = -/+ mu sqrt(phi)
          float *pp = ch.phi[colour] + (size_t)isub * nc + j;
          const float sd = rsqrt_approx(ph);
          const float a = __uint_as_float(__float_as_uint((m0 + bwm) * (ph * sd)) ^ ymask);
          float t = tn_lower_inv(fminf(a, kATail), kk);
          if (__any_sync(__activemask(), a > kATail) && a > kATail)
            t = tn_lower_tail(a, isub, (uint32_t)v, sweep, cid | kTagZTail, ch.key0,
                              ch.key1, &ok);
          const float r = __uint_as_float(__float_as_uint(t * sd) ^ ymask ^ 0x80000000u);
          const float zr = m0 + r;  // Z - b_WM WM
          float gm;
          if (ch.t_df == 3.f) {
            // Gamma(2, 1) = Exp(1) + Exp(1) = -ln(u1 u2), exactly (t link)
            gm = __fmul_rn(lg2_approx(__fmul_rn(u_of(gn), u_of(gu))), -kLn2);
          } else if (!gamma_mt_try(ch.mix_d, ch.mix_c, gn, gu, &gm)) {
            gm = gamma_mt_more(ch.mix_d, ch.mix_c, isub, (uint32_t)v, sweep,
                               cid | kTagPhiMore, ch.key0, ch.key1, &ok);
          }
          // the new weight 2 g / (r^2 + nu) with a MUFU reciprocal (r^2 + nu
          // >= 3; a few ulp, where the IEEE division's check and slow path
          // cost 4-6 % of the sweep)
          const float phn = __fmul_rn(2.f * gm, rcp_approx(fmaf(r, r, ch.t_df)));
          *pp = phn;
          const float wz = phn * zr;
          float px[P];
#pragma unroll
          for (int p = 0; p < P; ++p) {
            acc[p] = fmaf(x[p], wz, acc[p]);
            px[p] = phn * x[p];
          }
#pragma unroll
          for (int a2 = 0; a2 < P; ++a2)
#pragma unroll
            for (int b2 = 0; b2 <= a2; ++b2)
              qw[tri(a2, b2)] = fmaf(px[a2], x[b2], qw[tri(a2, b2)]);
          return;
        }
        const float a = __uint_as_float(__float_as_uint(m0 + bwm) ^ ymask);
        float t;
        if (SUPP) {
          t = tn_lower_inv<true>(a, kk);
        } else {
          t = tn_lower_inv(fminf(a, kATail), kk);
          // beyond 5 sigma: bounded rejection, entered by a warp only when
          // one of its lanes needs it
          if (__any_sync(__activemask(), a > kATail) && a > kATail)
            t = tn_lower_tail(a, isub, (uint32_t)v, sweep, cid | kTagZTail,
                              ch.key0, ch.key1, &ok);
        }
        const float zr = m0 + __uint_as_float(__float_as_uint(t) ^ ymask ^ 0x80000000u);
#pragma unroll
        for (int p = 0; p < P; ++p) {
          if constexpr (PAIRX)
            acc2[p].x = fmaf(x[p], zr, acc2[p].x);
          else
            acc[p] = fmaf(x[p], zr, acc[p]);
        }
      };
      // The probit groups on subject pairs (PAIRX): G groups of four subjects
      // (G Philox calls), x'beta, the inversion and X'(Z - bwm) each as 2G
      // f32x2 pairs of subjects (ii0 + 2h, ii0 + 2h + 1); one tail vote for
      // all 4G.  Per subject the same arithmetic as `subject`; the even and
      // odd subjects' X'Z sums are kept apart until the end of the voxel.
      // The whole-word step takes G = kGroups: with WIDE four Philox calls,
      // 16 subjects, eight independent pair chains for the scheduler (0.527
      // ms per sweep of the brain-sized study, N = 1000, P = 5, against 0.563
      // for G = 2 at three resident blocks; the same at P = 8), else two
      // (G = 2 gives four chains and was measured 1.6 % faster per sweep
      // than G = 1).  The results do not depend on G.
      constexpr int kGroups = WIDE ? 4 : 2;
      auto groupp = [&](auto gsz, int ii0, uint32_t ywg, const uint4 *rs, uint32_t i) {
        constexpr int G = decltype(gsz)::value;
        constexpr int H = 2 * G;
        const int m = ii0 >> 1;  // a multiple of H: rows m..m+H-1 share one pad group
        const float *xr0 = &Xs[m * RW + (m >> 4) * 4];
        float2 m0h[H], zh[H];
        float aq[2 * H];
#pragma unroll
        for (int h = 0; h < H; ++h) {
          const float *xr = xr0 + h * RW;
          float2 s = make_float2(0.f, 0.f);
#pragma unroll
          for (int p = 0; p + 1 < P; p += 2) {
            const float4 v4 = *reinterpret_cast<const float4 *>(xr + 2 * p);
            s = fma2(make_float2(v4.x, v4.y), bb[p], s);
            s = fma2(make_float2(v4.z, v4.w), bb[p + 1], s);
          }
          if (P & 1)
            s = fma2(*reinterpret_cast<const float2 *>(xr + 2 * (P - 1)), bb[P - 1], s);
          m0h[h] = s;
          const float2 a = add2(s, make_float2(bwm, bwm));
          aq[2 * h] = __uint_as_float(__float_as_uint(a.x) ^ ((ywg >> (2 * h)) << 31));
          aq[2 * h + 1] = __uint_as_float(__float_as_uint(a.y) ^ ((ywg >> (2 * h + 1)) << 31));
        }
        // (a subject beyond kATail gets a meaningless inversion here; the
        // rejection sampler below replaces it)
        float amax = aq[0];
#pragma unroll
        for (int h = 0; h < H; ++h) {
          const uint4 rr = rs[h >> 1];
          const float2 t = tn_lower_inv2(make_float2(aq[2 * h], aq[2 * h + 1]),
                                         pick4(rr, (2 * h) & 3), pick4(rr, (2 * h + 1) & 3));
          const uint32_t y0 = (ywg >> (2 * h)) << 31, y1 = (ywg >> (2 * h + 1)) << 31;
          zh[h] = add2(m0h[h],
                       make_float2(__uint_as_float(__float_as_uint(t.x) ^ y0 ^ 0x80000000u),
                                   __uint_as_float(__float_as_uint(t.y) ^ y1 ^ 0x80000000u)));
          amax = fmaxf(amax, fmaxf(aq[2 * h], aq[2 * h + 1]));
        }
        if (__any_sync(__activemask(), amax > kATail)) {
#pragma unroll
          for (int q = 0; q < 2 * H; ++q)
            if (aq[q] > kATail) {
              const uint32_t ym = (ywg >> q) << 31;
              const float t = tn_lower_tail(aq[q], i + q, (uint32_t)v, sweep,
                                            cid | kTagZTail, ch.key0, ch.key1, &ok);
              const float m0 = (q & 1) ? m0h[q >> 1].y : m0h[q >> 1].x;
              const float z = m0 + __uint_as_float(__float_as_uint(t) ^ ym ^ 0x80000000u);
              if (q & 1)
                zh[q >> 1].y = z;
              else
                zh[q >> 1].x = z;
            }
        }
        if constexpr (TC) {
          // the eight values go to this voxel's row of the warp's Z tile
          // (zeros from lanes without a voxel); the MMAs follow per slice
          if constexpr (H == 4) {
            float2 zz[4];
#pragma unroll
            for (int h = 0; h < 4; ++h) zz[h] = active ? zh[h] : make_float2(0.f, 0.f);
            tc_store_z(tc_zt, tid & 31, (ii0 >> 3) & 1, zz);
          }
        } else {
#pragma unroll
          for (int h = 0; h < H; ++h) {
            const float *xr = xr0 + h * RW;
#pragma unroll
            for (int p = 0; p + 1 < P; p += 2) {
              const float4 v4 = *reinterpret_cast<const float4 *>(xr + 2 * p);
              acc2[p] = fma2(make_float2(v4.x, v4.y), zh[h], acc2[p]);
              acc2[p + 1] = fma2(make_float2(v4.z, v4.w), zh[h], acc2[p + 1]);
            }
            if (P & 1)
              acc2[P - 1] = fma2(*reinterpret_cast<const float2 *>(xr + 2 * (P - 1)), zh[h],
                                 acc2[P - 1]);
          }
        }
      };
      // The t/logit links, four subjects: Z by inversion and the first
      // Marsaglia-Tsang attempt for all four without control flow, one vote
      // for the rare tail draws and gamma retries, then phi, X' Phi (Z - bwm)
      // and X' Phi X for the four in order.  The same arithmetic as `subject`.
      auto group4_mix = [&](int col0, uint32_t yw4, uint4 r, uint32_t i, uint4 g0,
                            uint4 g1, const float (&ph4)[4]) {
        float m0q[4], aq[4], sdq[4], rq[4], gq[4];
        bool bad[4];
        auto row = [&](int col, float (&x)[P]) {
          const float4 v0 = *reinterpret_cast<const float4 *>(&Xs[col * PP]);
          x[0] = v0.x;
          if (P > 1) x[1] = v0.y;
          if (P > 2) x[2] = v0.z;
          if (P > 3) x[3] = v0.w;
          if (P > 4) {
            const float4 v1 = *reinterpret_cast<const float4 *>(&Xs[col * PP + 4]);
            x[4] = v1.x;
            if (P > 5) x[5] = v1.y;
            if (P > 6) x[6] = v1.z;
            if (P > 7) x[7] = v1.w;
          }
        };
        const bool t3 = ch.t_df == 3.f;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          float x[P];
          row(col0 + q, x);
          float m0 = 0.f;
#pragma unroll
          for (int p = 0; p < P; ++p) m0 = fmaf(beta[p], x[p], m0);
          const uint32_t ym = (yw4 >> q) << 31;
          const float ph = ph4[q];
          const float sd = rsqrt_approx(ph);
          m0q[q] = m0;
          sdq[q] = sd;
          aq[q] = __uint_as_float(__float_as_uint((m0 + bwm) * (ph * sd)) ^ ym);
        }
        // the inversions and the first gamma attempts as f32x2 pairs:
        // subjects (0, 1) and (2, 3); the gamma words of subject 2h + s are
        // (gn, gu) = (.x, .y) for s = 0 and (.z, .w) for s = 1 of g_h
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int q0 = 2 * h, q1 = q0 + 1;
          // (beyond kATail the inversion is replaced by the rejection draw)
          const float2 t = tn_lower_inv2(make_float2(aq[q0], aq[q1]), pick4(r, q0),
                                         pick4(r, q1));
          const float2 rr = mul2(t, make_float2(sdq[q0], sdq[q1]));
          rq[q0] = __uint_as_float(__float_as_uint(rr.x) ^ ((yw4 >> q0) << 31) ^ 0x80000000u);
          rq[q1] = __uint_as_float(__float_as_uint(rr.y) ^ ((yw4 >> q1) << 31) ^ 0x80000000u);
          const uint4 gg = h ? g1 : g0;
          if (t3) {
            const float2 uu = mul2(u_of2(gg.x, gg.z), u_of2(gg.y, gg.w));
            const float2 g = mul2(make_float2(lg2_approx(uu.x), lg2_approx(uu.y)),
                                  splat2(-kLn2));
            gq[q0] = g.x;
            gq[q1] = g.y;
            bad[q0] = bad[q1] = false;
          } else {
            float2 g;
            bool o0, o1;
            gamma_mt_try2(ch.mix_d, ch.mix_c, gg.x, gg.z, gg.y, gg.w, &g, &o0, &o1);
            gq[q0] = g.x;
            gq[q1] = g.y;
            bad[q0] = !o0;
            bad[q1] = !o1;
          }
        }
        const bool rare = (fmaxf(fmaxf(aq[0], aq[1]), fmaxf(aq[2], aq[3])) > kATail) |
                          bad[0] | bad[1] | bad[2] | bad[3];
        if (__any_sync(__activemask(), rare)) {
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            if (aq[q] > kATail) {
              const uint32_t ym = (yw4 >> q) << 31;
              const float t = tn_lower_tail(aq[q], i + q, (uint32_t)v, sweep,
                                            cid | kTagZTail, ch.key0, ch.key1, &ok);
              rq[q] = __uint_as_float(__float_as_uint(t * sdq[q]) ^ ym ^ 0x80000000u);
            }
            if (bad[q])
              gq[q] = gamma_mt_more(ch.mix_d, ch.mix_c, i + q, (uint32_t)v, sweep,
                                    cid | kTagPhiMore, ch.key0, ch.key1, &ok);
          }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          float x[P];
          row(col0 + q, x);
          const float phn = __fmul_rn(2.f * gq[q], rcp_approx(fmaf(rq[q], rq[q], ch.t_df)));
          ch.phi[colour][(size_t)(i + q) * nc + j] = phn;
          const float wz = phn * (m0q[q] + rq[q]);
          float px[P];
#pragma unroll
          for (int p = 0; p < P; ++p) {
            acc[p] = fmaf(x[p], wz, acc[p]);
            px[p] = phn * x[p];
          }
#pragma unroll
          for (int a2 = 0; a2 < P; ++a2)
#pragma unroll
            for (int b2 = 0; b2 <= a2; ++b2)
              qw[tri(a2, b2) < NQ ? tri(a2, b2) : 0] =
                  fmaf(px[a2], x[b2], qw[tri(a2, b2) < NQ ? tri(a2, b2) : 0]);
        }
      };
      auto variate = [&](uint4 r, int q, uint32_t isub) -> uint32_t {
        if (SUPP) return __ldg(sup.ubits + (size_t)isub * d.V + v);
        return pick4(r, q);
      };
      const int nw = (cn + 31) >> 5;
      for (int wl = k; wl < nw; wl += LPV) {
        const int w = (i0 >> 5) + wl;
        uint32_t yw = (TC && !active) ? 0u : __ldg(yb + (size_t)w * nc + j);
        const int nbits = min(32, cn - (wl << 5));
        const int xo = (wl << 5) + wl;  // padded offset of bit 0
        const uint32_t i00 = (uint32_t)(i0 + (wl << 5));
        // MIX: the gamma variates of subjects i, i + 1 come from counter
        // i / 2 (normal, uniform each)
        auto gpair = [&](uint32_t i) -> uint4 {
          if (!MIX) return make_uint4(0, 0, 0, 0);
          return philox(make_uint4(i >> 1, (uint32_t)v, sweep, cid | kTagPhi), key);
        };
        // MIX: the weights phi of a group of four subjects are loaded one
        // group ahead (the stores of the current group may alias as far as
        // the compiler knows, so it would not hoist them itself)
        const float *phb = MIX ? ch.phi[colour] + j : nullptr;
        // (TC: a ragged last word also takes the whole-word path; its
        // subjects beyond the chunk have x = 0 and add nothing)
        if (TC || nbits == 32) {
          float phc[4] = {1.f, 1.f, 1.f, 1.f}, phx[4] = {1.f, 1.f, 1.f, 1.f};
          if (MIX) {
#pragma unroll
            for (int q = 0; q < 4; ++q) phc[q] = phb[(size_t)(i00 + q) * nc];
          }
          if constexpr (PAIRX) {
#pragma unroll 1
            for (int b = 0; b < 32; b += 4 * kGroups) {
              const uint32_t i = i00 + (uint32_t)b;
              uint4 rs[kGroups];
#pragma unroll
              for (int q = 0; q < kGroups; ++q)
                rs[q] = philox(make_uint4((i >> 2) + q, (uint32_t)v, sweep, cid | kTagZ), key);
              groupp(std::integral_constant<int, kGroups>{}, (wl << 5) + b, yw, rs, i);
              yw >>= 4 * kGroups;
              if constexpr (TC) {
                if (b & 8) {  // a 16-subject slice is complete
                  __syncwarp();
                  tc_slice<P>(tc_smem, ((wl << 5) + b) >> 4, tc_zt, tid & 31, tcd);
                  __syncwarp();
                }
              }
            }
          } else {
#pragma unroll 1
            for (int b = 0; b < 32; b += 4) {
              const uint32_t i = i00 + (uint32_t)b;
              if (MIX && b + 4 < 32) {
#pragma unroll
                for (int q = 0; q < 4; ++q) phx[q] = phb[(size_t)(i + 4 + q) * nc];
              }
              uint4 r = make_uint4(0, 0, 0, 0);
              if (!SUPP) r = philox(make_uint4(i >> 2, (uint32_t)v, sweep, cid | kTagZ), key);
              if constexpr (MIX) {
                group4_mix(xo + b, yw, r, i, gpair(i), gpair(i + 2), phc);
                yw >>= 4;
              } else {
                const uint4 g0 = gpair(i), g1 = gpair(i + 2);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                  const uint4 gq = q < 2 ? g0 : g1;
                  subject(xo + b + q, yw << 31, variate(r, q, i + q), i + q,
                          (q & 1) ? gq.z : gq.x, (q & 1) ? gq.w : gq.y, phc[q]);
                  yw >>= 1;
                }
              }
              if (MIX) {
#pragma unroll
                for (int q = 0; q < 4; ++q) phc[q] = phx[q];
              }
            }
          }
        } else {
          for (int b = 0; b < nbits; b += 4) {
            const uint32_t i = i00 + (uint32_t)b;
            uint4 r = make_uint4(0, 0, 0, 0);
            if (!SUPP) r = philox(make_uint4(i >> 2, (uint32_t)v, sweep, cid | kTagZ), key);
            if constexpr (PAIRX) {
              if (b + 4 <= nbits) {  // a whole group of the last word
                groupp(std::integral_constant<int, 1>{}, (wl << 5) + b, yw, &r, i);
                yw >>= 4;
                continue;
              }
            }
            const uint4 g0 = gpair(i), g1 = gpair(i + 2);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              const uint4 gq = q < 2 ? g0 : g1;
              if (b + q < nbits)
                subject(xo + b + q, yw << 31, variate(r, q, i + q), i + q,
                        (q & 1) ? gq.z : gq.x, (q & 1) ? gq.w : gq.y,
                        MIX ? phb[(size_t)(i + q) * nc] : 1.f);
              yw >>= 1;
            }
          }
        }
      }
    }
  }

  if constexpr (TC) {
    if (run) tc_finish<P>(tc_zt, tid & 31, tcd, acc);
  } else if constexpr (PAIRX) {
#pragma unroll
    for (int p = 0; p < P; ++p) acc[p] = acc2[p].x + acc2[p].y;
  }
  if (LPV > 1) {
#pragma unroll
    for (int p = 0; p < P; ++p)
#pragma unroll
      for (int o = LPV / 2; o > 0; o >>= 1)
        acc[p] += __shfl_xor_sync(0xffffffffu, acc[p], o);
    if constexpr (MIX) {
#pragma unroll
      for (int q = 0; q < NQ; ++q)
#pragma unroll
        for (int o = LPV / 2; o > 0; o >>= 1)
          qw[q] += __shfl_xor_sync(0xffffffffu, qw[q], o);
    }
  }

  // ---- dependency protocol (programmatic dependent launch) --------------
  // Everything above read only this colour's own coefficients, the design
  // and the outcome bits, all final since this colour's previous launch.
  // The beta update needs Omega and the other colour's new coefficients,
  // written by the previous kernel in the stream: wait for its completion
  // here, and only then let the next kernel start its own latent phase.
  // (Without a programmatic launch both calls return at once.)
  cudaGridDependencySynchronize();
  cudaTriggerProgrammaticLaunchCompletion();
  const long long nk = *ch.nkept;
  for (int t = tid; t < P * P; t += blockDim.x) {
    Om[t] = ch.omega_f[t];
    Xtx[t] = d.xtx[t];
  }
  __syncthreads();
  const bool leader = active && k == 0;
  int err = ok ? 0 : kErrTnCap;
  float bnew[P];   // the voxel's coefficients at the end of the sweep
  float pv[NT];    // its Omega pair products (colour 1)
  double wmt = 0.0;  // its term of the beta_WM conditional mean
#pragma unroll
  for (int p = 0; p < P; ++p) bnew[p] = beta[p];
#pragma unroll
  for (int q = 0; q < NT; ++q) pv[q] = 0.f;

  if (leader) {
    // ---- beta_v | rest  (Spat_Coefff, covar.cpp:142-180) ---------------
    float sumV[P];
#pragma unroll
    for (int p = 0; p < P; ++p) sumV[p] = 0.f;
#pragma unroll
    for (int t = 1; t <= 6; ++t) {
      const int sn = d.nb[colour][(size_t)t * nc + j];
#pragma unroll
      for (int p = 0; p < P; ++p) sumV[p] += ch.beta[(size_t)p * Vp + sn];
    }
    const unsigned nbm = d.nbm[colour][j];
    const float nnb = (float)__popc(nbm);
    float b[P], Q[NT];
#pragma unroll
    for (int a = 0; a < P; ++a) {
      float s = acc[a];
#pragma unroll
      for (int q = 0; q < P; ++q) s += Om[q + a * P] * sumV[q];
      b[a] = s;
#pragma unroll
      for (int q = 0; q <= a; ++q)
        Q[tri(a, q)] = (MIX ? qw[tri(a, q) < NQ ? tri(a, q) : 0] : Xtx[q + a * P]) +
                       nnb * Om[q + a * P];
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
      for (int p = 0; p < P; ++p) {
        ch.beta[(size_t)p * Vp + sc] = out[p];
        bnew[p] = out[p];
      }
    }
    err |= (okc ? 0 : kErrChol) | ((okc && !fin) ? kErrNaN : 0);

    // ---- beta_WM | Z, beta (betaMGPU, covarGPU.cu:585-640): this voxel's
    // WM_v * sum_i (Z_iv - x_i' beta_v) with the new beta_v; with X c = 1,
    // sum_i (Z_iv - bwm) = c' acc.
    if constexpr (WMU) {
      double sz = 0.0, sxb = 0.0;
#pragma unroll
      for (int p = 0; p < P; ++p) {
        sz += (double)d.cvec[p] * (double)acc[p];
        sxb += (double)d.xsum[p] * (double)bnew[p];
      }
      wmt = (double)wmv * (sz + (double)d.N * (double)bwm - sxb);
    }

    // ---- posterior running sums of the kept sweep (mcmc.cpp:637-645) --
    if (kept) {
#pragma unroll
      for (int p = 0; p < P; ++p) {
        const double x = (double)bnew[p];
        ch.acc_sum[(size_t)p * d.V + v] += x;
        ch.acc_sq[(size_t)p * d.V + v] += x * x;
      }
#pragma unroll
      for (int g2 = 0; g2 < P; ++g2)
        if (g2 < d.S)
          ch.prb_sum[(size_t)g2 * d.V + v] +=
              (double)(MIX ? prob_logit(bnew[g2], ch.inv_lf) : prob_sdnorm(bnew[g2] + bwm));
    }

    // ---- Omega pair products (Spat_Coef_Prec, covarGPU.cu:953-1013) -----
    // Every in-mask edge joins a colour-0 and a colour-1 voxel, so the
    // colour-1 pass sees each edge once.  For a forward neighbour (+x, +y,
    // +z) the reference tests the neighbour's row coefficient; for a
    // backward one the edge is counted when that neighbour is in the mask
    // and this voxel's row coefficient is nonzero (covar.cpp:235-253).
    if (colour == 1) {
#pragma unroll
      for (int t = 0; t < 6; ++t) {
        const int sn = d.nb[1][(size_t)(t + 1) * nc + j];
        const bool fwd = t & 1;
        const bool nin = (nbm >> t) & 1u;
        float dd[P];
        bool ind[P];
#pragma unroll
        for (int p = 0; p < P; ++p) {
          const float bn = ch.beta[(size_t)p * Vp + sn];
          dd[p] = bnew[p] - bn;
          ind[p] = fwd ? (bn != 0.f) : (nin && bnew[p] != 0.f);
        }
#pragma unroll
        for (int r = 0; r < P; ++r)
          if (ind[r]) {
#pragma unroll
            for (int c2 = 0; c2 <= r; ++c2) pv[tri(r, c2)] += dd[r] * dd[c2];
          }
      }
    }
  } else {
#pragma unroll
    for (int p = 0; p < P; ++p) bnew[p] = 0.f;  // no column-sum share
  }
  if (err) {
    atomicOr(ch.status, err);
    atomicOr(ch.any_status, err);
  }

  // ---- block partials: column sums and the beta_WM term (both colours),
  // pairs (colour 1)
  __shared__ double red[kMaxThreads / 32][kFusedVals];
  __shared__ double tot[kFusedVals];
  __shared__ int is_last;
  const int lane = tid & 31, warp = tid >> 5, nwarp = blockDim.x >> 5;
  constexpr int kColOff = kMaxPairs;
  constexpr int NV = NT + P + (WMU ? 1 : 0);  // values reduced per block
  // The pair products and coefficients of a warp's 32 voxels are summed in
  // FP32 by a fixed shuffle tree (this part's FP64 pipe does two lanes per
  // clock per SM: an FP64 tree over all 24 resident warps took about 15 us
  // per colour-1 launch), then in FP64 across warps and blocks; the beta_WM
  // term stays FP64 throughout.
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    if (colour == 0 && q < NT) continue;
    double val;
    if (q < NT + P) {
      float f = q < NT ? pv[q] : bnew[q - NT];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) f += __shfl_xor_sync(0xffffffffu, f, o);
      val = (double)f;
    } else {
      val = wmt;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) val += __shfl_xor_sync(0xffffffffu, val, o);
    }
    if (lane == 0)
      red[warp][q < NT ? q : (q < NT + P ? kColOff + (q - NT) : kWmOff)] = val;
  }
  __syncthreads();
  const int vpb = blockDim.x / LPV;
  const int lb = bm.start / vpb;
  const int nblk = max(1, (nc + vpb - 1) / vpb);  // blocks of this colour
  // Sum of one value over the blocks' partials (value-major, so a warp
  // reads consecutive blocks) in a fixed order, so the draw is bitwise
  // reproducible: lane l loads the blocks l, l + 32, ... of a 512-block
  // chunk together and adds them as a tree, then the lanes are combined.
  auto rows = [&](const double *base, int nrow) -> double {
    double s = 0.0;
    for (int c0 = 0; c0 < nrow; c0 += 512) {
      double v[16];
#pragma unroll
      for (int u = 0; u < 16; ++u) {
        const int r = c0 + lane + 32 * u;
        v[u] = r < nrow ? __ldcg(base + r) : 0.0;
      }
#pragma unroll
      for (int w = 8; w > 0; w >>= 1)
#pragma unroll
        for (int u = 0; u < w; ++u) v[u] += v[u + w];
      s += v[0];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
  };
  if (colour == 0) {
    if (tid < P || (WMU && tid == kMaxP)) {
      const int q = tid < P ? kColOff + tid : kWmOff;
      double s = 0.0;
      for (int w = 0; w < nwarp; ++w) s += red[w][q];
      ch.partials0[(size_t)tid * ch.pstride0 + lb] = s;
      __threadfence();
    }
    __syncthreads();
    if (tid == 0) is_last = atomicAdd(ch.done, 1u) == (unsigned)(nblk - 1);
    __syncthreads();
    if (!is_last) return;
    // The last colour-0 block sums the column sums (and the beta_WM term)
    // over the colour's blocks while colour 1 starts, and advances this
    // colour's count.
    __threadfence();
    for (int m = warp; m < P + (WMU ? 1 : 0); m += nwarp) {
      const int q = m < P ? m : kMaxP;
      const double s = rows(ch.partials0 + (size_t)q * ch.pstride0, nblk);
      if (lane == 0) ch.tot0[q] = s;
    }
    // the sweep's Bartlett variates (they do not depend on S), for the
    // Omega draw at the end of colour 1
    if (!SUPP && warp == nwarp - 1) {
      const int e = __reduce_or_sync(0xffffffffu, wishart_draws(ch, d, sweep_ll, lane, ch.wdraw));
      if (e && lane == 0) {
        atomicOr(ch.status, e);
        atomicOr(ch.any_status, e);
      }
    }
    if (tid == 0) {
      ch.sweep[0] = sweep_ll + 1;
      ch.done[0] = 0u;
      __threadfence();
    }
    return;
  }
  if (tid < kFusedVals) {
    const bool live =
        tid < kMaxPairs ? tid < NT : ((WMU && tid == kWmOff) || (tid - kColOff) < P);
    if (live) {
      double s = 0.0;
      for (int w = 0; w < nwarp; ++w) s += red[w][tid];
      ch.partials1[(size_t)tid * ch.pstride1 + lb] = s;
      __threadfence();
    }
  }
  __syncthreads();
  if (tid == 0) {
    const unsigned prev = atomicAdd(ch.done + 1, 1u);
    is_last = prev == (unsigned)(nblk - 1);
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  // warp w takes the live values m = w, w + nwarp, ...; colour 0's totals
  // (final since that kernel completed) are added to the column sums
  for (int m = warp; m < NV; m += nwarp) {
    const int q = m < NT ? m : (m < NT + P ? kColOff + (m - NT) : kWmOff);
    double s = rows(ch.partials1 + (size_t)q * ch.pstride1, nblk);
    if (q >= kColOff) s += __ldcg(ch.tot0 + (q == kWmOff ? kMaxP : q - kColOff));
    if (lane == 0) tot[q] = s;
  }
  __syncthreads();
  if (warp == 0)
    wishart_warp(ch, d, tot, (long long)sweep_ll, kept, nk, SUPP ? 1 : 0, sup, lane);
}

// Launch of one instantiation; with pdl the launch carries the
// programmatic-stream-serialization attribute, so it may start once every
// block of the previous kernel in the stream has passed its dependency
// point.
template <int P, int LPV, bool SUPP, bool MIX = false, bool WMU = false, bool TC = false,
          bool WIDE = false>
cudaError_t launch_one(int nblocks, int threads, cudaStream_t st, bool pdl,
                       const DatasetDev *ds, ChainDev *ch, const BlockMap *map,
                       int colour, const Supplied &sup) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(nblocks);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = 0;
  // the design slices and Z tiles of the tensor-core X'Z (the opt-in above
  // the default 48 KB is made by prepare_tc, outside any stream capture)
  if constexpr (TC) cfg.dynamicSmemBytes = (size_t)tc_smem_bytes(P, threads);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, fused_colour_kernel<P, LPV, SUPP, MIX, WMU, TC, WIDE>, ds,
                            ch, map, colour, sup);
}

// The dynamic shared memory opt-in of one tensor-core instantiation.
template <int P>
cudaError_t prepare_tc() {
  return cudaFuncSetAttribute(fused_colour_kernel<P, 1, false, false, false, true>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              tc_smem_bytes(P, kMaxThreads));
}

// Instantiation helper used by bsg_fused_l*.cu.
template <int LPV>
cudaError_t launch_fused_lpv(int P, int threads, bool supplied,
                             const DatasetDev *ds, ChainDev *ch,
                             const BlockMap *map, int nblocks, int colour,
                             const Supplied &sup, cudaStream_t st, bool pdl) {
  if (nblocks <= 0) return cudaSuccess;
  cudaError_t e = cudaErrorInvalidValue;
#define BSG_CASE(PP)                                                        \
  case PP:                                                                  \
    if (supplied) {                                                         \
      if constexpr (LPV == 1)                                               \
        e = launch_one<PP, LPV, true>(nblocks, threads, st, pdl, ds, ch,    \
                                      map, colour, sup);                    \
    } else {                                                                \
      e = launch_one<PP, LPV, false>(nblocks, threads, st, pdl, ds, ch,     \
                                     map, colour, sup);                     \
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
  return e;
}

}  // namespace bsg
