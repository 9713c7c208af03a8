// dg_packed.cuh -- two FP32 two-point flux evaluations per instruction
// stream, in the halves of float2 registers, on Blackwell's packed FP32
// instructions (FFMA2 / FADD2 / FMUL2: one instruction issues two FP32
// operations).  The FP32 flux-differencing kernels are bound by instruction
// issue, and the owner thread of a node evaluates N-1 fluxes per direction
// (its line partners); packing two of them halves the issue slots of their
// arithmetic.
//
// ranocha_x2<DIM, OA, OB>: flux_ranocha of the compressible Euler equations
// (Ranocha 2020, Ismail-Roe logarithmic means) between one owner state and
// two partner states, the first along direction OA, the second along OB.
// Same formulas, series and thresholds as Physics<DIM, EQ_EULER, float>::
// ranocha with ranocha_means (dg_physics.cuh); the rounding may differ from
// the scalar form by the placement of fused multiply-adds.
#pragma once
#include "dg_physics.cuh"

namespace trixi {
namespace pk {

__device__ __forceinline__ float2 bc(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 mk(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// a - b as a fused multiply-add (b * -1 is exact, one rounding)
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, bc(-1.0f), a); }

}  // namespace pk

// Both means of flux_ranocha for two state pairs: mean1 = ln_mean(x1, y1),
// inv_mean2 = 1 / ln_mean(x2, y2), per half; one reciprocal of
// (x1 + y1)(x2 + y2) per half, the series below the FP32 threshold and the
// logarithms only when a lane of the warp needs one.
__device__ __forceinline__ void ranocha_means_x2(float2 x1, float2 y1, float2 x2, float2 y2, float2 &mean1,
                                                 float2 &inv_mean2) {
  using namespace pk;
  const float2 s1 = add2(x1, y1), d1 = sub2(x1, y1), s2 = add2(x2, y2), d2 = sub2(x2, y2);
  const float2 ss = mul2(s1, s2);
  const float2 q = mk(__fdividef(1.0f, ss.x), __fdividef(1.0f, ss.y));
  const float2 r1 = mul2(s2, q), r2 = mul2(s1, q);
  const float2 f1 = mul2(d1, r1), f2 = mul2(d2, r2);
  const float2 u1 = mul2(f1, f1), u2 = mul2(f2, f2);
  // h(u) = 1/g(u) = 1 - u/3 - 4u^2/45 - 44u^3/945 and g(u) = 1 + u/3 + u^2/5 + u^3/7 (Horner)
  float2 h = fma2(u1, bc(float(-44.0 / 945.0)), bc(float(-4.0 / 45.0)));
  h = fma2(u1, h, bc(float(-1.0 / 3.0)));
  h = fma2(u1, h, bc(1.0f));
  float2 g = fma2(u2, bc(float(1.0 / 7.0)), bc(float(1.0 / 5.0)));
  g = fma2(u2, g, bc(float(1.0 / 3.0)));
  g = fma2(u2, g, bc(1.0f));
  mean1 = mul2(mul2(bc(0.5f), s1), h);
  inv_mean2 = mul2(mul2(bc(2.0f), r2), g);
  constexpr float thr = LnMeanThreshold<float>::value;
  const bool s1x = u1.x < thr, s1y = u1.y < thr, s2x = u2.x < thr, s2y = u2.y < thr;
  if (__any_sync(__activemask(), !(s1x && s1y && s2x && s2y))) {
    if (!s1x) mean1.x = __fdividef(d1.x, __logf(__fdividef(x1.x, y1.x)));
    if (!s1y) mean1.y = __fdividef(d1.y, __logf(__fdividef(x1.y, y1.y)));
    if (!s2x) inv_mean2.x = __fdividef(__logf(__fdividef(x2.x, y2.x)), d2.x);
    if (!s2y) inv_mean2.y = __fdividef(__logf(__fdividef(x2.y, y2.y)), d2.y);
  }
}

// f[v] (two halves) = flux_ranocha(w_own, w_a) along OA | flux_ranocha(w_own, w_b)
// along OB; w are primitive records (rho, v_1..v_DIM, p).
template <int DIM, int OA, int OB>
__device__ __forceinline__ void ranocha_x2(const float *wl, const float *wa, const float *wb, float2 *f,
                                           const PhysParams<float> &pp) {
  using namespace pk;
  const float2 rl = bc(wl[0]), pl = bc(wl[DIM + 1]);
  const float2 rr = mk(wa[0], wb[0]), pr = mk(wa[DIM + 1], wb[DIM + 1]);
  float2 rho_mean, inv_mean;
  ranocha_means_x2(rl, rr, mul2(rl, pr), mul2(rr, pl), rho_mean, inv_mean);
  const float2 inv_rho_p_mean = mul2(mul2(pl, pr), inv_mean);
  float2 vavg[DIM];
  float2 v2 = bc(0.0f);
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    const float2 vl = bc(wl[1 + d]), vr = mk(wa[1 + d], wb[1 + d]);
    vavg[d] = mul2(bc(0.5f), add2(vl, vr));
    v2 = fma2(vl, vr, v2);
  }
  const float2 v2avg = mul2(bc(0.5f), v2);
  const float2 pavg = mul2(bc(0.5f), add2(pl, pr));
  // the normal direction of each half
  const float2 vn = mk(vavg[OA].x, vavg[OB].y);
  const float2 vrn = mk(wa[1 + OA], wb[1 + OB]), vln = mk(wl[1 + OA], wl[1 + OB]);
  const float2 f0 = mul2(rho_mean, vn);
  f[0] = f0;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    const float2 pd = mk(d == OA ? pavg.x : 0.0f, d == OB ? pavg.y : 0.0f);
    f[1 + d] = fma2(f0, vavg[d], pd);
  }
  const float2 e_in = fma2(inv_rho_p_mean, bc(pp.inv_gm1), v2avg);
  const float2 work = mul2(bc(0.5f), fma2(pl, vrn, mul2(pr, vln)));
  f[DIM + 1] = fma2(f0, e_in, work);
}

}  // namespace trixi
