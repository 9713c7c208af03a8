// dg_physics.cuh -- equations and two-point fluxes for the DGSEM kernels.
//
// Device versions of the Trixi.jl physics the reference kernels call through
// `flux`, `volume_flux` and `surface_flux` (src/solvers/dg_2d_kernel.jl:18-19,
// 200-205, 947):
//   LinearScalarAdvectionEquation{1,2,3}D, CompressibleEulerEquations{1,2,3}D,
//   flux (physical), flux_ranocha, flux_central, flux_lax_friedrichs.
// The formulas are restated from the published methods: Ranocha (2020)
// EC/KEP flux with Ismail-Roe (2009) logarithmic means; Rusanov/LLF with the
// Davis wave-speed estimate (or the "naive" max(|v|)+max(c) variant).
//
// Orientation O is a template parameter so that every state array is
// indexed with compile-time constants (states stay in registers).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "dg_consts.h"
#include "dg_convert.cuh"

namespace trixi {

__host__ __device__ constexpr int ipow(int b, int e) { return e == 0 ? 1 : b * ipow(b, e - 1); }

template <int DIM, int EQ>
struct NVarsOf {
  static constexpr int value = (EQ == EQ_ADV) ? 1 : (EQ == EQ_MHD) ? (DIM == 1 ? 8 : 9) : DIM + 2;
};

template <typename R>
struct PhysParams {
  R gamma, gm1, inv_gm1;  // gamma, gamma-1, 1/(gamma-1)
  R a[3];                 // advection velocity
  R c_h;                  // GLM cleaning speed (ideal GLM-MHD)
};

// Precision-specific elementary operations.  FP64 keeps the library log and
// sqrt and divides through rcp_newton (below); the FP32 path of the
// mixed-precision kernels uses the fast hardware approximations (__fdividef:
// 2 ulp; __logf: absolute error ~2^-21 near 1), well inside its error budget
// (the rhs in FP32 is accurate to ~1e-6 relative).
__device__ __forceinline__ double dev_log(double x) { return log(x); }
__device__ __forceinline__ float dev_log(float x) { return __logf(x); }
// FP64 reciprocal by Newton-Raphson refinement r <- r + r (1 - x r) of the
// FP32 hardware approximation (relative error 2^-22 -> 2^-44 -> ~1 ulp of
// FP64 after the second step); the conversions run on the integer pipe, so
// the FP64 pipe -- the bound of the FP64 kernels -- sees 4 FMAs instead of an
// IEEE division.  Divisors are nonzero and within the float range (densities,
// pressures, their sums and differences, logarithms of their ratios).
__device__ __forceinline__ double rcp_newton(double x) {
  const float rf = __fdividef(1.0f, d2f_rn(x));
  double r = f2d_exact(rf);
  double e = fma(-x, r, 1.0);
  r = fma(r, e, r);
  e = fma(-x, r, 1.0);
  return fma(r, e, r);
}
__device__ __forceinline__ double dev_div(double a, double b) { return a * rcp_newton(b); }
__device__ __forceinline__ float dev_div(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double dev_rcp(double x) { return rcp_newton(x); }
__device__ __forceinline__ float dev_rcp(float x) { return __fdividef(1.0f, x); }
__device__ __forceinline__ double dev_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float dev_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double dev_fabs(double x) { return fabs(x); }
__device__ __forceinline__ float dev_fabs(float x) { return fabsf(x); }
__device__ __forceinline__ double dev_fmax(double x, double y) { return fmax(x, y); }
__device__ __forceinline__ float dev_fmax(float x, float y) { return fmaxf(x, y); }

// Ismail-Roe logarithmic mean (x - y)/(log x - log y) and its inverse.
// With s = x + y, f = (x - y)/s and u = f^2, ln_mean = (s/2) / g(u) where
// g(u) = artanh(f)/f = sum_k u^k/(2k+1) (Ismail & Roe 2009).  Below the
// threshold the series are used: h(u) = 1/g(u) = 1 - u/3 - 4u^2/45 - 44u^3/945
// + O(u^4) (the reversion of g) for the mean and g(u) for the inverse, so each
// mean costs one reciprocal of s; above it, log(x/y) is evaluated.  The
// threshold is 1e-4 in FP64 (truncation ~3e-18) and 1e-2 in FP32 (truncation
// ~3e-10, and log(x/y) is only formed for ratios above ~1.2, where FP32
// cancellation is harmless).  The adjoint differentiates the same branches.
template <typename R>
struct LnMeanThreshold;
template <>
struct LnMeanThreshold<double> {
  static constexpr double value = 1.0e-4;
};
template <>
struct LnMeanThreshold<float> {
  static constexpr float value = 1.0e-2f;
};

// h(u) = 1/g(u) and g(u) through u^3 (Horner), and their derivatives in u
template <typename R>
__device__ __forceinline__ R series_h(R u) {
  return R(1) + u * (R(-1.0 / 3.0) + u * (R(-4.0 / 45.0) + u * R(-44.0 / 945.0)));
}
template <typename R>
__device__ __forceinline__ R series_g(R u) {
  return R(1) + u * (R(1.0 / 3.0) + u * (R(1.0 / 5.0) + u * R(1.0 / 7.0)));
}
__device__ __forceinline__ double series_h_du(double u) {
  return -1.0 / 3.0 + u * (-8.0 / 45.0 + u * (-132.0 / 945.0));
}
__device__ __forceinline__ double series_g_du(double u) { return 1.0 / 3.0 + u * (2.0 / 5.0 + u * (3.0 / 7.0)); }

template <typename R>
__device__ __forceinline__ R ln_mean_series(R s, R u) {
  return R(0.5) * s * series_h(u);
}
template <typename R>
__device__ __forceinline__ R inv_ln_mean_series(R r, R u) {
  return R(2) * r * series_g(u);
}

template <typename R>
__device__ __forceinline__ R ln_mean(R x, R y) {
  const R s = x + y, d = x - y;
  const R r = dev_rcp(s);
  const R f = d * r;
  const R u = f * f;
  if (u < LnMeanThreshold<R>::value) return ln_mean_series(s, u);
  return dev_div(d, dev_log(dev_div(x, y)));
}

template <typename R>
__device__ __forceinline__ R inv_ln_mean(R x, R y) {
  const R s = x + y, d = x - y;
  const R r = dev_rcp(s);
  const R f = d * r;
  const R u = f * f;
  if (u < LnMeanThreshold<R>::value) return inv_ln_mean_series(r, u);
  return dev_div(dev_log(dev_div(x, y)), d);
}

// Both means of flux_ranocha, ln_mean(x1, y1) and inv_ln_mean(x2, y2), from a
// single reciprocal 1/((x1+y1)(x2+y2)).
template <typename R>
__device__ __forceinline__ void ranocha_means(R x1, R y1, R x2, R y2, R &mean1, R &inv_mean2) {
  const R s1 = x1 + y1, d1 = x1 - y1, s2 = x2 + y2, d2 = x2 - y2;
  const R q = dev_rcp(s1 * s2);
  const R r1 = s2 * q, r2 = s1 * q;
  const R f1 = d1 * r1, f2 = d2 * r2;
  const R u1 = f1 * f1, u2 = f2 * f2;
  const bool series1 = u1 < LnMeanThreshold<R>::value, series2 = u2 < LnMeanThreshold<R>::value;
  mean1 = ln_mean_series(s1, u1);
  inv_mean2 = inv_ln_mean_series(r2, u2);
  // the logarithmic forms only when a lane of the warp needs one (smooth
  // states stay on the series; each lane's result is the same either way)
  if (__any_sync(__activemask(), !(series1 && series2))) {
    if (!series1) mean1 = dev_div(d1, dev_log(dev_div(x1, y1)));
    if (!series2) inv_mean2 = dev_div(dev_log(dev_div(x2, y2)), d2);
  }
}

// Physics of one equation system.  States: `u` conservative, `w` primitive
// (rho, v_1..v_DIM, p) for Euler; for advection w == u.
template <int DIM, int EQ, typename R>
struct Physics;

template <int DIM, typename R>
struct Physics<DIM, EQ_ADV, R> {
  static constexpr int NV = 1;
  __device__ __forceinline__ static void prim(const R *u, R *w, const PhysParams<R> &) { w[0] = u[0]; }
  __device__ __forceinline__ static void cons_from_prim(const R *w, R *u, const PhysParams<R> &) { u[0] = w[0]; }
  template <int O>
  __device__ __forceinline__ static void flux(const R *u, const R *, R *f, const PhysParams<R> &pp) {
    f[0] = pp.a[O] * u[0];
  }
  template <int O>
  __device__ __forceinline__ static void ranocha(const R *ul, const R *, const R *ur, const R *, R *f,
                                                 const PhysParams<R> &pp) {
    f[0] = R(0.5) * (pp.a[O] * ul[0] + pp.a[O] * ur[0]);
  }
  template <int O>
  __device__ __forceinline__ static void central(const R *ul, const R *, const R *ur, const R *, R *f,
                                                 const PhysParams<R> &pp) {
    f[0] = R(0.5) * (pp.a[O] * ul[0] + pp.a[O] * ur[0]);
  }
  template <int O>
  __device__ __forceinline__ static R max_speed(const R *, const R *, const R *, const R *, bool,
                                                const PhysParams<R> &pp) {
    return dev_fabs(pp.a[O]);
  }
  template <int O>
  __device__ __forceinline__ static void min_max_speed(const R *, const R *, R &lmin, R &lmax,
                                                       const PhysParams<R> &pp) {
    lmin = pp.a[O];
    lmax = pp.a[O];
  }
  // (flux_hlle is refused for linear advection on the host)
  template <int O>
  __device__ __forceinline__ static void min_max_speed_einfeldt(const R *, const R *wl, const R *, const R *wr,
                                                                R &lmin, R &lmax, const PhysParams<R> &pp) {
    min_max_speed<O>(wl, wr, lmin, lmax, pp);
  }
};

template <int DIM, typename R>
struct Physics<DIM, EQ_EULER, R> {
  static constexpr int NV = DIM + 2;
  __device__ __forceinline__ static void prim(const R *u, R *w, const PhysParams<R> &pp) {
    const R rho = u[0];
    const R inv_rho = dev_rcp(rho);
    R kin = R(0);
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      w[1 + d] = u[1 + d] * inv_rho;
      kin += u[1 + d] * w[1 + d];
    }
    w[0] = rho;
    w[DIM + 1] = pp.gm1 * (u[DIM + 1] - R(0.5) * kin);
  }
  __device__ __forceinline__ static void cons_from_prim(const R *w, R *u, const PhysParams<R> &pp) {
    R kin = R(0);
    u[0] = w[0];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      u[1 + d] = w[0] * w[1 + d];
      kin += u[1 + d] * w[1 + d];
    }
    u[DIM + 1] = w[DIM + 1] * pp.inv_gm1 + R(0.5) * kin;
  }
  // physical flux f_O(u)
  template <int O>
  __device__ __forceinline__ static void flux(const R *u, const R *w, R *f, const PhysParams<R> &) {
    const R p = w[DIM + 1];
    f[0] = u[1 + O];
#pragma unroll
    for (int d = 0; d < DIM; ++d) f[1 + d] = u[1 + O] * w[1 + d] + (d == O ? p : R(0));
    f[DIM + 1] = (u[DIM + 1] + p) * w[1 + O];
  }
  // Ranocha (2020) entropy-conserving / kinetic-energy-preserving flux.
  template <int O>
  __device__ __forceinline__ static void ranocha(const R *, const R *wl, const R *, const R *wr, R *f,
                                                 const PhysParams<R> &pp) {
    const R rl = wl[0], rr = wr[0], pl = wl[DIM + 1], pr = wr[DIM + 1];
    R rho_mean, inv_mean;
    ranocha_means(rl, rr, rl * pr, rr * pl, rho_mean, inv_mean);
    const R inv_rho_p_mean = pl * pr * inv_mean;
    R vavg[DIM];
    R v2avg = R(0);
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      vavg[d] = R(0.5) * (wl[1 + d] + wr[1 + d]);
      v2avg += wl[1 + d] * wr[1 + d];
    }
    v2avg *= R(0.5);
    const R pavg = R(0.5) * (pl + pr);
    const R f0 = rho_mean * vavg[O];
    f[0] = f0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) f[1 + d] = f0 * vavg[d] + (d == O ? pavg : R(0));
    f[DIM + 1] = f0 * (v2avg + inv_rho_p_mean * pp.inv_gm1) + R(0.5) * (pl * wr[1 + O] + pr * wl[1 + O]);
  }
  // Shima, Kuya, Tamaki, Kawai (2021), "Preventing spurious pressure
  // oscillations in split convective form discretization for compressible
  // flows", JCP 427: the kinetic-energy and pressure-equilibrium preserving
  // flux (arithmetic means; product mean of the kinetic energy; internal
  // energy {{p}}{{v}}/(gamma-1); pressure work (p_l v_r + p_r v_l)/2).
  template <int O>
  __device__ __forceinline__ static void shima(const R *, const R *wl, const R *, const R *wr, R *f,
                                               const PhysParams<R> &pp) {
    const R rho_avg = R(0.5) * (wl[0] + wr[0]);
    const R pl = wl[DIM + 1], pr = wr[DIM + 1];
    const R p_avg = R(0.5) * (pl + pr);
    R vavg[DIM];
    R kin = R(0);
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      vavg[d] = R(0.5) * (wl[1 + d] + wr[1 + d]);
      kin += wl[1 + d] * wr[1 + d];
    }
    kin *= R(0.5);
    const R f0 = rho_avg * vavg[O];
    f[0] = f0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) f[1 + d] = f0 * vavg[d] + (d == O ? p_avg : R(0));
    f[DIM + 1] = p_avg * vavg[O] * pp.inv_gm1 + f0 * kin + R(0.5) * (pl * wr[1 + O] + pr * wl[1 + O]);
  }
  template <int O>
  __device__ __forceinline__ static void central(const R *ul, const R *wl, const R *ur, const R *wr, R *f,
                                                 const PhysParams<R> &pp) {
    R fl[NV], fr[NV];
    flux<O>(ul, wl, fl, pp);
    flux<O>(ur, wr, fr, pp);
#pragma unroll
    for (int v = 0; v < NV; ++v) f[v] = R(0.5) * (fl[v] + fr[v]);
  }
  template <int O>
  __device__ __forceinline__ static R max_speed(const R *, const R *wl, const R *, const R *wr, bool naive,
                                                const PhysParams<R> &pp) {
    const R cl = dev_sqrt(dev_div(pp.gamma * wl[DIM + 1], wl[0]));
    const R cr = dev_sqrt(dev_div(pp.gamma * wr[DIM + 1], wr[0]));
    if (naive) return dev_fmax(dev_fabs(wl[1 + O]), dev_fabs(wr[1 + O])) + dev_fmax(cl, cr);
    return dev_fmax(dev_fabs(wl[1 + O]) + cl, dev_fabs(wr[1 + O]) + cr);
  }
  // naive signal-speed estimates of HLL: min(v_l - c_l, v_r - c_r), max(v_l + c_l, v_r + c_r)
  template <int O>
  __device__ __forceinline__ static void min_max_speed(const R *wl, const R *wr, R &lmin, R &lmax,
                                                       const PhysParams<R> &pp) {
    const R cl = dev_sqrt(dev_div(pp.gamma * wl[DIM + 1], wl[0]));
    const R cr = dev_sqrt(dev_div(pp.gamma * wr[DIM + 1], wr[0]));
    lmin = fminf_(wl[1 + O] - cl, wr[1 + O] - cr);
    lmax = dev_fmax(wl[1 + O] + cl, wr[1 + O] + cr);
  }
  // Einfeldt's signal speeds (Einfeldt, Munz, Roe, Sjogreen, JCP 92 (1991)):
  // Roe averages with sqrt(rho) weights, v~ and H~ = (E + p)/rho averaged,
  // c~^2 = (gamma - 1)(H~ - |v~|^2/2); the states' sound speeds scaled by
  // beta = sqrt((gamma - 1)/(2 gamma)); both bounds enclose zero:
  // lmin = min(v~_O - c~, v_l,O - beta c_l, 0), lmax = max(v~_O + c~, v_r,O + beta c_r, 0)
  template <int O>
  __device__ __forceinline__ static void min_max_speed_einfeldt(const R *ul, const R *wl, const R *ur, const R *wr,
                                                                R &lmin, R &lmax, const PhysParams<R> &pp) {
    const R sl = dev_sqrt(wl[0]), sr = dev_sqrt(wr[0]);
    const R inv = dev_rcp(sl + sr);
    const R hl = dev_div(ul[DIM + 1] + wl[DIM + 1], wl[0]), hr = dev_div(ur[DIM + 1] + wr[DIM + 1], wr[0]);
    R v2 = R(0), vo = R(0);
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      const R vd = (sl * wl[1 + d] + sr * wr[1 + d]) * inv;
      v2 += vd * vd;
      if (d == O) vo = vd;
    }
    const R h = (sl * hl + sr * hr) * inv;
    const R c = dev_sqrt(pp.gm1 * (h - R(0.5) * v2));
    const R beta = dev_sqrt(dev_div(R(0.5) * pp.gm1, pp.gamma));
    const R cl = dev_sqrt(dev_div(pp.gamma * wl[DIM + 1], wl[0]));
    const R cr = dev_sqrt(dev_div(pp.gamma * wr[DIM + 1], wr[0]));
    lmin = fminf_(fminf_(vo - c, wl[1 + O] - beta * cl), R(0));
    lmax = dev_fmax(dev_fmax(vo + c, wr[1 + O] + beta * cr), R(0));
  }
  __device__ __forceinline__ static R fminf_(R a, R b) { return a < b ? a : b; }
};

// Ideal GLM-MHD (IdealGlmMhdEquations{1,2,3}D).  Conservative variables
// (rho, rho v1, rho v2, rho v3, E, B1, B2, B3[, psi]), primitive record
// (rho, v1, v2, v3, p, B1, B2, B3[, psi]); three velocity and field
// components in every dimension, psi (and the nonconservative terms) in 2D and
// 3D only.  GLM formulation of Derigs, Winters, Gassner, Walch, Bohm, JCP 364
// (2018): E = p/(gamma-1) + rho|v|^2/2 + |B|^2/2 + psi^2/2; the conservative
// flux carries the cleaning terms c_h psi and c_h B_O; v . grad psi and the
// Powell source are the nonconservative terms.
template <int DIM, typename R>
struct Physics<DIM, EQ_MHD, R> {
  static constexpr int NV = (DIM == 1) ? 8 : 9;
  static constexpr bool PSI = (DIM > 1);
  __device__ __forceinline__ static void prim(const R *u, R *w, const PhysParams<R> &pp) {
    const R rho = u[0];
    const R inv_rho = dev_rcp(rho);
    R kin = R(0), mag = R(0);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      w[1 + d] = u[1 + d] * inv_rho;
      kin += u[1 + d] * w[1 + d];
      mag += u[5 + d] * u[5 + d];
      w[5 + d] = u[5 + d];
    }
    R e = u[4] - R(0.5) * kin - R(0.5) * mag;
    if constexpr (PSI) {
      e -= R(0.5) * u[8] * u[8];
      w[8] = u[8];
    }
    w[0] = rho;
    w[4] = pp.gm1 * e;
  }
  __device__ __forceinline__ static void cons_from_prim(const R *w, R *u, const PhysParams<R> &pp) {
    R kin = R(0), mag = R(0);
    u[0] = w[0];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      u[1 + d] = w[0] * w[1 + d];
      kin += u[1 + d] * w[1 + d];
      mag += w[5 + d] * w[5 + d];
      u[5 + d] = w[5 + d];
    }
    R e = w[4] * pp.inv_gm1 + R(0.5) * kin + R(0.5) * mag;
    if constexpr (PSI) {
      e += R(0.5) * w[8] * w[8];
      u[8] = w[8];
    }
    u[4] = e;
  }
  template <int O>
  __device__ __forceinline__ static void flux(const R *u, const R *w, R *f, const PhysParams<R> &pp) {
    const R p = w[4];
    const R mag = R(0.5) * (w[5] * w[5] + w[6] * w[6] + w[7] * w[7]);
    const R vB = w[1] * w[5] + w[2] * w[6] + w[3] * w[7];
    const R kin = R(0.5) * (u[1] * w[1] + u[2] * w[2] + u[3] * w[3]);
    const R BO = w[5 + O];
    f[0] = u[1 + O];
#pragma unroll
    for (int d = 0; d < 3; ++d) f[1 + d] = u[1 + O] * w[1 + d] - BO * w[5 + d] + (d == O ? p + mag : R(0));
    R fe = (kin + pp.gamma * pp.inv_gm1 * p + R(2) * mag) * w[1 + O] - BO * vB;
    if constexpr (PSI) fe += pp.c_h * w[8] * BO;
    f[4] = fe;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      if (d == O) f[5 + d] = PSI ? pp.c_h * w[8] : R(0);
      else f[5 + d] = w[1 + O] * w[5 + d] - w[1 + d] * BO;
    }
    if constexpr (PSI) f[8] = pp.c_h * BO;
  }
  // Hindenlang & Gassner (2019), "A new entropy conservative two-point flux
  // for ideal MHD equations derived from first principles" (HONOM 2019):
  // Ismail-Roe logarithmic means of rho and rho/p, arithmetic means of v, p,
  // psi, product means of the magnetic terms; the energy flux follows from the
  // entropy-conservation condition with the nonconservative Powell term.
  template <int O>
  __device__ __forceinline__ static void hindenlang_gassner(const R *, const R *wl, const R *, const R *wr, R *f,
                                                            const PhysParams<R> &pp) {
    const R rl = wl[0], rr = wr[0], pl = wl[4], pr = wr[4];
    R rho_mean, inv_mean;
    ranocha_means(rl, rr, rl * pr, rr * pl, rho_mean, inv_mean);
    const R inv_rho_p_mean = pl * pr * inv_mean;
    R vavg[3];
    R v2avg = R(0), b2avg = R(0);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      vavg[d] = R(0.5) * (wl[1 + d] + wr[1 + d]);
      v2avg += wl[1 + d] * wr[1 + d];
      b2avg += wl[5 + d] * wr[5 + d];
    }
    v2avg *= R(0.5);
    b2avg *= R(0.5);
    const R pavg = R(0.5) * (pl + pr);
    const R BOl = wl[5 + O], BOr = wr[5 + O];
    const R f0 = rho_mean * vavg[O];
    f[0] = f0;
#pragma unroll
    for (int d = 0; d < 3; ++d)
      f[1 + d] = f0 * vavg[d] + (d == O ? pavg + b2avg : R(0)) - R(0.5) * (BOl * wr[5 + d] + BOr * wl[5 + d]);
    const R vOl = wl[1 + O], vOr = wr[1 + O];
    R e = pl * vOr + pr * vOl;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      if (d == O) continue;
      e += (vOl + vOr) * wl[5 + d] * wr[5 + d];
      e -= wl[1 + d] * BOl * wr[5 + d] + wr[1 + d] * BOr * wl[5 + d];
      f[5 + d] = R(0.5) * (vOl * wl[5 + d] - wl[1 + d] * BOl + vOr * wr[5 + d] - wr[1 + d] * BOr);
    }
    if constexpr (PSI) {
      e += pp.c_h * (BOl * wr[8] + BOr * wl[8]);
      f[5 + O] = pp.c_h * R(0.5) * (wl[8] + wr[8]);
      f[8] = pp.c_h * R(0.5) * (BOl + BOr);
    } else {
      f[5 + O] = R(0);
    }
    f[4] = f0 * (v2avg + inv_rho_p_mean * pp.inv_gm1) + R(0.5) * e;
  }
  template <int O>
  __device__ __forceinline__ static void ec(const R *ul, const R *wl, const R *ur, const R *wr, R *f,
                                            const PhysParams<R> &pp) {
    hindenlang_gassner<O>(ul, wl, ur, wr, f, pp);
  }
  template <int O>
  __device__ __forceinline__ static void central(const R *ul, const R *wl, const R *ur, const R *wr, R *f,
                                                 const PhysParams<R> &pp) {
    R fl[NV], fr[NV];
    flux<O>(ul, wl, fl, pp);
    flux<O>(ur, wr, fr, pp);
#pragma unroll
    for (int v = 0; v < NV; ++v) f[v] = R(0.5) * (fl[v] + fr[v]);
  }
  // fast magnetosonic speed along O:
  // c_f^2 = (a^2 + b^2)/2 + sqrt((a^2 + b^2)^2 - 4 a^2 b_O^2)/2, a^2 = gamma p/rho, b = B/sqrt(rho)
  template <int O>
  __device__ __forceinline__ static R fast_speed(const R *w, const PhysParams<R> &pp) {
    const R inv_rho = dev_rcp(w[0]);
    const R a2 = pp.gamma * w[4] * inv_rho;
    const R b2 = (w[5] * w[5] + w[6] * w[6] + w[7] * w[7]) * inv_rho;
    const R bo2 = w[5 + O] * w[5 + O] * inv_rho;
    const R s = a2 + b2;
    return dev_sqrt(R(0.5) * (s + dev_sqrt(s * s - R(4) * a2 * bo2)));
  }
  template <int O>
  __device__ __forceinline__ static void min_max_speed(const R *wl, const R *wr, R &lmin, R &lmax,
                                                       const PhysParams<R> &pp) {
    const R cl = fast_speed<O>(wl, pp), cr = fast_speed<O>(wr, pp);
    const R a = wl[1 + O] - cl, b = wr[1 + O] - cr;
    lmin = a < b ? a : b;
    lmax = dev_fmax(wl[1 + O] + cl, wr[1 + O] + cr);
  }
  // Einfeldt's signal speeds with the Roe-type average of Cargo and Gallice
  // (JCP 136 (1997)): sqrt(rho) weights for v and H = (E + p + |B|^2/2)/rho,
  // crossed weights for B; rho^ = sqrt(rho_l rho_r),
  // X = |B_l - B_r|^2 / (2 (sqrt(rho_l) + sqrt(rho_r))^2) (their eq. 4.12),
  // b^2 = |B~|^2/rho^, a^2 = (2 - gamma) X + (gamma - 1)(H~ - |v~|^2/2 - b^2),
  // c_f~^2 = (a^2 + b^2 + sqrt((a^2 + b^2)^2 - 4 a^2 B~_O^2/rho^))/2;
  // lmin = min(v_l,O - c_f,l, v~_O - c_f~), lmax = max(v_r,O + c_f,r, v~_O + c_f~)
  template <int O>
  __device__ __forceinline__ static void min_max_speed_einfeldt(const R *ul, const R *wl, const R *ur, const R *wr,
                                                                R &lmin, R &lmax, const PhysParams<R> &pp) {
    const R sl = dev_sqrt(wl[0]), sr = dev_sqrt(wr[0]);
    const R inv = dev_rcp(sl + sr), inv_prod = dev_rcp(sl * sr);
    const R ql = sl * inv, qr = sr * inv;
    const R ml = wl[5] * wl[5] + wl[6] * wl[6] + wl[7] * wl[7];
    const R mr = wr[5] * wr[5] + wr[6] * wr[6] + wr[7] * wr[7];
    const R hl = dev_div(ul[4] + wl[4] + R(0.5) * ml, wl[0]), hr = dev_div(ur[4] + wr[4] + R(0.5) * mr, wr[0]);
    R v2 = R(0), b2 = R(0), x = R(0), vo = R(0), bo = R(0);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const R vd = wl[1 + d] * ql + wr[1 + d] * qr;
      const R bd = wl[5 + d] * qr + wr[5 + d] * ql;
      const R db = wl[5 + d] - wr[5 + d];
      v2 += vd * vd;
      b2 += bd * bd;
      x += db * db;
      if (d == O) { vo = vd; bo = bd; }
    }
    x *= R(0.5) * inv * inv;
    b2 *= inv_prod;
    const R h = hl * ql + hr * qr;
    const R a2 = (R(2) - pp.gamma) * x + pp.gm1 * (h - R(0.5) * v2 - b2);
    const R s = a2 + b2;
    const R cf = dev_sqrt(R(0.5) * (s + dev_sqrt(s * s - R(4) * a2 * bo * bo * inv_prod)));
    const R cl = fast_speed<O>(wl, pp), cr = fast_speed<O>(wr, pp);
    const R a = wl[1 + O] - cl, b = vo - cf;
    lmin = a < b ? a : b;
    lmax = dev_fmax(wr[1 + O] + cr, vo + cf);
  }
  template <int O>
  __device__ __forceinline__ static R max_speed(const R *, const R *wl, const R *, const R *wr, bool naive,
                                                const PhysParams<R> &pp) {
    const R cl = fast_speed<O>(wl, pp), cr = fast_speed<O>(wr, pp);
    if (naive) return dev_fmax(dev_fabs(wl[1 + O]), dev_fabs(wr[1 + O])) + dev_fmax(cl, cr);
    return dev_fmax(dev_fabs(wl[1 + O]) + cl, dev_fabs(wr[1 + O]) + cr);
  }
  // f += s * Phi_O(u_own, u_other): the Powell term phi_P(own) B_O(other) and
  // the GLM transport term v_O(own) phi_GLM(own) psi(other), phi_P = (0, B,
  // v.B, v, 0), phi_GLM = (0, 0, 0, 0, psi, 0, 0, 0, 1) (Derigs et al. 2018;
  // Bohm et al., JCP 422 (2020)).  2D/3D only.
  template <int O>
  __device__ __forceinline__ static void add_noncons(const R *wown, const R *wother, R s, R *f) {
    if constexpr (PSI) {
      const R b = s * wother[5 + O], q = s * wother[8];
      const R vB = wown[1] * wown[5] + wown[2] * wown[6] + wown[3] * wown[7];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        f[1 + d] += wown[5 + d] * b;
        f[5 + d] += wown[1 + d] * b;
      }
      f[4] += vB * b + wown[1 + O] * wown[8] * q;
      f[8] += wown[1 + O] * q;
    }
  }
};

// The entropy-conservative two-point flux of each system: flux_ranocha for
// Euler, the central flux for linear advection, flux_hindenlang_gassner for
// ideal GLM-MHD (the same kernel path serves FLUX_RANOCHA and FLUX_HG).
template <int DIM, int EQ, typename R, int O>
__device__ __forceinline__ void ec_flux(const R *ul, const R *wl, const R *ur, const R *wr, R *f,
                                        const PhysParams<R> &pp) {
  using P = Physics<DIM, EQ, R>;
  if constexpr (EQ == EQ_MHD) P::template ec<O>(ul, wl, ur, wr, f, pp);
  else P::template ranocha<O>(ul, wl, ur, wr, f, pp);
}

// HLL (Harten, Lax, van Leer 1983) with the naive signal-speed estimates
// (flux_hll) or Einfeldt's (flux_hlle):
// f_l when lmin >= 0, f_r when lmax <= 0, else
// (lmax f_l - lmin f_r + lmin lmax (u_r - u_l)) / (lmax - lmin).
template <int DIM, int EQ, typename R, int O>
__device__ __forceinline__ void hll_flux(const R *ul, const R *wl, const R *ur, const R *wr, R *f,
                                         const PhysParams<R> &pp, bool einfeldt = false) {
  using P = Physics<DIM, EQ, R>;
  R lmin, lmax;
  if (einfeldt) P::template min_max_speed_einfeldt<O>(ul, wl, ur, wr, lmin, lmax, pp);
  else P::template min_max_speed<O>(wl, wr, lmin, lmax, pp);
  R fl[P::NV], fr[P::NV];
  P::template flux<O>(ul, wl, fl, pp);
  P::template flux<O>(ur, wr, fr, pp);
  if (lmin >= R(0)) {
#pragma unroll
    for (int v = 0; v < P::NV; ++v) f[v] = fl[v];
  } else if (lmax <= R(0)) {
#pragma unroll
    for (int v = 0; v < P::NV; ++v) f[v] = fr[v];
  } else {
    const R inv = dev_rcp(lmax - lmin);
#pragma unroll
    for (int v = 0; v < P::NV; ++v) f[v] = (lmax * fl[v] - lmin * fr[v] + lmin * lmax * (ur[v] - ul[v])) * inv;
  }
}

// Two-point flux dispatch (kind is warp-uniform).  HLL = 0 leaves the HLL
// family (flux_hll, flux_hlle) out: the periodic fused kernels are built
// without it, and the host sends those problems to the instantiations with
// boundary support, which carry it.  Inlined at the kernels' many
// runtime-dispatched call sites, flux_hlle alone slowed the 3D
// shock-capturing kernel by 6 % (out of line, behind a call: 3 %).
template <int DIM, int EQ, typename R, int O, int HLL = 1, int EC = 1>
__device__ __forceinline__ void two_point_flux(int kind, const R *ul, const R *wl, const R *ur, const R *wr, R *f,
                                               const PhysParams<R> &pp) {
  using P = Physics<DIM, EQ, R>;
  if (EC && (kind == FLUX_RANOCHA || kind == FLUX_HG)) {
    ec_flux<DIM, EQ, R, O>(ul, wl, ur, wr, f, pp);
  } else if (HLL && (kind == FLUX_HLL || kind == FLUX_HLLE)) {
    hll_flux<DIM, EQ, R, O>(ul, wl, ur, wr, f, pp, kind == FLUX_HLLE);
  } else if (kind == FLUX_CENTRAL) {
    P::template central<O>(ul, wl, ur, wr, f, pp);
  } else {
    P::template central<O>(ul, wl, ur, wr, f, pp);
    const R lam = P::template max_speed<O>(ul, wl, ur, wr, kind == FLUX_LLF_NAIVE, pp);
#pragma unroll
    for (int v = 0; v < P::NV; ++v) f[v] += -R(0.5) * lam * (ur[v] - ul[v]);
  }
}

// Two-point flux with the kind fixed at compile time (volume fluxes).
template <int DIM, int EQ, typename R, int O, int KIND>
__device__ __forceinline__ void two_point_flux_t(const R *ul, const R *wl, const R *ur, const R *wr, R *f,
                                                 const PhysParams<R> &pp) {
  using P = Physics<DIM, EQ, R>;
  if constexpr (KIND == FLUX_RANOCHA || KIND == FLUX_HG) {
    ec_flux<DIM, EQ, R, O>(ul, wl, ur, wr, f, pp);
  } else if constexpr (KIND == FLUX_SHIMA && EQ == EQ_EULER) {
    P::template shima<O>(ul, wl, ur, wr, f, pp);
  } else if constexpr (KIND == FLUX_CENTRAL) {
    P::template central<O>(ul, wl, ur, wr, f, pp);
  } else {
    two_point_flux<DIM, EQ, R, O>(KIND, ul, wl, ur, wr, f, pp);
  }
}

}  // namespace trixi
