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

namespace trixi {

__host__ __device__ constexpr int ipow(int b, int e) { return e == 0 ? 1 : b * ipow(b, e - 1); }

template <int DIM, int EQ>
struct NVarsOf {
  static constexpr int value = (EQ == EQ_ADV) ? 1 : DIM + 2;
};

template <typename R>
struct PhysParams {
  R gamma, gm1, inv_gm1;  // gamma, gamma-1, 1/(gamma-1)
  R a[3];                 // advection velocity
};

__device__ __forceinline__ double dev_log(double x) { return log(x); }
__device__ __forceinline__ float dev_log(float x) { return logf(x); }
__device__ __forceinline__ double dev_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float dev_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double dev_fabs(double x) { return fabs(x); }
__device__ __forceinline__ float dev_fabs(float x) { return fabsf(x); }
__device__ __forceinline__ double dev_fmax(double x, double y) { return fmax(x, y); }
__device__ __forceinline__ float dev_fmax(float x, float y) { return fmaxf(x, y); }

// Ismail-Roe logarithmic mean (x - y)/(log x - log y) with the series
// 1/(1 + u/3 + u^2/5 + u^3/7) in u = ((x-y)/(x+y))^2 below 1e-4.
template <typename R>
__device__ __forceinline__ R ln_mean(R x, R y) {
  const R f2 = (x * (x - R(2) * y) + y * y) / (x * (x + R(2) * y) + y * y);
  if (f2 < R(1.0e-4)) return (x + y) * R(52.5) / (R(105) + f2 * (R(35) + f2 * (R(21) + f2 * R(15))));
  return (y - x) / dev_log(y / x);
}

template <typename R>
__device__ __forceinline__ R inv_ln_mean(R x, R y) {
  const R f2 = (x * (x - R(2) * y) + y * y) / (x * (x + R(2) * y) + y * y);
  if (f2 < R(1.0e-4)) return (R(105) + f2 * (R(35) + f2 * (R(21) + f2 * R(15)))) / (R(52.5) * (x + y));
  return dev_log(y / x) / (y - x);
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
};

template <int DIM, typename R>
struct Physics<DIM, EQ_EULER, R> {
  static constexpr int NV = DIM + 2;
  __device__ __forceinline__ static void prim(const R *u, R *w, const PhysParams<R> &pp) {
    const R rho = u[0];
    R kin = R(0);
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      w[1 + d] = u[1 + d] / rho;
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
    const R rho_mean = ln_mean(rl, rr);
    const R inv_rho_p_mean = pl * pr * inv_ln_mean(rl * pr, rr * pl);
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
    const R cl = dev_sqrt(pp.gamma * wl[DIM + 1] / wl[0]);
    const R cr = dev_sqrt(pp.gamma * wr[DIM + 1] / wr[0]);
    if (naive) return dev_fmax(dev_fabs(wl[1 + O]), dev_fabs(wr[1 + O])) + dev_fmax(cl, cr);
    return dev_fmax(dev_fabs(wl[1 + O]) + cl, dev_fabs(wr[1 + O]) + cr);
  }
};

// Two-point flux dispatch (kind is warp-uniform).
template <int DIM, int EQ, typename R, int O>
__device__ __forceinline__ void two_point_flux(int kind, const R *ul, const R *wl, const R *ur, const R *wr, R *f,
                                               const PhysParams<R> &pp) {
  using P = Physics<DIM, EQ, R>;
  if (kind == FLUX_RANOCHA) {
    P::template ranocha<O>(ul, wl, ur, wr, f, pp);
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
  if constexpr (KIND == FLUX_RANOCHA) {
    P::template ranocha<O>(ul, wl, ur, wr, f, pp);
  } else if constexpr (KIND == FLUX_CENTRAL) {
    P::template central<O>(ul, wl, ur, wr, f, pp);
  } else {
    two_point_flux<DIM, EQ, R, O>(KIND, ul, wl, ur, wr, f, pp);
  }
}

}  // namespace trixi
