// dg_indicator.cuh -- the arithmetic of the Hennemann-Gassner shock
// indicator (src/solvers/indicators.jl:7-42; Hennemann, Rueda-Ramirez,
// Hindenlang, Gassner, JCP 426 (2021)) used by the indicator kernel
// (dg_aux.cu): the indicator variable of a node, the modal energy sums of an
// element (sequential in FP64, the oracle's order; by a warp in FP32) and
// alpha from the sums.
#pragma once
#include "dg_convert.cuh"

namespace trixi {

__device__ __forceinline__ double ind_div(double a, double b) { return a / b; }
__device__ __forceinline__ float ind_div(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double ind_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float ind_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double ind_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float ind_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double ind_exp(double x) { return exp(x); }
__device__ __forceinline__ float ind_exp(float x) { return __expf(x); }

// The indicator variable of one node from its conservative values (already
// in the compute type R): rho * p (density_pressure) or p (pressure), with
// one reciprocal of rho.  Euler: DIM momenta then the energy; ideal GLM-MHD
// (mhd): three momenta, energy, B, and psi when nv == 9.
template <int DIM, typename R>
__device__ __forceinline__ R ind_value(const R *c, R gm1, bool mhd, int nv, int variable) {
  const R half = R(0.5);
  const R rho = c[0];
  const R inv = ind_div(R(1), rho);
  R kin = R(0), p;
  if (mhd) {  // p = (gamma-1)(E - rho|v|^2/2 - |B|^2/2 - psi^2/2)
    R mag = R(0);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const R m = c[1 + d], B = c[5 + d];
      kin += m * (m * inv);
      mag += B * B;
    }
    if (nv == 9) mag += c[8] * c[8];
    p = gm1 * (c[4] - half * kin - half * mag);
  } else {
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      const R m = c[1 + d];
      kin += m * (m * inv);
    }
    p = gm1 * (c[DIM + 1] - half * kin);
  }
  return variable ? p : rho * p;
}

// One of the three modal energy sums of an element from its Legendre
// coefficients c[NN] (node order): which = 0 all modes, 1 without the
// highest, 2 without the two highest (by the largest one-dimensional degree);
// a sequential fold in node order with uncontracted multiplies and adds.
template <int DIM, int N, typename R>
__device__ __forceinline__ R ind_energy_sum(const R *c, int which) {
  constexpr int NN = (DIM == 1) ? N : (DIM == 2 ? N * N : N * N * N);
  R sum = R(0);
  for (int n = 0; n < NN; ++n) {
    int maxc = n % N;
    if (DIM > 1) maxc = max(maxc, (n / N) % N);
    if (DIM > 2) maxc = max(maxc, n / (N * N));
    const bool take = (which == 0) || (which == 1 && maxc < N - 1) || (which == 2 && maxc < N - 2);
    if (take) sum = ind_add(sum, ind_mul(c[n], c[n]));  // no contraction: the oracle's roundings
  }
  return sum;
}

// The three modal energy sums of one element folded by one warp (the FP32
// indicator of the mixed-precision rhs): lane l accumulates nodes l, l + 32,
// ... in order, then a fixed xor-shuffle tree adds the lanes (IEEE addition
// commutes, so every lane ends with the same three sums; the result does not
// depend on the launch).  The FP64 indicator keeps the oracle's sequential
// fold (ind_energy_sum).
template <int DIM, int N>
__device__ __forceinline__ void ind_energy_sums_warp(const float *c, int lane, float &total, float &clip1,
                                                     float &clip2) {
  constexpr int NN = (DIM == 1) ? N : (DIM == 2 ? N * N : N * N * N);
  float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f;
  for (int n = lane; n < NN; n += 32) {
    int maxc = n % N;
    if (DIM > 1) maxc = max(maxc, (n / N) % N);
    if (DIM > 2) maxc = max(maxc, n / (N * N));
    const float q = __fmul_rn(c[n], c[n]);
    s0 = __fadd_rn(s0, q);
    if (maxc < N - 1) s1 = __fadd_rn(s1, q);
    if (maxc < N - 2) s2 = __fadd_rn(s2, q);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    s0 = __fadd_rn(s0, __shfl_xor_sync(0xffffffffu, s0, off));
    s1 = __fadd_rn(s1, __shfl_xor_sync(0xffffffffu, s1, off));
    s2 = __fadd_rn(s2, __shfl_xor_sync(0xffffffffu, s2, off));
  }
  total = s0;
  clip1 = s1;
  clip2 = s2;
}

// alpha_raw from the three energy sums: the larger relative energy of the
// highest and second-highest modes, the logistic function around the
// threshold, alpha_min / 1 - alpha_min cut-offs and the alpha_max cap
// (src/solvers/indicators.jl:22-38).
template <typename R>
__device__ __forceinline__ double ind_alpha(R total, R clip1, R clip2, double threshold_, double param_s_,
                                            double amax, double amin) {
  const R f1 = (total != R(0)) ? (total - clip1) / total : R(0);
  const R f2 = (clip1 != R(0)) ? (clip1 - clip2) / clip1 : R(0);
  const R energy = f1 > f2 ? f1 : f2;
  const R threshold = R(threshold_);
  double al = double(R(1) / (R(1) + ind_exp(-R(param_s_) / threshold * (energy - threshold))));
  if (al < amin) al = 0.0;
  if (al > 1.0 - amin) al = 1.0;
  return fmin(amax, al);
}

}  // namespace trixi
