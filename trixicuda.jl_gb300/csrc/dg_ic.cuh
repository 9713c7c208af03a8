// dg_ic.cuh -- the built-in initial conditions (also the Dirichlet boundary
// functions of non-periodic meshes) and the source term of the Euler
// convergence test, evaluated pointwise on the device in FP64.
#pragma once
#include "dg_analysis.h"
#include "dg_physics.cuh"

namespace trixi {

constexpr int SRC_NONE = 0;              // TRIXI_SOURCE_NONE
constexpr int SRC_CONVERGENCE_TEST = 1;  // TRIXI_SOURCE_CONVERGENCE_TEST
constexpr int SRC_EOC_EULER = 2;         // TRIXI_SOURCE_EOC_TEST_EULER

// The manufactured solution of the Euler-gravity convergence test
// (Schlottke-Lakemper, Winters, Ranocha, Gassner, "A purely hyperbolic
// discretization of the Poisson equation for self-gravitating flows", JCP 442
// (2021)): rho = c + A sin(pi (sum_d x_d - t)) with c = 2, A = 0.1, v_d = 1.
// Its gravitational potential solves lap phi = 4 pi G (rho - c):
// phi = -4 G A sin(.) / (ndims pi), so grad p = -rho grad phi holds with
// p = K rho^2, K = 2 G / (ndims pi), G = 1.
template <int DIM>
struct EocEulerGravity {
  static constexpr double c = 2.0, A = 0.1, pi = 3.14159265358979323846;
  static constexpr double K = 2.0 / (DIM * pi);
  __device__ __forceinline__ static void phase(const double *x, double t, double &sn, double &cs) {
    double s = 0.0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) s += x[d];
    sincos(pi * (s - t), &sn, &cs);
  }
};

// Ideal GLM-MHD: the convergence tests are the smooth circularly polarised
// Alfven waves -- 1D and 2D after Derigs et al., JCP 317 (2016) (rho = 1,
// p = 0.1, amplitude 0.1, unit background field along the propagation
// direction: the x axis in 1D, alpha = pi/4 in 2D; speed 1), 3D after
// Altmann's thesis (2012) (propagation along (1, 0, 2)/sqrt 5 on [-1, 1]^3,
// amplitude 0.2, p = 1); the weak blast wave is the Euler one in a uniform
// field B = (1, 1, 1).  psi = 0 (2D/3D).
template <int DIM>
__device__ void eval_ic_mhd(int kind, const double *x, double t, const IcParams &ip, double *u) {
  constexpr int NV = (DIM == 1) ? 8 : 9;
  if (kind == IC_CONSTANT) {
    for (int v = 0; v < NV; ++v) u[v] = ip.p[v];
    return;
  }
  double rho, v[3] = {0.0, 0.0, 0.0}, p, B[3];
  const double pi = 3.14159265358979323846;
  if (kind == IC_CONVERGENCE_TEST) {
    rho = 1.0;
    if (DIM == 1) {
      double sn, cs;
      sincos(2.0 * pi * (x[0] + t), &sn, &cs);
      v[1] = 0.1 * sn;
      v[2] = 0.1 * cs;
      p = 0.1;
      B[0] = 1.0;
      B[1] = v[1];
      B[2] = v[2];
    } else if (DIM == 2) {
      const double alpha = 0.25 * pi;
      const double ca = cos(alpha), sa = sin(alpha);
      const double x_perp = x[0] * ca + x[1] * sa;
      double sn, cs;
      sincos(2.0 * pi * (x_perp + t), &sn, &cs);
      const double b_perp = 0.1 * sn;
      v[0] = -b_perp * sa;
      v[1] = b_perp * ca;
      v[2] = 0.1 * cs;
      p = 0.1;
      B[0] = ca + v[0];
      B[1] = sa + v[1];
      B[2] = v[2];
    } else {
      const double omega = 2.0 * pi, r = 2.0, e = 0.2;
      const double nx = 1.0 / sqrt(r * r + 1.0), ny = r / sqrt(r * r + 1.0);
      const double va = omega / ny;
      const double ph = omega / ny * (nx * (x[0] - 0.5 * r) + ny * (x[2] - 0.5 * r)) - va * t;
      double sn, cs;
      sincos(ph, &sn, &cs);
      v[0] = -e * ny * cs;
      v[1] = e * sn;
      v[2] = e * nx * cs;
      p = 1.0;
      B[0] = nx - v[0];
      B[1] = -v[1];
      B[2] = ny - v[2];
    }
  } else {  // weak blast wave in B = (1, 1, 1)
    double r2 = 0.0;
    for (int d = 0; d < DIM; ++d) r2 += x[d] * x[d];
    const double rr = sqrt(r2);
    const bool out = rr > 0.5;
    rho = out ? 1.0 : 1.1691;
    p = out ? 1.0 : 1.245;
    if (!out) {
      if (DIM == 1) {
        v[0] = 0.1882 * (x[0] > 0 ? 1.0 : (x[0] < 0 ? -1.0 : 0.0));
      } else if (DIM == 2) {
        const double phi = atan2(x[1], x[0]);
        v[0] = 0.1882 * cos(phi);
        v[1] = 0.1882 * sin(phi);
      } else {
        const double phi = atan2(x[1], x[0]);
        const double theta = (rr == 0.0) ? 0.0 : acos(fmin(1.0, fmax(-1.0, x[2] / rr)));
        v[0] = 0.1882 * cos(phi) * sin(theta);
        v[1] = 0.1882 * sin(phi) * sin(theta);
        v[2] = 0.1882 * cos(theta);
      }
    }
    B[0] = B[1] = B[2] = 1.0;
  }
  u[0] = rho;
  double kin = 0.0, mag = 0.0;
  for (int d = 0; d < 3; ++d) {
    u[1 + d] = rho * v[d];
    kin += v[d] * v[d];
    mag += B[d] * B[d];
    u[5 + d] = B[d];
  }
  u[4] = p / (ip.gamma - 1.0) + 0.5 * rho * kin + 0.5 * mag;
  if (NV == 9) u[NV - 1] = 0.0;
}

template <int DIM, int EQ>
__device__ void eval_ic(int kind, const double *x, double t, const IcParams &ip, double *u) {
  constexpr int NV = NVarsOf<DIM, EQ>::value;
  if constexpr (EQ == EQ_MHD) {
    eval_ic_mhd<DIM>(kind, x, t, ip, u);
    return;
  }
  if (kind == IC_CONSTANT) {
    for (int v = 0; v < NV; ++v) u[v] = ip.p[v];
    return;
  }
  if (kind == IC_CONVERGENCE_TEST) {
    const double c = ip.p[0], A = ip.p[1], L = ip.p[2];
    const double omega = 2.0 * 3.14159265358979323846 / L;
    if (EQ == EQ_ADV) {
      double s = 0.0;
      for (int d = 0; d < DIM; ++d) s += x[d] - ip.a[d] * t;
      u[0] = c + A * sin(omega * s);
    } else {
      double s = 0.0;
      for (int d = 0; d < DIM; ++d) s += x[d];
      const double ini = c + A * sin(omega * (s - t));
      u[0] = ini;
      for (int d = 0; d < DIM; ++d) u[1 + d] = ini;
      u[DIM + 1] = ini * ini;
    }
    return;
  }
  if (kind == IC_EOC_EULER_GRAVITY) {
    using M = EocEulerGravity<DIM>;
    double sn, cs;
    M::phase(x, t, sn, cs);
    const double rho = M::c + M::A * sn;
    u[0] = rho;
    for (int d = 0; d < DIM; ++d) u[1 + d] = rho;
    u[DIM + 1] = M::K * rho * rho / (ip.gamma - 1.0) + 0.5 * DIM * rho;
    return;
  }
  // IC_WEAK_BLAST_WAVE (Euler): inside r <= 0.5 rho 1.1691, radial v 0.1882, p 1.245
  double r2 = 0.0;
  for (int d = 0; d < DIM; ++d) r2 += x[d] * x[d];
  const double r = sqrt(r2);
  const bool out = r > 0.5;
  const double rho = out ? 1.0 : 1.1691, p = out ? 1.0 : 1.245;
  double v[3] = {0.0, 0.0, 0.0};
  if (!out) {
    if (DIM == 1) {
      v[0] = 0.1882 * (x[0] > 0 ? 1.0 : (x[0] < 0 ? -1.0 : 0.0));
    } else if (DIM == 2) {
      const double phi = atan2(x[1], x[0]);
      v[0] = 0.1882 * cos(phi);
      v[1] = 0.1882 * sin(phi);
    } else {
      const double phi = atan2(x[1], x[0]);
      const double theta = (r == 0.0) ? 0.0 : acos(fmin(1.0, fmax(-1.0, x[2] / r)));
      v[0] = 0.1882 * cos(phi) * sin(theta);
      v[1] = 0.1882 * sin(phi) * sin(theta);
      v[2] = 0.1882 * cos(theta);
    }
  }
  double kin = 0.0;
  u[0] = rho;
  for (int d = 0; d < DIM; ++d) {
    u[1 + d] = rho * v[d];
    kin += v[d] * v[d];
  }
  u[DIM + 1] = p / (ip.gamma - 1.0) + 0.5 * rho * kin;
}


// Source term of the Euler convergence test: S = du/dt + div F(u) for the
// manufactured solution rho = rho v_d = c + A sin(omega (sum_d x_d - t)),
// E = rho^2 (derived symbolically; rho_x = omega A cos(omega (sum_d x_d - t)),
// g = gamma):
//   1D: (0, rho_x (g-1)(4 rho - 1)/2, same)
//   2D: (rho_x, rho_x (2 g rho - g - 2 rho + 2) [x2], 2 rho_x (2 g rho - g - rho + 1))
//   3D: (2 rho_x, rho_x (4 g rho - 3 g - 4 rho + 7)/2 [x3], rho_x (12 g rho - 9 g - 4 rho + 9)/2)
// prm = (c, A, L).  Linear advection has none (its convergence test is exact).
// kind SRC_EOC_EULER: S = du/dt + div F(u) for the Euler-gravity manufactured
// solution above (derived symbolically; rx = pi A cos(pi (sum_d x_d - t)),
// K = 2/(ndims pi), g = gamma): the gravity terms -rho grad phi, -rho v.grad phi
// that the Euler equations lack, plus the mass and momentum left over in 2D/3D:
//   mass      (ndims - 1) rx
//   momentum  rx ((ndims - 1) + 2 K rho)                     [each component]
//   energy    rx ((ndims - 1)(2 K rho/(g - 1) + ndims/2) + 2 ndims K rho)
template <int DIM, int EQ>
__device__ __forceinline__ void source_convergence(const double *prm, double g, const double *x, double t,
                                                   double *s, int kind = SRC_CONVERGENCE_TEST) {
  if constexpr (EQ == EQ_EULER) {
    if (kind == SRC_EOC_EULER) {
      using M = EocEulerGravity<DIM>;
      double sn, cs;
      M::phase(x, t, sn, cs);
      const double rho = M::c + M::A * sn, rx = M::pi * M::A * cs;
      const double kr2 = 2.0 * M::K * rho;
      s[0] = (DIM - 1) * rx;
#pragma unroll
      for (int d = 0; d < DIM; ++d) s[1 + d] = rx * ((DIM - 1) + kr2);
      s[DIM + 1] = rx * ((DIM - 1) * (kr2 / (g - 1.0) + 0.5 * DIM) + DIM * kr2);
      return;
    }
  }
  if constexpr (EQ == EQ_EULER) {
    const double omega = 2.0 * 3.14159265358979323846 / prm[2];
    double sx = 0.0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) sx += x[d];
    double sn, cs;
    sincos(omega * (sx - t), &sn, &cs);
    const double rho = prm[0] + prm[1] * sn, rx = omega * prm[1] * cs;
    if constexpr (DIM == 1) {
      s[0] = 0.0;
      s[1] = s[2] = 0.5 * rx * (g - 1.0) * (4.0 * rho - 1.0);
    } else if constexpr (DIM == 2) {
      s[0] = rx;
      s[1] = s[2] = rx * (2.0 * g * rho - g - 2.0 * rho + 2.0);
      s[3] = 2.0 * rx * (2.0 * g * rho - g - rho + 1.0);
    } else {
      s[0] = 2.0 * rx;
      s[1] = s[2] = s[3] = 0.5 * rx * (4.0 * g * rho - 3.0 * g - 4.0 * rho + 7.0);
      s[4] = 0.5 * rx * (12.0 * g * rho - 9.0 * g - 4.0 * rho + 9.0);
    }
  } else {
    s[0] = 0.0;
  }
}

}  // namespace trixi
