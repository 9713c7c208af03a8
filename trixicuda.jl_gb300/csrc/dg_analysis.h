// dg_analysis.h -- host interface of the analysis / initial-condition kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "dg_consts.h"

namespace trixi {

constexpr int IC_CONSTANT = 0;          // TRIXI_IC_CONSTANT
constexpr int IC_CONVERGENCE_TEST = 1;  // TRIXI_IC_CONVERGENCE_TEST
constexpr int IC_WEAK_BLAST_WAVE = 2;   // TRIXI_IC_WEAK_BLAST_WAVE
constexpr int IC_EOC_EULER_GRAVITY = 3; // TRIXI_IC_EOC_TEST_COUPLED_EULER_GRAVITY
constexpr int IC_LAST = IC_EOC_EULER_GRAVITY;

struct IcParams {
  double p[9];       // kind-specific parameters (a constant state: nvars values)
  double a[3];       // advection velocity
  double gamma;
  double xa[16];     // analysis nodes on [-1, 1] (error norms)
};

struct MaxDtHost {
  int dim = 2, eq = 1, N = 0;
  int64_t E = 0;
  const double *u = nullptr, *inv_jac = nullptr;
  double gamma = 1.4, a[3] = {0, 0, 0};
  unsigned long long *acc = nullptr;
  double *dt = nullptr;
};

struct IntegrateHost {
  int dim = 2, eq = 1, N = 0, which = 0, nq = 1;
  int64_t E = 0;
  const double *u = nullptr, *du = nullptr, *inv_jac = nullptr, *w = nullptr;
  double gamma = 1.4;
  double *partial = nullptr;  // [E][nq]
  double *out = nullptr;      // [nq] device
};

struct IcHost {
  int dim = 2, eq = 1, N = 0, kind = 0;
  int64_t E = 0;
  const double *coords = nullptr;
  IcParams ip{};
  double t = 0;
  double *u = nullptr;
};

struct ErrorNormHost {
  int dim = 2, eq = 1, N = 0, NA = 0, nv = 1, kind = 0;
  int64_t E = 0;
  const double *u = nullptr, *uref = nullptr, *coords = nullptr;
  IcParams ip{};
  double t = 0;
  const double *vdm = nullptr, *wa = nullptr, *inv_jac = nullptr;
  double *l2p = nullptr, *linfp = nullptr;   // [E][nv]
  double *l2_out = nullptr, *linf_out = nullptr;  // [nv] device
};

cudaError_t launch_max_dt(const MaxDtHost &h, cudaStream_t s);
cudaError_t launch_integrate(const IntegrateHost &h, cudaStream_t s);
cudaError_t launch_initial_condition(const IcHost &h, cudaStream_t s);
cudaError_t launch_error_norms_all(const ErrorNormHost &h, cudaStream_t s);

}  // namespace trixi
