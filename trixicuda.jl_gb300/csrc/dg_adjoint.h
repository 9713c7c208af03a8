// dg_adjoint.h -- host interface of the adjoint kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "dg_host.h"

namespace trixi {

struct AdjointHost {
  int dim = 2, N = 0, eq = 1, vol = 1;
  const double *u = nullptr, *lu_in = nullptr, *lk_in = nullptr;
  double *lu_out = nullptr, *lk_out = nullptr;
  const int32_t *face_table = nullptr;
  const double *inv_jac = nullptr;
  int64_t nelements = 0;
  int surface_flux = 1, volume_flux = 1;
  double rk_a = 0, rk_b = 0, dt = 1;
  double gamma = 1.4, adv[3] = {0, 0, 0};
  double dsplit[HOST_NMAX * HOST_NMAX] = {};
  double dhat[HOST_NMAX * HOST_NMAX] = {};
  double lhat_l = 0, lhat_r = 0;
  int pdl = 0;      // programmatic dependent launch after the previous stage kernel
  int u_ready = 0;  // u was written before the previous kernel started (read before the wait)
};

bool adjoint_supported(int dim, int N, int eq, int vol, int vflux, int sflux, bool has_mortars);
cudaError_t launch_adjoint(const AdjointHost &a, cudaStream_t s);

// J = 1/2 sum_e J_e sum_nodes w (rho - rho_target)^2; ubar = dJ/du (device)
cudaError_t launch_density_objective(int dim, int N, int nv, int64_t E, const double *u, const double *rho_target,
                                     const double *inv_jac, const double *w, double *ubar, double *partial,
                                     double *out, cudaStream_t s);

}  // namespace trixi
