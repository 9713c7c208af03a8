// dg_adjoint.cu -- instantiation of the adjoint kernels and the density
// objective used by the adjoint solve.
#include <algorithm>

#include "dg_adjoint.cuh"
#include "dg_adjoint.h"

namespace trixi {

bool adjoint_supported(int dim, int N, int eq, int vol, int vflux, int sflux, bool has_mortars) {
  if (has_mortars || dim < 1 || dim > 3 || N < 2 || N > HOST_NMAX) return false;
  auto smooth_flux = [](int f) { return f == FLUX_RANOCHA || f == FLUX_CENTRAL; };
  if (eq == EQ_ADV) {
    // surface fluxes whose cotangents Adjoint<DIM, EQ_ADV>::two_point_vjp forms:
    // the upwind family (LLF, HLL) and the central average (central, ranocha)
    const bool sflux_ok = sflux == FLUX_LLF || sflux == FLUX_LLF_NAIVE || sflux == FLUX_HLL ||
                          sflux == FLUX_CENTRAL || sflux == FLUX_RANOCHA;
    return sflux_ok && (vol == VOL_WEAK || (vol == VOL_FD && vflux == FLUX_CENTRAL));
  }
  return vol == VOL_FD && smooth_flux(vflux) && smooth_flux(sflux);
}

namespace {

template <int DIM, int N, int EQ, int VOL>
cudaError_t launch_t(const AdjointHost &a, cudaStream_t s) {
  using K = AdjointKernel<DIM, N, EQ, VOL>;
  AdjointParams p;
  p.u = a.u;
  p.lu_in = a.lu_in;
  p.lk_in = a.lk_in;
  p.lu_out = a.lu_out;
  p.lk_out = a.lk_out;
  p.face_table = a.face_table;
  p.inv_jac = a.inv_jac;
  p.nelements = a.nelements;
  p.surface_flux = a.surface_flux;
  p.volume_flux = a.volume_flux;
  p.rk_a = a.rk_a;
  p.rk_b = a.rk_b;
  p.dt = a.dt;
  p.pp.gamma = a.gamma;
  p.pp.gm1 = a.gamma - 1.0;
  p.pp.inv_gm1 = 1.0 / (a.gamma - 1.0);
  for (int d = 0; d < 3; ++d) p.pp.a[d] = a.adv[d];
  for (int i = 0; i < NMAXT * NMAXT; ++i) {
    p.dsplit[i] = i < N * N ? a.dsplit[i] : 0.0;
    p.dhat[i] = i < N * N ? a.dhat[i] : 0.0;
  }
  p.lhat_l = a.lhat_l;
  p.lhat_r = a.lhat_r;
  const size_t smem = K::smem_for(K::EPB);
  static const cudaError_t attr = cudaFuncSetAttribute(dg_adjoint_kernel<DIM, N, EQ, VOL>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  if (attr != cudaSuccess) return attr;
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  const int64_t grid = (a.nelements + K::EPB - 1) / K::EPB;
  if (grid <= 0) return cudaSuccess;
  p.pdl = a.pdl;
  p.u_ready = a.u_ready;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(K::BLOCK);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr_pdl[1];
  attr_pdl[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr_pdl[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr_pdl;
  cfg.numAttrs = a.pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, dg_adjoint_kernel<DIM, N, EQ, VOL>, p);
}

template <int DIM, int N>
cudaError_t launch_n(const AdjointHost &a, cudaStream_t s) {
  if (a.eq == EQ_ADV) return a.vol == VOL_WEAK ? launch_t<DIM, N, EQ_ADV, VOL_WEAK>(a, s) : launch_t<DIM, N, EQ_ADV, VOL_FD>(a, s);
  return launch_t<DIM, N, EQ_EULER, VOL_FD>(a, s);
}

template <int DIM>
cudaError_t launch_dim(const AdjointHost &a, cudaStream_t s) {
  switch (a.N) {
    case 2: return launch_n<DIM, 2>(a, s);
    case 3: return launch_n<DIM, 3>(a, s);
    case 4: return launch_n<DIM, 4>(a, s);
    case 5: return launch_n<DIM, 5>(a, s);
    case 6: return launch_n<DIM, 6>(a, s);
  }
  return cudaErrorNotSupported;
}

__global__ void density_objective_kernel(int dim, int N, int nv, int64_t E, const double *__restrict__ u,
                                         const double *__restrict__ rho_t, const double *__restrict__ inv_jac,
                                         const double *__restrict__ w, double *__restrict__ ubar,
                                         double *__restrict__ partial) {
  const int64_t e = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (e >= E) return;
  int NN = N;
  for (int d = 1; d < dim; ++d) NN *= N;
  double J = 1.0;
  for (int d = 0; d < dim; ++d) J /= inv_jac[e];
  double acc = 0.0;
  for (int n = lane; n < NN; n += 32) {
    int r = n;
    double wt = 1.0;
    for (int d = 0; d < dim; ++d) {
      wt *= w[r % N];
      r /= N;
    }
    const int64_t g = (e * NN + n) * nv;
    const double diff = u[g] - rho_t[e * NN + n];
    acc += 0.5 * wt * J * diff * diff;
    if (ubar) {
      ubar[g] = wt * J * diff;
      for (int v = 1; v < nv; ++v) ubar[g + v] = 0.0;
    }
  }
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if (lane == 0) partial[e] = acc;
}

__global__ void sum_kernel(int64_t n, const double *__restrict__ x, double *__restrict__ out) {
  __shared__ double sm[1024];
  double v = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) v += x[i];
  sm[threadIdx.x] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sm[threadIdx.x] += sm[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sm[0];
}

}  // namespace

cudaError_t launch_adjoint(const AdjointHost &a, cudaStream_t s) {
  switch (a.dim) {
    case 1: return launch_dim<1>(a, s);
    case 2: return launch_dim<2>(a, s);
    case 3: return launch_dim<3>(a, s);
  }
  return cudaErrorNotSupported;
}

cudaError_t launch_density_objective(int dim, int N, int nv, int64_t E, const double *u, const double *rho_target,
                                     const double *inv_jac, const double *w, double *ubar, double *partial,
                                     double *out, cudaStream_t s) {
  const int per_block = 8;
  density_objective_kernel<<<(unsigned)((E + per_block - 1) / per_block), 32 * per_block, 0, s>>>(
      dim, N, nv, E, u, rho_target, inv_jac, w, ubar, partial);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  sum_kernel<<<1, 1024, 0, s>>>(E, partial, out);
  return cudaGetLastError();
}

}  // namespace trixi
