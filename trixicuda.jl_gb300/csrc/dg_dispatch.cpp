// dg_dispatch.cpp -- selects the compiled fused-kernel instantiation.
#include "dg_host.h"

namespace trixi {

bool fused_supported(int dim, int N, int eq, int vol, int vflux) {
  if (dim < 1 || dim > 3 || N < 2 || N > HOST_NMAX) return false;
  if (eq == 0) return vol == 0 || (vol == 1 && vflux == 2);  // advection: weak form, central flux differencing
  if (eq == 2) {  // ideal GLM-MHD: polydeg <= 4; FD with flux_hindenlang_gassner / flux_central, SC with the former
    if (N > 5) return false;
    return (vol == 1 && (vflux == 4 || vflux == 2)) || (vol == 2 && vflux == 4);
  }
  if (vflux == 4) return false;  // flux_hindenlang_gassner is the MHD flux
  if (vol == 0) return true;
  if (vol == 1 || vol == 2) return vflux == 1 || vflux == 2 || vflux == 5;  // flux_ranocha, flux_central, flux_shima_etal
  return false;
}

cudaError_t launch_fused(int dim, int N, int eq, int vol, int vflux, bool mixed, const FusedHost &h,
                         cudaStream_t s) {
  if (!fused_supported(dim, N, eq, vol, vflux)) return cudaErrorNotSupported;
  // the HLL family (flux_hll, flux_hlle) is compiled into the instantiations
  // with boundary support (they run periodic meshes as well) and into the
  // flux_shima_etal ones, not into the other periodic kernels
  // (the FV flux counts for shock capturing only)
  const bool fv_hll = vol == 2 && (h.fv_flux == FLUX_HLL || h.fv_flux == FLUX_HLLE);
  const bool hll = (h.surface_flux == FLUX_HLL || h.surface_flux == FLUX_HLLE || fv_hll) && vflux != FLUX_SHIMA;
  // ... and the entropy-conservative surface / FV flux of shock capturing
  // is left out of the periodic Euler and advection shock-capturing kernels
  const bool ec_sc = vol == 2 && eq != 2 && vflux != FLUX_SHIMA &&
                     (h.surface_flux == FLUX_RANOCHA || h.surface_flux == FLUX_HG ||
                      h.fv_flux == FLUX_RANOCHA || h.fv_flux == FLUX_HG);
  if (eq == 2) {  // ideal GLM-MHD (no source terms)
    if (h.src_kind != 0) return cudaErrorNotSupported;
    if (h.bc_kind >= 0 || hll) {  // non-periodic or the HLL family: the Dirichlet instantiations
      switch (dim) {
        case 1: return mixed ? launch_fused_1d_f32_mhd_bnd(N, eq, vol, vflux, h, s) : launch_fused_1d_f64_mhd_bnd(N, eq, vol, vflux, h, s);
        case 2: return mixed ? launch_fused_2d_f32_mhd_bnd(N, eq, vol, vflux, h, s) : launch_fused_2d_f64_mhd_bnd(N, eq, vol, vflux, h, s);
        case 3: return mixed ? launch_fused_3d_f32_mhd_bnd(N, eq, vol, vflux, h, s) : launch_fused_3d_f64_mhd_bnd(N, eq, vol, vflux, h, s);
      }
      return cudaErrorNotSupported;
    }
    switch (dim) {
      case 1: return mixed ? launch_fused_1d_f32_mhd(N, eq, vol, vflux, h, s) : launch_fused_1d_f64_mhd(N, eq, vol, vflux, h, s);
      case 2: return mixed ? launch_fused_2d_f32_mhd(N, eq, vol, vflux, h, s) : launch_fused_2d_f64_mhd(N, eq, vol, vflux, h, s);
      case 3: return mixed ? launch_fused_3d_f32_mhd(N, eq, vol, vflux, h, s) : launch_fused_3d_f64_mhd(N, eq, vol, vflux, h, s);
    }
    return cudaErrorNotSupported;
  }
  if (h.bc_kind >= 0 || h.src_kind != 0 || hll || ec_sc) {  // the instantiations with boundary states and sources
    if (vflux == 5) return cudaErrorNotSupported;  // flux_shima_etal: periodic kernels only
    switch (dim) {
      case 1:
        return mixed ? launch_fused_1d_f32_bnd(N, eq, vol, vflux, h, s) : launch_fused_1d_f64_bnd(N, eq, vol, vflux, h, s);
      case 2:
        return mixed ? launch_fused_2d_f32_bnd(N, eq, vol, vflux, h, s) : launch_fused_2d_f64_bnd(N, eq, vol, vflux, h, s);
      case 3:
        return mixed ? launch_fused_3d_f32_bnd(N, eq, vol, vflux, h, s) : launch_fused_3d_f64_bnd(N, eq, vol, vflux, h, s);
    }
    return cudaErrorNotSupported;
  }
  switch (dim) {
    case 1: return mixed ? launch_fused_1d_f32(N, eq, vol, vflux, h, s) : launch_fused_1d_f64(N, eq, vol, vflux, h, s);
    case 2: return mixed ? launch_fused_2d_f32(N, eq, vol, vflux, h, s) : launch_fused_2d_f64(N, eq, vol, vflux, h, s);
    case 3: return mixed ? launch_fused_3d_f32(N, eq, vol, vflux, h, s) : launch_fused_3d_f64(N, eq, vol, vflux, h, s);
  }
  return cudaErrorNotSupported;
}

}  // namespace trixi
