// dg_host.h -- host-side interface between the C ABI layer and the kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "dg_analysis.h"
#include "dg_consts.h"

namespace trixi {

constexpr int HOST_NMAX = 6;  // largest N = polydeg + 1 with compiled kernels

// records the message returned by trixi_last_error(NULL, ...) (trixi_api.cu)
void set_last_error(int status, const char *msg);

// Launch arguments of the fused kernel, precision independent.
struct FusedHost {
  const double *u_in = nullptr;
  double *out = nullptr;
  double *k = nullptr;
  const int32_t *face_table = nullptr;
  const double *mortar_flux = nullptr;
  const double *inv_jac = nullptr;
  const double *alpha = nullptr;
  const double *dt_elem = nullptr;
  // FP32 copies of u_in / u_out (FP32-mixed Euler and MHD RK stages of
  // trixi_rk_steps); null when absent
  const float *u32_in = nullptr;
  float *u32_out = nullptr;
  int *err = nullptr;
  int64_t nelements = 0;
  int mode = 1;
  int surface_flux = 0, fv_flux = 0;
  double rk_a = 0, rk_b = 0, dt = 0, atol = 0;
  double gamma = 1.4;
  double adv[3] = {0, 0, 0};
  double c_h = 0.0;  // GLM cleaning speed (ideal GLM-MHD)
  int N = 0;
  double dsplit[HOST_NMAX * HOST_NMAX] = {};  // row-major, diagonal zeroed
  double dhat[HOST_NMAX * HOST_NMAX] = {};    // row-major
  double invw[HOST_NMAX] = {};
  double lhat_l = 0, lhat_r = 0;
  // tile of the fused kernel: warps per group and groups per block (0 = the
  // compile-time defaults); a non-null tile_out makes launch_fused report the
  // kernel's tile limits instead of launching
  int wpg = 0, gpb = 0;
  int pdl = 0;  // launch as a programmatic dependent launch (overlaps the launch with the previous kernel's tail)
  struct FusedTile *tile_out = nullptr;
  // non-periodic meshes and source terms
  const double *coords = nullptr;  // [E][NN][DIM]
  double t = 0.0;
  int bc_kind = -1, src_kind = 0;
  IcParams bc{};
  double src[3] = {0, 0, 0};
};

// Tile limits of one fused-kernel instantiation.
struct FusedTile {
  int epg = 0;            // elements per group (compile time)
  int min_wpg = 0;        // warps owning the group's nodes
  int def_wpg = 0, def_gpb = 0;
  size_t group_smem = 0;  // bytes of shared memory per group
  int max_warps = 16;     // warps per block allowed by the instantiation's launch bounds
};

// Returns cudaErrorNotSupported when the combination is not compiled.
cudaError_t launch_fused(int dim, int N, int eq, int vol, int vflux, bool mixed, const FusedHost &h,
                         cudaStream_t s);
bool fused_supported(int dim, int N, int eq, int vol, int vflux);

cudaError_t launch_fused_1d_f64(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s);
cudaError_t launch_fused_1d_f32_bnd(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s);
cudaError_t launch_fused_1d_f64_bnd(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s);
cudaError_t launch_fused_2d_f32_bnd(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s);
cudaError_t launch_fused_2d_f64_bnd(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s);
cudaError_t launch_fused_3d_f32_bnd(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s);
cudaError_t launch_fused_3d_f64_bnd(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s);
cudaError_t launch_fused_2d_f64(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s);
cudaError_t launch_fused_3d_f64(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s);
cudaError_t launch_fused_1d_f32(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s);
cudaError_t launch_fused_2d_f32(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s);
cudaError_t launch_fused_3d_f32(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s);
// ideal GLM-MHD instantiations (periodic meshes)
cudaError_t launch_fused_1d_f64_mhd(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s);
cudaError_t launch_fused_1d_f32_mhd(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s);
cudaError_t launch_fused_2d_f64_mhd(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s);
cudaError_t launch_fused_2d_f32_mhd(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s);
cudaError_t launch_fused_3d_f64_mhd(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s);
cudaError_t launch_fused_3d_f32_mhd(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s);
cudaError_t launch_fused_1d_f64_mhd_bnd(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s);
cudaError_t launch_fused_1d_f32_mhd_bnd(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s);
cudaError_t launch_fused_2d_f64_mhd_bnd(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s);
cudaError_t launch_fused_2d_f32_mhd_bnd(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s);
cudaError_t launch_fused_3d_f64_mhd_bnd(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s);
cudaError_t launch_fused_3d_f32_mhd_bnd(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s);

// Auxiliary kernels (dg_aux.cu).
struct MortarHost {
  int dim = 2, N = 0, eq = 0, nv = 1;
  int64_t nmortars = 0;
  const double *u = nullptr;
  const int64_t *neighbor_ids = nullptr;  // [nchild+1, M] 1-based
  const int64_t *large_sides = nullptr;
  const int64_t *orientations = nullptr;
  double *mortar_flux = nullptr;           // [M*(nchild+1)][NF][NV]
  int surface_flux = 0;
  bool mixed = false;
  double gamma = 1.4, adv[3] = {0, 0, 0};
  double c_h = 0.0;
  double fwd_up[HOST_NMAX * HOST_NMAX] = {}, fwd_lo[HOST_NMAX * HOST_NMAX] = {};  // row-major [j][i]
  double rev_up[HOST_NMAX * HOST_NMAX] = {}, rev_lo[HOST_NMAX * HOST_NMAX] = {};  // row-major [k][j]
  int *err = nullptr;
};
cudaError_t launch_mortar_flux(const MortarHost &m, cudaStream_t s);

struct IndicatorHost {
  int dim = 2, N = 0, nv = 4, eq = 1;
  bool mixed = false;  // FP32 arithmetic (the FP32-mixed rhs), else FP64
  int variable = 0;    // 0: density_pressure, 1: pressure
  int64_t nelements = 0;
  const double *u = nullptr;
  const float *u32 = nullptr;  // FP32 copy of u (mixed only): read in place of u when not null
  double *alpha_raw = nullptr;
  double *alpha = nullptr;                 // smoothed output
  const int32_t *face_table = nullptr;     // [E][2*DIM]
  const int32_t *slot_neighbors = nullptr; // [slot][4] element ids (-1 padded) for mortar faces
  int smooth = 1;
  double gamma = 1.4;
  double alpha_max = 0.5, alpha_min = 0.001;
  double threshold = 0, parameter_s = 0;
  double ivdm[HOST_NMAX * HOST_NMAX] = {};  // row-major inverse Vandermonde
  int pdl = 0;  // launch both kernels as programmatic dependent launches
};
cudaError_t launch_indicator(const IndicatorHost &ih, cudaStream_t s);

// Stage kernels with the reference's stage split (FP64).
struct StageHost {
  int dim = 2, N = 0, nv = 1, eq = 0;
  int64_t nelements = 0, ninterfaces = 0, nmortars = 0;
  const int64_t *if_neighbor_ids = nullptr, *if_orientations = nullptr;
  const int64_t *mo_neighbor_ids = nullptr, *mo_large_sides = nullptr, *mo_orientations = nullptr;
  double *interfaces_u = nullptr;
  double *sfv = nullptr;
  double *mortar_u[4] = {nullptr, nullptr, nullptr, nullptr};
  int surface_flux = 0;
  double gamma = 1.4, adv[3] = {0, 0, 0};
  double c_h = 0.0;
  double fwd_up[HOST_NMAX * HOST_NMAX] = {}, fwd_lo[HOST_NMAX * HOST_NMAX] = {};
  double rev_up[HOST_NMAX * HOST_NMAX] = {}, rev_lo[HOST_NMAX * HOST_NMAX] = {};
  double lhat_l = 0, lhat_r = 0;
  const double *inv_jac = nullptr;
  // non-periodic meshes and source terms
  int64_t nboundaries = 0;
  const int64_t *bnd_neighbor_ids = nullptr, *bnd_sides = nullptr, *bnd_orientations = nullptr;
  double *boundaries_u = nullptr;  // [B][NF][nv][2]
  const double *coords = nullptr;  // [E][NN][DIM]
  int bc_kind = -1, src_kind = 0;
  IcParams bc{};
  double src[3] = {0, 0, 0};
};
cudaError_t stage_prolong2interfaces(const StageHost &sh, const double *u, cudaStream_t s);
cudaError_t stage_prolong2boundaries(const StageHost &sh, const double *u, cudaStream_t s);
cudaError_t stage_boundary_flux(const StageHost &sh, double t, cudaStream_t s);
cudaError_t stage_sources(const StageHost &sh, double *du, double t, cudaStream_t s);
cudaError_t stage_interface_flux(const StageHost &sh, cudaStream_t s);
cudaError_t stage_prolong2mortars(const StageHost &sh, const double *u, cudaStream_t s);
cudaError_t stage_mortar_flux(const StageHost &sh, cudaStream_t s);
cudaError_t stage_surface_integral(const StageHost &sh, double *du, cudaStream_t s);
cudaError_t stage_jacobian(const StageHost &sh, double *du, cudaStream_t s);

}  // namespace trixi
