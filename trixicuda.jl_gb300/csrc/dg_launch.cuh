// dg_launch.cuh -- instantiation and launch of the fused kernel for one
// (dimension, compute precision).  Included by fused_{1,2,3}d_{f64,f32}.cu,
// which are compiled in parallel.
#pragma once
#include <algorithm>

#include "dg_adv.cuh"
#include "dg_fused.cuh"
#include "dg_host.h"

namespace trixi {

template <int DIM, int N, int EQ, typename R, int VOL, int VF, int BND>
cudaError_t launch_one(const FusedHost &h, cudaStream_t s) {
  using K = FusedKernel<DIM, N, EQ, R, VOL, VF, BND>;
  FusedParams<R> p;
  p.u_in = h.u_in;
  p.out = h.out;
  p.k = h.k;
  p.face_table = h.face_table;
  p.mortar_flux = h.mortar_flux;
  p.inv_jac = h.inv_jac;
  p.alpha = h.alpha;
  p.dt_elem = h.dt_elem;
  // the FP32 state copies exist for the FP32 instantiations only
  p.u32_in = (sizeof(R) == 4) ? h.u32_in : nullptr;
  p.u32_out = (sizeof(R) == 4) ? h.u32_out : nullptr;
  p.err = h.err;
  p.nelements = h.nelements;
  p.mode = h.mode;
  p.surface_flux = h.surface_flux;
  p.fv_flux = h.fv_flux;
  p.rk_a = h.rk_a;
  p.rk_b = h.rk_b;
  p.dt = h.dt;
  p.use_k = (h.rk_a != 0.0);
  p.coords = h.coords;
  p.t = h.t;
  p.bc_kind = h.bc_kind;
  p.src_kind = h.src_kind;
  p.bc = h.bc;
  for (int i = 0; i < 3; ++i) p.src[i] = h.src[i];
  const uintptr_t addr_bits = (uintptr_t)h.u_in | (uintptr_t)h.out | (uintptr_t)h.k | (uintptr_t)h.mortar_flux;
  p.vec16 = (addr_bits & 15u) == 0;
  p.atol = h.atol;
  p.pp.gamma = R(h.gamma);
  p.pp.gm1 = R(h.gamma - 1.0);
  p.pp.inv_gm1 = R(1.0 / (h.gamma - 1.0));
  for (int d = 0; d < 3; ++d) p.pp.a[d] = R(h.adv[d]);
  p.pp.c_h = R(h.c_h);
  for (int i = 0; i < NMAXT * NMAXT; ++i) {
    p.dsplit[i] = R(0);
    p.dhat[i] = R(0);
  }
  for (int i = 0; i < N * N; ++i) {
    p.dsplit[i] = R(h.dsplit[i]);
    p.dhat[i] = R(h.dhat[i]);
  }
  for (int i = 0; i < NMAXT; ++i) p.invw[i] = R(i < N ? h.invw[i] : 0.0);
  p.lhat_l = R(h.lhat_l);
  p.lhat_r = R(h.lhat_r);
  if constexpr (EQ == EQ_ADV && BND == 0) {
    // linear advection on periodic / mortar meshes: the dedicated kernel
    // (dg_adv.cuh).  Its block shape is fixed; the tile reported is that
    // block and is the only one accepted, so the tile tuner has a single
    // candidate
    using A = AdvKernel<DIM, N, R, VOL>;
    if (h.u32_in || h.u32_out) return cudaErrorNotSupported;  // it keeps no FP32 state copy
    if (h.tile_out) {
      h.tile_out->epg = 1;
      h.tile_out->min_wpg = h.tile_out->def_wpg = h.tile_out->max_warps = A::BLOCK / 32;
      h.tile_out->def_gpb = 1;
      h.tile_out->group_smem = 0;
      return cudaSuccess;
    }
    p.wpg = p.gpb = 1;
    const int64_t grid = (h.nelements + A::EPB - 1) / A::EPB;
    if (grid <= 0) return cudaSuccess;
    if (grid > 0x7fffffffLL) return cudaErrorInvalidValue;
    constexpr auto kernel = adv_entry<DIM, N, R, VOL>();
    if (h.pdl) {
      p.pdl = 1;
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3((unsigned)grid);
      cfg.blockDim = dim3(A::BLOCK);
      cfg.dynamicSmemBytes = 0;
      cfg.stream = s;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
      attr[0].val.programmaticStreamSerializationAllowed = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      return cudaLaunchKernelEx(&cfg, kernel, p);
    }
    p.pdl = 0;
    kernel<<<(unsigned)grid, A::BLOCK, 0, s>>>(p);
    return cudaGetLastError();
  }
  if (h.tile_out) {
    h.tile_out->epg = K::EPG;
    h.tile_out->min_wpg = K::warps_for(K::EPG);
    h.tile_out->def_wpg = K::WPG;
    h.tile_out->def_gpb = K::GPB;
    h.tile_out->group_smem = K::GROUP_SMEM;
    h.tile_out->max_warps = K::MAX_WARPS;
    return cudaSuccess;
  }
  // tile: the requested one when valid, else the compile-time defaults
  int wpg = K::WPG, gpb = K::GPB;
  if (h.wpg >= K::warps_for(K::EPG) && h.wpg <= 8 && h.gpb >= 1 && h.gpb <= 15 && h.gpb * h.wpg <= K::MAX_WARPS &&
      (size_t)h.gpb * K::GROUP_SMEM <= 200 * 1024) {
    wpg = h.wpg;
    gpb = h.gpb;
  }
  p.wpg = wpg;
  p.gpb = gpb;
  const int epb = gpb * K::EPG;  // elements per block
  const dim3 block(32 * wpg, gpb);  // x: threads of a group, y: groups
  const size_t smem = (size_t)gpb * K::GROUP_SMEM;
  // opt in once per instantiation to the large dynamic shared-memory carve-out
  constexpr auto kernel = fused_entry<DIM, N, EQ, R, VOL, VF, BND>();
  static const cudaError_t attr = cudaFuncSetAttribute(kernel,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  if (attr != cudaSuccess) return attr;
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  const int64_t grid = (h.nelements + epb - 1) / epb;
  if (grid <= 0) return cudaSuccess;
  if (grid > 0x7fffffffLL) return cudaErrorInvalidValue;
  if (h.pdl) {
    p.pdl = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, p);
  }
  p.pdl = 0;
  kernel<<<(unsigned)grid, block, smem, s>>>(p);
  return cudaGetLastError();
}

template <int DIM, int N, typename R, int BND>
cudaError_t launch_n(int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s) {
  if (eq == EQ_ADV) {
    if (vol == VOL_WEAK) return launch_one<DIM, N, EQ_ADV, R, VOL_WEAK, FLUX_CENTRAL, BND>(h, s);
    if (vol == VOL_FD) return launch_one<DIM, N, EQ_ADV, R, VOL_FD, FLUX_CENTRAL, BND>(h, s);
    return cudaErrorNotSupported;
  }
  if (vol == VOL_WEAK) return launch_one<DIM, N, EQ_EULER, R, VOL_WEAK, FLUX_CENTRAL, BND>(h, s);
  if (vol == VOL_FD) {
    if (vflux == FLUX_RANOCHA) return launch_one<DIM, N, EQ_EULER, R, VOL_FD, FLUX_RANOCHA, BND>(h, s);
    if (vflux == FLUX_CENTRAL) return launch_one<DIM, N, EQ_EULER, R, VOL_FD, FLUX_CENTRAL, BND>(h, s);
    if constexpr (!BND)
      if (vflux == FLUX_SHIMA) return launch_one<DIM, N, EQ_EULER, R, VOL_FD, FLUX_SHIMA, BND>(h, s);
    return cudaErrorNotSupported;
  }
  if (vol == VOL_SC) {
    if (vflux == FLUX_RANOCHA) return launch_one<DIM, N, EQ_EULER, R, VOL_SC, FLUX_RANOCHA, BND>(h, s);
    if (vflux == FLUX_CENTRAL) return launch_one<DIM, N, EQ_EULER, R, VOL_SC, FLUX_CENTRAL, BND>(h, s);
    if constexpr (!BND)
      if (vflux == FLUX_SHIMA) return launch_one<DIM, N, EQ_EULER, R, VOL_SC, FLUX_SHIMA, BND>(h, s);
  }
  return cudaErrorNotSupported;
}

// ideal GLM-MHD: flux differencing (flux_hindenlang_gassner or flux_central)
// and shock capturing (flux_hindenlang_gassner), polydeg 1..4
template <int DIM, int N, typename R, int BND>
cudaError_t launch_n_mhd(int vol, int vflux, const FusedHost &h, cudaStream_t s) {
  if (vol == VOL_FD) {
    if (vflux == FLUX_HG) return launch_one<DIM, N, EQ_MHD, R, VOL_FD, FLUX_HG, BND>(h, s);
    if (vflux == FLUX_CENTRAL) return launch_one<DIM, N, EQ_MHD, R, VOL_FD, FLUX_CENTRAL, BND>(h, s);
  }
  if (vol == VOL_SC && vflux == FLUX_HG) return launch_one<DIM, N, EQ_MHD, R, VOL_SC, FLUX_HG, BND>(h, s);
  return cudaErrorNotSupported;
}

// BND = 1: non-periodic meshes (Dirichlet states as the neighbour traces)
template <int DIM, typename R, int BND = 0>
cudaError_t launch_dim_mhd(int N, int vol, int vflux, const FusedHost &h, cudaStream_t s) {
  switch (N) {
    case 2: return launch_n_mhd<DIM, 2, R, BND>(vol, vflux, h, s);
    case 3: return launch_n_mhd<DIM, 3, R, BND>(vol, vflux, h, s);
    case 4: return launch_n_mhd<DIM, 4, R, BND>(vol, vflux, h, s);
    case 5: return launch_n_mhd<DIM, 5, R, BND>(vol, vflux, h, s);
    default: return cudaErrorNotSupported;
  }
}

template <int DIM, typename R, int BND>
cudaError_t launch_dim(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s) {
  switch (N) {
    case 2: return launch_n<DIM, 2, R, BND>(eq, vol, vflux, h, s);
    case 3: return launch_n<DIM, 3, R, BND>(eq, vol, vflux, h, s);
    case 4: return launch_n<DIM, 4, R, BND>(eq, vol, vflux, h, s);
    case 5: return launch_n<DIM, 5, R, BND>(eq, vol, vflux, h, s);
    case 6: return launch_n<DIM, 6, R, BND>(eq, vol, vflux, h, s);
    default: return cudaErrorNotSupported;
  }
}

}  // namespace trixi
