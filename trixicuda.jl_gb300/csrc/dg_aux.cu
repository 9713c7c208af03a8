// dg_aux.cu -- auxiliary DGSEM kernels:
//   * mortar pre-pass of the fused path (one block per mortar),
//   * Hennemann-Gassner indicator + smoothing on the GPU,
//   * stage kernels with the reference's stage split, filling the reference
//     containers (interfaces.u, surface_flux_values, mortar u arrays).
#include <algorithm>

#include "dg_host.h"
#include "dg_ic.cuh"
#include "dg_convert.cuh"
#include "dg_indicator.cuh"
#include "dg_physics.cuh"

namespace trixi {

// Node index of the point at position `a` along orientation o whose face
// coordinates are given by face index f (remaining dimensions in increasing
// order, first fastest) -- the index order of interfaces.u and
// surface_flux_values in src/solvers/containers_{2,3}d.jl.
__device__ __forceinline__ int node_of(int dim, int N, int o, int a, int f) {
  if (dim == 1) return a;
  if (dim == 2) return (o == 0) ? a + N * f : f + N * a;
  const int f1 = f % N, f2 = f / N;
  if (o == 0) return a + N * f1 + N * N * f2;
  if (o == 1) return f1 + N * a + N * N * f2;
  return f1 + N * f2 + N * N * a;
}

template <int DIM, int EQ, typename R>
__device__ __forceinline__ void flux_dispatch(int kind, int o, const R *ul, const R *wl, const R *ur, const R *wr,
                                              R *f, const PhysParams<R> &pp) {
  if (o == 0) two_point_flux<DIM, EQ, R, 0>(kind, ul, wl, ur, wr, f, pp);
  if constexpr (DIM > 1) if (o == 1) two_point_flux<DIM, EQ, R, 1>(kind, ul, wl, ur, wr, f, pp);
  if constexpr (DIM > 2) if (o == 2) two_point_flux<DIM, EQ, R, 2>(kind, ul, wl, ur, wr, f, pp);
}

// f += s * Phi_o(own, other), the nonconservative term of ideal GLM-MHD in
// 2D/3D (nothing for the other systems)
template <int DIM, int EQ, typename R>
__device__ __forceinline__ void add_noncons_rt(int o, const R *wown, const R *wother, R s, R *f) {
  if constexpr (EQ == EQ_MHD && DIM > 1) {
    using P = Physics<DIM, EQ, R>;
    if (o == 0) P::template add_noncons<0>(wown, wother, s, f);
    if (o == 1) P::template add_noncons<1>(wown, wother, s, f);
    if constexpr (DIM > 2) if (o == 2) P::template add_noncons<2>(wown, wother, s, f);
  }
}

template <typename R>
static PhysParams<R> make_pp(double gamma, const double *adv, double c_h = 0.0) {
  PhysParams<R> pp;
  pp.gamma = R(gamma);
  pp.gm1 = R(gamma - 1.0);
  pp.inv_gm1 = R(1.0 / (gamma - 1.0));
  for (int d = 0; d < 3; ++d) pp.a[d] = R(adv[d]);
  pp.c_h = R(c_h);
  return pp;
}

struct Mats {
  double fwd_up[HOST_NMAX * HOST_NMAX], fwd_lo[HOST_NMAX * HOST_NMAX];
  double rev_up[HOST_NMAX * HOST_NMAX], rev_lo[HOST_NMAX * HOST_NMAX];
};

// ---------------------------------------------------------------------------
// Mortar pre-pass (fused path).  Per mortar: project the large element's face
// trace onto each small face (forward_lower/upper, tensor product in 3D, FP64),
// evaluate the surface flux on the small faces, and back-project to the large
// face with reverse_lower/upper (exact L2 projection, FP64).  Results go to
// per-face slots [slot][NF][NV]: slot m*(nchild+1)+c for small child c, and
// m*(nchild+1)+nchild for the large face.  Follows
// src/solvers/dg_2d_kernel.jl:1167-1397 and dg_3d_kernel.jl:1361-1770.
// ---------------------------------------------------------------------------
template <int DIM, int EQ, typename R>
__global__ void mortar_prepass_kernel(int N, int64_t M, const double *__restrict__ u,
                                      const int64_t *__restrict__ nid, const int64_t *__restrict__ large_sides,
                                      const int64_t *__restrict__ orientations, double *__restrict__ out,
                                      int surface_flux, PhysParams<R> pp, Mats mats, int *err) {
  constexpr int NV = NVarsOf<DIM, EQ>::value;
  constexpr int NC = 1 << (DIM - 1);
  extern __shared__ __align__(16) double sm[];
  const int NF = (DIM == 2) ? N : N * N;
  const int NN = NF * N;
  double *s_large = sm;               // [NF][NV]
  double *s_fstar = sm + NF * NV;     // [NC][NF][NV]
  const int64_t m = blockIdx.x;
  if (m >= M) return;
  const int o = (int)orientations[m] - 1;
  const int ls = (int)large_sides[m];
  const int64_t large = nid[NC + (NC + 1) * m] - 1;
  const int large_a = (ls == 1) ? N - 1 : 0;
  const int small_a = (ls == 1) ? 0 : N - 1;
  for (int i = threadIdx.x; i < NF * NV; i += blockDim.x) {
    const int f = i / NV, v = i - (i / NV) * NV;
    s_large[i] = u[(large * NN + node_of(DIM, N, o, large_a, f)) * NV + v];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < NC * NF; i += blockDim.x) {
    const int c = i / NF, f = i - c * NF;
    const int64_t small = nid[c + (NC + 1) * m] - 1;
    double pl[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) pl[v] = 0.0;
    if (DIM == 2) {
      const double *F = (c == 1) ? mats.fwd_up : mats.fwd_lo;
      for (int jj = 0; jj < N; ++jj)
#pragma unroll
        for (int v = 0; v < NV; ++v) pl[v] += F[f * N + jj] * s_large[jj * NV + v];
    } else {
      const double *F1 = (c & 1) ? mats.fwd_up : mats.fwd_lo;   // first tangent: left/right
      const double *F2 = (c >> 1) ? mats.fwd_up : mats.fwd_lo;  // second tangent: lower/upper
      const int fa = f % N, fb = f / N;
      for (int jb = 0; jb < N; ++jb) {
        double t[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) t[v] = 0.0;
        for (int ja = 0; ja < N; ++ja)
#pragma unroll
          for (int v = 0; v < NV; ++v) t[v] += F1[fa * N + ja] * s_large[(ja + N * jb) * NV + v];
#pragma unroll
        for (int v = 0; v < NV; ++v) pl[v] += F2[fb * N + jb] * t[v];
      }
    }
    R ul[NV], ur[NV], wl[NV], wr[NV], fs[NV];
    const double *us = u + (small * NN + node_of(DIM, N, o, small_a, f)) * NV;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      ul[v] = R(ls == 1 ? pl[v] : us[v]);
      ur[v] = R(ls == 1 ? us[v] : pl[v]);
    }
    Physics<DIM, EQ, R>::prim(ul, wl, pp);
    Physics<DIM, EQ, R>::prim(ur, wr, pp);
    flux_dispatch<DIM, EQ, R>(surface_flux, o, ul, wl, ur, wr, fs, pp);
    // nonconservative terms (mortar_flux_kernel!, src/solvers/dg_2d_kernel.jl:1290-1344):
    // the small element's flux adds 0.5 Phi(u_large, u_small) ("primary"), the
    // one projected to the large element 0.5 Phi(u_small, u_large) ("secondary"),
    // u_large being the large element's trace projected onto the small face
    R fsec[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) fsec[v] = fs[v];
    if constexpr (EQ == EQ_MHD && DIM > 1) {
      const R *w_large = (ls == 1) ? wl : wr, *w_small = (ls == 1) ? wr : wl;
      add_noncons_rt<DIM, EQ, R>(o, w_large, w_small, R(0.5), fs);
      add_noncons_rt<DIM, EQ, R>(o, w_small, w_large, R(0.5), fsec);
    }
    double *dst = out + ((m * (NC + 1) + c) * NF + f) * NV;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      s_fstar[(c * NF + f) * NV + v] = double(fsec[v]);
      dst[v] = double(fs[v]);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < NF * NV; i += blockDim.x) {
    const int f = i / NV, v = i - (i / NV) * NV;
    double s = 0.0;
    if (DIM == 2) {
      for (int c = 0; c < NC; ++c) {
        const double *Rm = (c == 1) ? mats.rev_up : mats.rev_lo;
        for (int jj = 0; jj < N; ++jj) s += Rm[f * N + jj] * s_fstar[(c * NF + jj) * NV + v];
      }
    } else {
      const int fa = f % N, fb = f / N;
      for (int c = 0; c < NC; ++c) {
        const double *R1 = (c & 1) ? mats.rev_up : mats.rev_lo;
        const double *R2 = (c >> 1) ? mats.rev_up : mats.rev_lo;
        for (int jb = 0; jb < N; ++jb) {
          double t = 0.0;
          for (int ja = 0; ja < N; ++ja) t += R1[fa * N + ja] * s_fstar[(c * NF + ja + N * jb) * NV + v];
          s += R2[fb * N + jb] * t;
        }
      }
    }
    out[((m * (NC + 1) + NC) * NF + f) * NV + v] = s;
  }
}

template <int DIM, int EQ, typename R>
static cudaError_t launch_mortar_t(const MortarHost &mh, cudaStream_t s) {
  constexpr int NV = NVarsOf<DIM, EQ>::value;
  constexpr int NC = 1 << (DIM - 1);
  const int NF = (DIM == 2) ? mh.N : mh.N * mh.N;
  Mats mats;
  std::copy(mh.fwd_up, mh.fwd_up + HOST_NMAX * HOST_NMAX, mats.fwd_up);
  std::copy(mh.fwd_lo, mh.fwd_lo + HOST_NMAX * HOST_NMAX, mats.fwd_lo);
  std::copy(mh.rev_up, mh.rev_up + HOST_NMAX * HOST_NMAX, mats.rev_up);
  std::copy(mh.rev_lo, mh.rev_lo + HOST_NMAX * HOST_NMAX, mats.rev_lo);
  const size_t smem = sizeof(double) * (size_t)(NF * NV + NC * NF * NV);
  const int block = std::max(32, std::min(256, ((NC * NF + 31) / 32) * 32));
  mortar_prepass_kernel<DIM, EQ, R><<<(unsigned)mh.nmortars, block, smem, s>>>(
      mh.N, mh.nmortars, mh.u, mh.neighbor_ids, mh.large_sides, mh.orientations, mh.mortar_flux, mh.surface_flux,
      make_pp<R>(mh.gamma, mh.adv, mh.c_h), mats, mh.err);
  return cudaGetLastError();
}

cudaError_t launch_mortar_flux(const MortarHost &mh, cudaStream_t s) {
  if (mh.nmortars <= 0) return cudaSuccess;
  if (mh.eq == EQ_MHD) {
    if (mh.dim == 2) return mh.mixed ? launch_mortar_t<2, EQ_MHD, float>(mh, s) : launch_mortar_t<2, EQ_MHD, double>(mh, s);
    if (mh.dim == 3) return mh.mixed ? launch_mortar_t<3, EQ_MHD, float>(mh, s) : launch_mortar_t<3, EQ_MHD, double>(mh, s);
    return cudaErrorNotSupported;
  }
  if (mh.dim == 2) {
    if (mh.eq == EQ_ADV) return mh.mixed ? launch_mortar_t<2, EQ_ADV, float>(mh, s) : launch_mortar_t<2, EQ_ADV, double>(mh, s);
    return mh.mixed ? launch_mortar_t<2, EQ_EULER, float>(mh, s) : launch_mortar_t<2, EQ_EULER, double>(mh, s);
  }
  if (mh.dim == 3) {
    if (mh.eq == EQ_ADV) return mh.mixed ? launch_mortar_t<3, EQ_ADV, float>(mh, s) : launch_mortar_t<3, EQ_ADV, double>(mh, s);
    return mh.mixed ? launch_mortar_t<3, EQ_EULER, float>(mh, s) : launch_mortar_t<3, EQ_EULER, double>(mh, s);
  }
  return cudaErrorNotSupported;
}

// ---------------------------------------------------------------------------
// Hennemann-Gassner indicator (src/solvers/indicators.jl:7-42; Hennemann et al.
// 2021): rho*p per node, modal coefficients via the inverse Legendre
// Vandermonde dimension by dimension, energy fractions of the highest and
// second-highest modes, logistic blending with alpha_min / alpha_max clipping.
// ---------------------------------------------------------------------------
struct IvdmMat {
  double m[HOST_NMAX * HOST_NMAX];
};

// Eight elements per block, N a compile-time constant, compute type R
// (double; float in the FP32-mixed rhs, states narrowed on the integer pipe).
// Each warp computes rho*p and the modal transform of one element.  Then warp 0
// accumulates the three energy sums of all eight elements at once -- three
// lanes per element, each a sequential fold in node order, the oracle's
// order, so the FP64 result matches it bit for bit.  An FP64 warp instruction
// occupies GB300's narrow FP64 pipe for the whole warp however few lanes are
// active, so a sequential fold per element on a single lane cost ~0.4 ms per
// call on the 3D level-5 mesh; folding 24 sums in one instruction stream
// divides that by eight.
template <typename R>
__device__ __forceinline__ R ind_load(const double *p) { return R(*p); }
template <>
__device__ __forceinline__ float ind_load<float>(const double *p) { return from_double<float>(*p); }
// the FP32 copy of u that trixi_rk_steps keeps between FP32-mixed stages
// holds the same narrowing of u
template <typename R>
__device__ __forceinline__ R ind_load(const float *p) { return *p; }

// In: double (u itself) or float (its FP32 copy, FP32 arithmetic only)
template <int DIM, int N, typename R, typename In = double>
__global__ void __launch_bounds__(256) indicator_raw_kernel(int64_t E, const In *__restrict__ u,
                                                            double *__restrict__ alpha_raw, double gamma_, double amax,
                                                            double amin, double threshold_, double param_s_,
                                                            IvdmMat ivdm, int mhd, int nv, int variable,
                                                            int pdl) {
  if (pdl) {
    // programmatic dependent launch: the next kernel may start launching;
    // u (the previous kernel's output) is read only after this wait
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
  }
  constexpr int NN = (DIM == 1) ? N : (DIM == 2 ? N * N : N * N * N);
  constexpr int WPB = 8;  // warps (elements) per block
  extern __shared__ __align__(16) unsigned char sm_raw[];
  R *s_iv = reinterpret_cast<R *>(sm_raw);  // [N][N] inverse Vandermonde (lanes read it at different indices)
  for (int i = threadIdx.x; i < N * N; i += blockDim.x) s_iv[i] = R(ivdm.m[i]);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t e0 = (int64_t)blockIdx.x * WPB;
  const int64_t e = e0 + warp;
  R *a = s_iv + N * N + warp * 2 * NN, *b = a + NN;
  if (e < E) {
    const R gm1 = R(gamma_ - 1.0);
    for (int n = lane; n < NN; n += 32) {
      const In *un = u + (e * NN + n) * nv;
      R c[9];
#pragma unroll
      for (int v = 0; v < 9; ++v)
        if (v < nv) c[v] = ind_load<R>(un + v);
      a[n] = ind_value<DIM, R>(c, gm1, mhd != 0, nv, variable);
    }
    __syncwarp();
    R *src = a, *dst = b;
    int stride = 1;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      for (int n = lane; n < NN; n += 32) {
        const int c = (n / stride) % N;
        const int nb = n - c * stride;
        R acc = R(0);
#pragma unroll
        for (int m = 0; m < N; ++m) acc += s_iv[c * N + m] * src[nb + m * stride];
        dst[n] = acc;
      }
      __syncwarp();
      R *t = src;
      src = dst;
      dst = t;
      stride *= N;
    }
  }
  // the transform alternates between a and b per dimension: after DIM passes
  // the coefficients sit in a when DIM is even, in b when it is odd
  if constexpr (sizeof(R) == 4) {
    // FP32: each warp folds its own element
    if (e < E) {
      float total, clip1, clip2;
      ind_energy_sums_warp<DIM, N>((DIM & 1) ? b : a, lane, total, clip1, clip2);
      if (lane == 0) alpha_raw[e] = ind_alpha<R>(total, clip1, clip2, threshold_, param_s_, amax, amin);
    }
    return;
  }
  __syncthreads();
  if (warp != 0) return;
  const int el = lane / 3, which = lane - 3 * (lane / 3);  // which: 0 all modes, 1 without the highest, 2 without two
  const bool active = lane < 3 * WPB && e0 + el < E;
  R sum = R(0);
  if (active) sum = ind_energy_sum<DIM, N, R>(s_iv + N * N + el * 2 * NN + ((DIM & 1) ? NN : 0), which);
  const R clip1 = __shfl_down_sync(0xffffffffu, sum, 1), clip2 = __shfl_down_sync(0xffffffffu, sum, 2);
  if (active && which == 0) alpha_raw[e0 + el] = ind_alpha<R>(sum, clip1, clip2, threshold_, param_s_, amax, amin);
}

// A launch that may be a programmatic dependent launch (the kernel then
// executes griddepcontrol.wait before reading its predecessor's output).
template <typename... KArgs, typename... Args>
static cudaError_t launch_maybe_pdl(void (*kernel)(KArgs...), unsigned grid, unsigned block, size_t smem,
                                    cudaStream_t s, bool pdl, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

template <int DIM, int N>
static cudaError_t launch_indicator_raw(const IndicatorHost &ih, cudaStream_t s) {
  constexpr int NN = (DIM == 1) ? N : (DIM == 2 ? N * N : N * N * N);
  const int64_t grid = (ih.nelements + 7) / 8;
  IvdmMat iv;
  std::copy(ih.ivdm, ih.ivdm + HOST_NMAX * HOST_NMAX, iv.m);
  if (ih.mixed && ih.u32) {
    const size_t smem = sizeof(float) * (size_t)(N * N + 8 * 2 * NN);
    return launch_maybe_pdl(&indicator_raw_kernel<DIM, N, float, float>, (unsigned)grid, 256, smem, s, ih.pdl != 0,
                            ih.nelements, ih.u32, ih.alpha_raw, ih.gamma, ih.alpha_max, ih.alpha_min, ih.threshold,
                            ih.parameter_s, iv, ih.eq == EQ_MHD ? 1 : 0, ih.nv, ih.variable, ih.pdl);
  } else if (ih.mixed) {
    const size_t smem = sizeof(float) * (size_t)(N * N + 8 * 2 * NN);
    return launch_maybe_pdl(&indicator_raw_kernel<DIM, N, float, double>, (unsigned)grid, 256, smem, s, ih.pdl != 0,
                            ih.nelements, ih.u, ih.alpha_raw, ih.gamma, ih.alpha_max, ih.alpha_min, ih.threshold,
                            ih.parameter_s, iv, ih.eq == EQ_MHD ? 1 : 0, ih.nv, ih.variable, ih.pdl);
  } else {
    const size_t smem = sizeof(double) * (size_t)(N * N + 8 * 2 * NN);
    return launch_maybe_pdl(&indicator_raw_kernel<DIM, N, double, double>, (unsigned)grid, 256, smem, s, ih.pdl != 0,
                            ih.nelements, ih.u, ih.alpha_raw, ih.gamma, ih.alpha_max, ih.alpha_min, ih.threshold,
                            ih.parameter_s, iv, ih.eq == EQ_MHD ? 1 : 0, ih.nv, ih.variable, ih.pdl);
  }
  return cudaGetLastError();
}

template <int DIM>
static cudaError_t launch_indicator_dim(const IndicatorHost &ih, cudaStream_t s) {
  switch (ih.N) {
    case 2: return launch_indicator_raw<DIM, 2>(ih, s);
    case 3: return launch_indicator_raw<DIM, 3>(ih, s);
    case 4: return launch_indicator_raw<DIM, 4>(ih, s);
    case 5: return launch_indicator_raw<DIM, 5>(ih, s);
    case 6: return launch_indicator_raw<DIM, 6>(ih, s);
  }
  return cudaErrorNotSupported;
}

// alpha[e] = max(alpha_raw[e], 0.5 * alpha_raw[face neighbours]) -- the result
// of Trixi's apply_smoothing! over interfaces and mortars.
__global__ void indicator_smooth_kernel(int dim, int64_t E, const double *__restrict__ alpha_raw,
                                        double *__restrict__ alpha, const int32_t *__restrict__ face_table,
                                        const int32_t *__restrict__ slot_nbrs, int smooth, int pdl) {
  if (pdl) {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
  }
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  double a = alpha_raw[e];
  if (smooth) {
    for (int f = 0; f < 2 * dim; ++f) {
      const int32_t nb = face_table[e * 2 * dim + f];
      if (nb >= 0) {
        a = fmax(a, 0.5 * alpha_raw[nb]);
      } else if (nb != FACE_BOUNDARY) {  // a domain boundary has no neighbour to smooth with
        const int32_t slot = -nb - 1;
        for (int j = 0; j < 4; ++j) {
          const int32_t n2 = slot_nbrs[slot * 4 + j];
          if (n2 >= 0) a = fmax(a, 0.5 * alpha_raw[n2]);
        }
      }
    }
  }
  alpha[e] = a;
}

cudaError_t launch_indicator(const IndicatorHost &ih, cudaStream_t s) {
  if (ih.nelements <= 0) return cudaSuccess;
  cudaError_t e = (ih.dim == 1) ? launch_indicator_dim<1>(ih, s)
                  : (ih.dim == 2) ? launch_indicator_dim<2>(ih, s) : launch_indicator_dim<3>(ih, s);
  if (e != cudaSuccess) return e;
  return launch_maybe_pdl(&indicator_smooth_kernel, (unsigned)((ih.nelements + 255) / 256), 256, 0, s, ih.pdl != 0,
                          ih.dim, ih.nelements, (const double *)ih.alpha_raw, ih.alpha, ih.face_table,
                          ih.slot_neighbors, ih.smooth, ih.pdl);
}

// ---------------------------------------------------------------------------
// Stage kernels (FP64), reference container layouts.
// ---------------------------------------------------------------------------

// prolong_interfaces_kernel! (dg_2d_kernel.jl:907-935, dg_3d_kernel.jl:1121-1152)
__global__ void prolong_interfaces_kernel(int dim, int N, int nv, int64_t I, const double *__restrict__ u,
                                          const int64_t *__restrict__ nid, const int64_t *__restrict__ ori,
                                          double *__restrict__ iu) {
  int NF = 1;
  for (int d = 1; d < dim; ++d) NF *= N;
  const int NN = NF * N;
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= I * NF * nv) return;
  const int v = (int)(idx % nv);
  const int f = (int)((idx / nv) % NF);
  const int64_t k = idx / ((int64_t)nv * NF);
  const int o = (int)ori[k] - 1;
  const int64_t left = nid[2 * k] - 1, right = nid[2 * k + 1] - 1;
  iu[2 * idx + 0] = u[(left * NN + node_of(dim, N, o, N - 1, f)) * nv + v];
  iu[2 * idx + 1] = u[(right * NN + node_of(dim, N, o, 0, f)) * nv + v];
}

// prolong_boundaries_kernel! (dg_2d_kernel.jl:1037-1064): boundaries_u[2, nv,
// NF, B] holds the element's trace on its side of the boundary (index 1 when
// the element lies on the left, 2 on the right) and zero on the other side
__global__ void prolong_boundaries_kernel(int dim, int N, int nv, int64_t B, const double *__restrict__ u,
                                          const int64_t *__restrict__ nid, const int64_t *__restrict__ side,
                                          const int64_t *__restrict__ ori, double *__restrict__ bu) {
  int NF = 1;
  for (int d = 1; d < dim; ++d) NF *= N;
  const int NN = NF * N;
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= B * NF * nv) return;
  const int v = (int)(idx % nv);
  const int f = (int)((idx / nv) % NF);
  const int64_t b = idx / ((int64_t)nv * NF);
  const int o = (int)ori[b] - 1, sd = (int)side[b];
  const int64_t e = nid[b] - 1;
  const double in = u[(e * NN + node_of(dim, N, o, sd == 1 ? N - 1 : 0, f)) * nv + v];
  bu[2 * idx + 0] = sd == 1 ? in : 0.0;
  bu[2 * idx + 1] = sd == 2 ? in : 0.0;
}

// boundary_flux_kernel! (dg_2d_kernel.jl:1067-1110) for Dirichlet boundaries:
// the surface flux between the inner trace and the boundary function's state
// at the face node, the inner state on the left when the boundary is the
// element's upper face (directions 2, 4, 6)
template <int DIM, int EQ>
__global__ void boundary_flux_kernel(int N, int64_t B, const double *__restrict__ bu,
                                     const double *__restrict__ coords, const int64_t *__restrict__ nid,
                                     const int64_t *__restrict__ side, const int64_t *__restrict__ ori, double t,
                                     int bc_kind, IcParams bc, int kind, PhysParams<double> pp,
                                     double *__restrict__ sfv) {
  constexpr int NV = NVarsOf<DIM, EQ>::value;
  const int NF = (DIM == 1) ? 1 : (DIM == 2 ? N : N * N);
  const int NN = NF * N;
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= B * NF) return;
  const int f = (int)(idx % NF);
  const int64_t b = idx / NF;
  const int o = (int)ori[b] - 1, sd = (int)side[b];
  const int64_t e = nid[b] - 1;
  double ui[NV], wi[NV], ub[NV], wb[NV], fs[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) ui[v] = bu[2 * ((b * NF + f) * NV + v) + (sd - 1)];
  eval_ic<DIM, EQ>(bc_kind, coords + (e * NN + node_of(DIM, N, o, sd == 1 ? N - 1 : 0, f)) * DIM, t, bc, ub);
  Physics<DIM, EQ, double>::prim(ui, wi, pp);
  Physics<DIM, EQ, double>::prim(ub, wb, pp);
  if (sd == 1)
    flux_dispatch<DIM, EQ, double>(kind, o, ui, wi, ub, wb, fs, pp);
  else
    flux_dispatch<DIM, EQ, double>(kind, o, ub, wb, ui, wi, fs, pp);
  // nonconservative terms: the element's side, 0.5 Phi(u_inner, u_boundary), as
  // at interfaces (the argument order Trixi.jl's boundary condition uses for
  // them is not part of the reference repository)
  add_noncons_rt<DIM, EQ, double>(o, wi, wb, 0.5, fs);
  const int dir = 2 * o + (sd == 1 ? 1 : 0);
#pragma unroll
  for (int v = 0; v < NV; ++v) sfv[v + NV * (f + (int64_t)NF * (dir + 2 * DIM * e))] = fs[v];
}

// calc_sources!: du += source(x, t) at every node (after the Jacobian)
template <int DIM, int EQ>
__global__ void sources_kernel(int N, int64_t E, const double *__restrict__ coords, double t, double c, double A,
                               double L, double gamma, double *__restrict__ du, int kind) {
  constexpr int NV = NVarsOf<DIM, EQ>::value;
  int NN = 1;
  for (int d = 0; d < DIM; ++d) NN *= N;
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= E * NN) return;
  const double prm[3] = {c, A, L};
  double s[NV];
  source_convergence<DIM, EQ>(prm, gamma, coords + q * DIM, t, s, kind);
#pragma unroll
  for (int v = 0; v < NV; ++v) du[q * NV + v] += s[v];
}

// surface_flux_kernel! + interface_flux_kernel! (dg_2d_kernel.jl:938-1006)
template <int DIM, int EQ>
__global__ void interface_flux_kernel(int N, int64_t I, const double *__restrict__ iu, const int64_t *__restrict__ nid,
                                      const int64_t *__restrict__ ori, double *__restrict__ sfv, int kind,
                                      PhysParams<double> pp) {
  constexpr int NV = NVarsOf<DIM, EQ>::value;
  const int NF = (DIM == 1) ? 1 : (DIM == 2 ? N : N * N);
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= I * NF) return;
  const int f = (int)(idx % NF);
  const int64_t k = idx / NF;
  const int o = (int)ori[k] - 1;
  double ul[NV], ur[NV], wl[NV], wr[NV], fs[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    ul[v] = iu[2 * ((k * NF + f) * NV + v) + 0];
    ur[v] = iu[2 * ((k * NF + f) * NV + v) + 1];
  }
  Physics<DIM, EQ, double>::prim(ul, wl, pp);
  Physics<DIM, EQ, double>::prim(ur, wr, pp);
  flux_dispatch<DIM, EQ, double>(kind, o, ul, wl, ur, wr, fs, pp);
  const int64_t left = nid[2 * k] - 1, right = nid[2 * k + 1] - 1;
  // nonconservative terms: left adds 0.5 Phi(u_ll, u_rr), right 0.5 Phi(u_rr, u_ll)
  // (surface_noncons_flux_kernel! + interface_flux_kernel!, dg_2d_kernel.jl:958-1035)
  double fr[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) fr[v] = fs[v];
  add_noncons_rt<DIM, EQ, double>(o, wl, wr, 0.5, fs);
  add_noncons_rt<DIM, EQ, double>(o, wr, wl, 0.5, fr);
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    sfv[v + NV * (f + (int64_t)NF * ((2 * o + 1) + 2 * DIM * left))] = fs[v];
    sfv[v + NV * (f + (int64_t)NF * ((2 * o) + 2 * DIM * right))] = fr[v];
  }
}

// prolong_mortars_small2small_kernel! + prolong_mortars_large2small_kernel!
// (dg_2d_kernel.jl:1167-1259, dg_3d_kernel.jl:1361-1500)
struct MortarArrays {
  double *a[4];
};
__global__ void prolong_mortars_kernel(int dim, int N, int nv, int64_t M, const double *__restrict__ u,
                                       const int64_t *__restrict__ nid, const int64_t *__restrict__ ls_,
                                       const int64_t *__restrict__ ori, MortarArrays arr, Mats mats) {
  const int NC = 1 << (dim - 1);
  const int NF = (dim == 2) ? N : N * N;
  const int NN = NF * N;
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= M * NC * NF * nv) return;
  const int v = (int)(idx % nv);
  const int f = (int)((idx / nv) % NF);
  const int c = (int)((idx / ((int64_t)nv * NF)) % NC);
  const int64_t m = idx / ((int64_t)nv * NF * NC);
  const int o = (int)ori[m] - 1;
  const int ls = (int)ls_[m];
  const int64_t large = nid[NC + (NC + 1) * m] - 1;
  const int64_t small = nid[c + (NC + 1) * m] - 1;
  const int small_side = (ls == 1) ? 1 : 0;
  const int small_a = (ls == 1) ? 0 : N - 1;
  const int large_a = (ls == 1) ? N - 1 : 0;
  double s = 0.0;
  if (dim == 2) {
    const double *F = (c == 1) ? mats.fwd_up : mats.fwd_lo;
    for (int jj = 0; jj < N; ++jj) s += F[f * N + jj] * u[(large * NN + node_of(dim, N, o, large_a, jj)) * nv + v];
  } else {
    const double *F1 = (c & 1) ? mats.fwd_up : mats.fwd_lo;
    const double *F2 = (c >> 1) ? mats.fwd_up : mats.fwd_lo;
    const int fa = f % N, fb = f / N;
    for (int jb = 0; jb < N; ++jb) {
      double t = 0.0;
      for (int ja = 0; ja < N; ++ja) t += F1[fa * N + ja] * u[(large * NN + node_of(dim, N, o, large_a, ja + N * jb)) * nv + v];
      s += F2[fb * N + jb] * t;
    }
  }
  double *dst = arr.a[c];
  const int64_t j = (m * NF + f) * nv + v;
  dst[2 * j + small_side] = u[(small * NN + node_of(dim, N, o, small_a, f)) * nv + v];
  dst[2 * j + (1 - small_side)] = s;
}

// mortar_flux_kernel! + mortar_flux_copy_to_kernel! (dg_2d_kernel.jl:1262-1397,
// dg_3d_kernel.jl:1503-1770): one block per mortar.
template <int DIM, int EQ>
__global__ void mortar_flux_stage_kernel(int N, int64_t M, MortarArrays arr, const int64_t *__restrict__ nid,
                                         const int64_t *__restrict__ ls_, const int64_t *__restrict__ ori,
                                         double *__restrict__ sfv, int kind, PhysParams<double> pp, Mats mats) {
  constexpr int NV = NVarsOf<DIM, EQ>::value;
  constexpr int NC = 1 << (DIM - 1);
  extern __shared__ __align__(16) double sm[];
  const int NF = (DIM == 2) ? N : N * N;
  const int64_t m = blockIdx.x;
  if (m >= M) return;
  const int o = (int)ori[m] - 1;
  const int ls = (int)ls_[m];
  const int small_dir = 2 * o + (ls - 1);
  const int large_dir = 2 * o + (ls == 1 ? 1 : 0);
  const int64_t large = nid[NC + (NC + 1) * m] - 1;
  for (int i = threadIdx.x; i < NC * NF; i += blockDim.x) {
    const int c = i / NF, f = i - c * NF;
    double ul[NV], ur[NV], wl[NV], wr[NV], fs[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const int64_t j = (m * NF + f) * NV + v;
      ul[v] = arr.a[c][2 * j + 0];
      ur[v] = arr.a[c][2 * j + 1];
    }
    Physics<DIM, EQ, double>::prim(ul, wl, pp);
    Physics<DIM, EQ, double>::prim(ur, wr, pp);
    flux_dispatch<DIM, EQ, double>(kind, o, ul, wl, ur, wr, fs, pp);
    const int64_t small = nid[c + (NC + 1) * m] - 1;
    // nonconservative terms: primary 0.5 Phi(u_large, u_small) to the small
    // element, secondary 0.5 Phi(u_small, u_large) projected to the large one
    double fsec[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) fsec[v] = fs[v];
    if constexpr (EQ == EQ_MHD) {
      const double *w_large = (ls == 1) ? wl : wr, *w_small = (ls == 1) ? wr : wl;
      add_noncons_rt<DIM, EQ, double>(o, w_large, w_small, 0.5, fs);
      add_noncons_rt<DIM, EQ, double>(o, w_small, w_large, 0.5, fsec);
    }
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      sm[(c * NF + f) * NV + v] = fsec[v];
      sfv[v + NV * (f + (int64_t)NF * (small_dir + 2 * DIM * small))] = fs[v];
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < NF * NV; i += blockDim.x) {
    const int f = i / NV, v = i - (i / NV) * NV;
    double s = 0.0;
    if (DIM == 2) {
      for (int c = 0; c < NC; ++c) {
        const double *Rm = (c == 1) ? mats.rev_up : mats.rev_lo;
        for (int jj = 0; jj < N; ++jj) s += Rm[f * N + jj] * sm[(c * NF + jj) * NV + v];
      }
    } else {
      const int fa = f % N, fb = f / N;
      for (int c = 0; c < NC; ++c) {
        const double *R1 = (c & 1) ? mats.rev_up : mats.rev_lo;
        const double *R2 = (c >> 1) ? mats.rev_up : mats.rev_lo;
        for (int jb = 0; jb < N; ++jb) {
          double t = 0.0;
          for (int ja = 0; ja < N; ++ja) t += R1[fa * N + ja] * sm[(c * NF + ja + N * jb) * NV + v];
          s += R2[fb * N + jb] * t;
        }
      }
    }
    sfv[v + NV * (f + (int64_t)NF * (large_dir + 2 * DIM * large))] = s;
  }
}

// surface_integral_kernel! (dg_2d_kernel.jl:1400-1421, dg_3d_kernel.jl:1773-1799)
__global__ void surface_integral_kernel(int dim, int N, int nv, int64_t E, double *__restrict__ du,
                                        const double *__restrict__ sfv, double factor1, double factor2) {
  int NF = 1;
  for (int d = 1; d < dim; ++d) NF *= N;
  const int NN = NF * N;
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= E * NN * nv) return;
  const int v = (int)(idx % nv);
  const int n = (int)((idx / nv) % NN);
  const int64_t e = idx / ((int64_t)nv * NN);
  double neg = 0.0, pos = 0.0;
  bool on_face = false;
  int r = n;
  int coords[3] = {0, 0, 0};
  for (int d = 0; d < dim; ++d) { coords[d] = r % N; r /= N; }
  for (int d = 0; d < dim; ++d) {
    const int c = coords[d];
    if (c != 0 && c != N - 1) continue;
    on_face = true;
    int f = 0, s = 1;
    for (int dd = 0; dd < dim; ++dd) {
      if (dd == d) continue;
      f += coords[dd] * s;
      s *= N;
    }
    if (c == 0) neg += sfv[v + nv * (f + (int64_t)NF * (2 * d + 2 * dim * e))];
    if (c == N - 1) pos += sfv[v + nv * (f + (int64_t)NF * (2 * d + 1 + 2 * dim * e))];
  }
  if (!on_face) return;
  du[idx] -= neg * factor1;
  du[idx] += pos * factor2;
}

// jacobian_kernel! (dg_2d_kernel.jl:1424-1437)
__global__ void jacobian_kernel(int64_t per, int64_t E, double *__restrict__ du, const double *__restrict__ inv_jac) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= E * per) return;
  du[idx] *= -inv_jac[idx / per];
}

static Mats mats_of(const StageHost &sh) {
  Mats m;
  std::copy(sh.fwd_up, sh.fwd_up + HOST_NMAX * HOST_NMAX, m.fwd_up);
  std::copy(sh.fwd_lo, sh.fwd_lo + HOST_NMAX * HOST_NMAX, m.fwd_lo);
  std::copy(sh.rev_up, sh.rev_up + HOST_NMAX * HOST_NMAX, m.rev_up);
  std::copy(sh.rev_lo, sh.rev_lo + HOST_NMAX * HOST_NMAX, m.rev_lo);
  return m;
}

static inline unsigned blocks_for(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

cudaError_t stage_prolong2interfaces(const StageHost &sh, const double *u, cudaStream_t s) {
  int NF = 1;
  for (int d = 1; d < sh.dim; ++d) NF *= sh.N;
  const int64_t n = sh.ninterfaces * NF * sh.nv;
  if (n == 0) return cudaSuccess;
  prolong_interfaces_kernel<<<blocks_for(n, 256), 256, 0, s>>>(sh.dim, sh.N, sh.nv, sh.ninterfaces, u,
                                                             sh.if_neighbor_ids, sh.if_orientations, sh.interfaces_u);
  return cudaGetLastError();
}

template <int DIM, int EQ>
static cudaError_t launch_iflux(const StageHost &sh, cudaStream_t s) {
  const int NF = (DIM == 1) ? 1 : (DIM == 2 ? sh.N : sh.N * sh.N);
  const int64_t n = sh.ninterfaces * NF;
  if (n == 0) return cudaSuccess;
  interface_flux_kernel<DIM, EQ><<<blocks_for(n, 128), 128, 0, s>>>(sh.N, sh.ninterfaces, sh.interfaces_u,
                                                                   sh.if_neighbor_ids, sh.if_orientations, sh.sfv,
                                                                   sh.surface_flux, make_pp<double>(sh.gamma, sh.adv, sh.c_h));
  return cudaGetLastError();
}

cudaError_t stage_interface_flux(const StageHost &sh, cudaStream_t s) {
  const bool adv = sh.eq == EQ_ADV;
  if (sh.eq == EQ_MHD) {
    switch (sh.dim) {
      case 1: return launch_iflux<1, EQ_MHD>(sh, s);
      case 2: return launch_iflux<2, EQ_MHD>(sh, s);
      case 3: return launch_iflux<3, EQ_MHD>(sh, s);
    }
    return cudaErrorNotSupported;
  }
  switch (sh.dim) {
    case 1: return adv ? launch_iflux<1, EQ_ADV>(sh, s) : launch_iflux<1, EQ_EULER>(sh, s);
    case 2: return adv ? launch_iflux<2, EQ_ADV>(sh, s) : launch_iflux<2, EQ_EULER>(sh, s);
    case 3: return adv ? launch_iflux<3, EQ_ADV>(sh, s) : launch_iflux<3, EQ_EULER>(sh, s);
  }
  return cudaErrorNotSupported;
}

cudaError_t stage_prolong2boundaries(const StageHost &sh, const double *u, cudaStream_t s) {
  if (sh.nboundaries == 0) return cudaSuccess;
  const int NF = (sh.dim == 1) ? 1 : (sh.dim == 2 ? sh.N : sh.N * sh.N);
  const int64_t n = sh.nboundaries * NF * sh.nv;
  prolong_boundaries_kernel<<<blocks_for(n, 256), 256, 0, s>>>(sh.dim, sh.N, sh.nv, sh.nboundaries, u,
                                                             sh.bnd_neighbor_ids, sh.bnd_sides, sh.bnd_orientations,
                                                             sh.boundaries_u);
  return cudaGetLastError();
}

template <int DIM, int EQ>
static cudaError_t launch_bflux(const StageHost &sh, double t, cudaStream_t s) {
  const int NF = (DIM == 1) ? 1 : (DIM == 2 ? sh.N : sh.N * sh.N);
  const int64_t n = sh.nboundaries * NF;
  boundary_flux_kernel<DIM, EQ><<<blocks_for(n, 128), 128, 0, s>>>(
      sh.N, sh.nboundaries, sh.boundaries_u, sh.coords, sh.bnd_neighbor_ids, sh.bnd_sides, sh.bnd_orientations, t,
      sh.bc_kind, sh.bc, sh.surface_flux, make_pp<double>(sh.gamma, sh.adv, sh.c_h), sh.sfv);
  return cudaGetLastError();
}

cudaError_t stage_boundary_flux(const StageHost &sh, double t, cudaStream_t s) {
  if (sh.nboundaries == 0) return cudaSuccess;
  if (sh.eq == EQ_MHD) {
    switch (sh.dim) {
      case 1: return launch_bflux<1, EQ_MHD>(sh, t, s);
      case 2: return launch_bflux<2, EQ_MHD>(sh, t, s);
      case 3: return launch_bflux<3, EQ_MHD>(sh, t, s);
    }
    return cudaErrorNotSupported;
  }
  const bool adv = sh.eq == EQ_ADV;
  switch (sh.dim) {
    case 1: return adv ? launch_bflux<1, EQ_ADV>(sh, t, s) : launch_bflux<1, EQ_EULER>(sh, t, s);
    case 2: return adv ? launch_bflux<2, EQ_ADV>(sh, t, s) : launch_bflux<2, EQ_EULER>(sh, t, s);
    case 3: return adv ? launch_bflux<3, EQ_ADV>(sh, t, s) : launch_bflux<3, EQ_EULER>(sh, t, s);
  }
  return cudaErrorNotSupported;
}

cudaError_t stage_sources(const StageHost &sh, double *du, double t, cudaStream_t s) {
  if (sh.src_kind == SRC_NONE || sh.eq != EQ_EULER) return cudaSuccess;
  int NN = 1;
  for (int d = 0; d < sh.dim; ++d) NN *= sh.N;
  const int64_t n = sh.nelements * NN;
  switch (sh.dim) {
    case 1:
      sources_kernel<1, EQ_EULER><<<blocks_for(n, 256), 256, 0, s>>>(sh.N, sh.nelements, sh.coords, t, sh.src[0],
                                                                     sh.src[1], sh.src[2], sh.gamma, du, sh.src_kind);
      break;
    case 2:
      sources_kernel<2, EQ_EULER><<<blocks_for(n, 256), 256, 0, s>>>(sh.N, sh.nelements, sh.coords, t, sh.src[0],
                                                                     sh.src[1], sh.src[2], sh.gamma, du, sh.src_kind);
      break;
    default:
      sources_kernel<3, EQ_EULER><<<blocks_for(n, 256), 256, 0, s>>>(sh.N, sh.nelements, sh.coords, t, sh.src[0],
                                                                     sh.src[1], sh.src[2], sh.gamma, du, sh.src_kind);
  }
  return cudaGetLastError();
}

cudaError_t stage_prolong2mortars(const StageHost &sh, const double *u, cudaStream_t s) {
  if (sh.nmortars == 0 || sh.dim < 2) return cudaSuccess;
  const int NC = 1 << (sh.dim - 1);
  const int NF = (sh.dim == 2) ? sh.N : sh.N * sh.N;
  const int64_t n = sh.nmortars * NC * NF * sh.nv;
  MortarArrays arr;
  for (int c = 0; c < 4; ++c) arr.a[c] = sh.mortar_u[c];
  prolong_mortars_kernel<<<blocks_for(n, 256), 256, 0, s>>>(sh.dim, sh.N, sh.nv, sh.nmortars, u, sh.mo_neighbor_ids,
                                                          sh.mo_large_sides, sh.mo_orientations, arr, mats_of(sh));
  return cudaGetLastError();
}

template <int DIM, int EQ>
static cudaError_t launch_mflux(const StageHost &sh, cudaStream_t s) {
  constexpr int NV = NVarsOf<DIM, EQ>::value;
  constexpr int NC = 1 << (DIM - 1);
  const int NF = (DIM == 2) ? sh.N : sh.N * sh.N;
  MortarArrays arr;
  for (int c = 0; c < 4; ++c) arr.a[c] = sh.mortar_u[c];
  const size_t smem = sizeof(double) * (size_t)NC * NF * NV;
  mortar_flux_stage_kernel<DIM, EQ><<<(unsigned)sh.nmortars, 128, smem, s>>>(
      sh.N, sh.nmortars, arr, sh.mo_neighbor_ids, sh.mo_large_sides, sh.mo_orientations, sh.sfv, sh.surface_flux,
      make_pp<double>(sh.gamma, sh.adv, sh.c_h), mats_of(sh));
  return cudaGetLastError();
}

cudaError_t stage_mortar_flux(const StageHost &sh, cudaStream_t s) {
  if (sh.nmortars == 0 || sh.dim < 2) return cudaSuccess;
  if (sh.eq == EQ_MHD) return sh.dim == 2 ? launch_mflux<2, EQ_MHD>(sh, s) : launch_mflux<3, EQ_MHD>(sh, s);
  const bool adv = sh.eq == EQ_ADV;
  if (sh.dim == 2) return adv ? launch_mflux<2, EQ_ADV>(sh, s) : launch_mflux<2, EQ_EULER>(sh, s);
  return adv ? launch_mflux<3, EQ_ADV>(sh, s) : launch_mflux<3, EQ_EULER>(sh, s);
}

cudaError_t stage_surface_integral(const StageHost &sh, double *du, cudaStream_t s) {
  int NN = sh.N;
  for (int d = 1; d < sh.dim; ++d) NN *= sh.N;
  const int64_t n = sh.nelements * NN * sh.nv;
  if (n == 0) return cudaSuccess;
  surface_integral_kernel<<<blocks_for(n, 256), 256, 0, s>>>(sh.dim, sh.N, sh.nv, sh.nelements, du, sh.sfv,
                                                           sh.lhat_l, sh.lhat_r);
  return cudaGetLastError();
}

cudaError_t stage_jacobian(const StageHost &sh, double *du, cudaStream_t s) {
  int NN = sh.N;
  for (int d = 1; d < sh.dim; ++d) NN *= sh.N;
  const int64_t per = (int64_t)NN * sh.nv;
  const int64_t n = sh.nelements * per;
  if (n == 0) return cudaSuccess;
  jacobian_kernel<<<blocks_for(n, 256), 256, 0, s>>>(per, sh.nelements, du, sh.inv_jac);
  return cudaGetLastError();
}

}  // namespace trixi
