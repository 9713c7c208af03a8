// dg_fused.cuh -- the fused TreeMesh DGSEM right-hand-side kernel.
//
// One launch computes, for a tile of `epb` consecutive elements,
//   volume integral  (weak form, flux differencing, or the DG-FV blend of
//                     shock capturing)           reference: dg_2d_kernel.jl:55-105, 164-225, 496-606
//   interface/mortar surface fluxes              reference: dg_2d_kernel.jl:907-1006, 1262-1397
//   surface integral                             reference: dg_2d_kernel.jl:1400-1421
//   apply_jacobian                               reference: dg_2d_kernel.jl:1424-1437
//   and optionally the 2N low-storage RK stage update (OrdinaryDiffEq's
//   CarpenterKennedy2N54 broadcast, outside the reference).
//
// Work decomposition.  A block holds GPB independent groups; a group of WPG
// warps owns EPG consecutive elements (chosen at compile time so that each
// warp's flux items fall in one direction/section) and synchronises only
// among itself.  Phase A: one owner thread per node loads its u (and k) into
// registers and stores the node's conservative and primitive variables, in
// the compute precision, as a record in shared memory; all threads of the
// group stage the neighbours' face nodes.  Phase B: one thread per two-point
// flux evaluates every flux the group needs, each exactly once per element:
// the symmetric volume fluxes f#(u_i, u_m), i < m, on every line (N(N-1)/2
// per line instead of the reference's N^2), the surface fluxes on the
// element's 2*ndims faces (the neighbour's adjacent node is read straight
// from u -- "owner computes", no interfaces.u or surface_flux_values round
// trip through HBM; mortar faces read the flux prepared by the mortar
// kernel), and for shock capturing the LGL subcell FV fluxes.  Phase C: the
// owner thread sums D_split / D_hat times the staged fluxes along each
// dimension, adds the surface terms, scales by -J^{-1}, and stores du or
// performs the RK update, in the reference layout.
//
// FP32-mixed variants of this plan (each measured; see the constants below):
// the volume fluxes are not phase-B items but "owner pairs" (the owner thread
// evaluates its partner fluxes into registers, packed two per FP32
// instruction stream for Euler flux_ranocha); the surface fluxes overwrite
// their trace records; inside trixi_rk_steps the flux states and traces come
// from an FP32 copy of the state that the previous stage wrote; in the packed
// 3D kernels u and k travel to shared memory by cp.async during phases A-B
// instead of occupying registers.
#pragma once
#include "dg_convert.cuh"
#include "dg_ic.cuh"
#include "dg_packed.cuh"
#include "dg_physics.cuh"

namespace trixi {

constexpr int NMAXT = 6;  // largest N = polydeg + 1 compiled

template <typename R>
struct FusedParams {
  const double *__restrict__ u_in;          // [E][NN][NV]
  double *__restrict__ out;                 // du (VOLUME/RHS) or u_out (RK)
  double *__restrict__ k;                   // RK register (RK)
  const int32_t *__restrict__ face_table;   // [E][2*DIM]: >=0 neighbour element, <0: -(slot+1)
  const double *__restrict__ mortar_flux;   // [slot][NF][NV]
  const double *__restrict__ inv_jac;       // [E]
  const double *__restrict__ alpha;         // [E] (shock capturing)
  const double *__restrict__ dt_elem;       // [E] per-element time step (batched ensembles) or null
  int *err;                                 // device error word
  int64_t nelements;
  int mode;
  int surface_flux, fv_flux;
  double rk_a, rk_b, dt;
  int use_k;                                // RK: read k (rk_a != 0)
  int wpg, gpb;                             // tile: warps per group, groups per block
  int pdl;                                  // launched as a programmatic dependent launch
  // non-periodic meshes and source terms
  const double *__restrict__ coords;        // [E][NN][DIM] node coordinates (boundaries / sources)
  double t;                                 // time of this rhs evaluation
  int bc_kind;                              // Dirichlet boundary function (IC_* kind)
  int src_kind;                             // SRC_*
  IcParams bc;                              // its parameters
  double src[3];                            // (c, A, L) of the convergence-test source
  int vec16;                                // u_in, out, k, mortar_flux 16-byte aligned
  double atol;                              // dg-only test for alpha
  // FP32-mixed RK stages inside trixi_rk_steps: the previous stage's output
  // narrowed to FP32 (round to nearest even, the narrowing phase A applies to
  // u_in), read in place of u_in for the flux states, and this stage's output
  // narrowed the same way for the next stage; null when absent
  const float *__restrict__ u32_in;         // [E][NN][NV]
  float *__restrict__ u32_out;              // [E][NN][NV]
  PhysParams<R> pp;
  R dsplit[NMAXT * NMAXT];                  // row-major [i][m], diagonal zeroed
  R dhat[NMAXT * NMAXT];                    // row-major [i][m]
  R invw[NMAXT];
  R lhat_l, lhat_r;                         // 1/w_1, 1/w_N (boundary_interpolation)
};

// Node index of the point at position a along orientation O on line t (the
// face index of the line: remaining coordinates in increasing order).
template <int DIM, int N, int O>
__device__ __forceinline__ int line_node(int t, int a) {
  if constexpr (DIM == 1) {
    return a;
  } else if constexpr (DIM == 2) {
    return (O == 0) ? a + t * N : t + a * N;
  } else {
    const int t1 = t % N, t2 = t / N;
    if constexpr (O == 0) return a + t1 * N + t2 * N * N;
    else if constexpr (O == 1) return t1 + a * N + t2 * N * N;
    else return t1 + t2 * N + a * N * N;
  }
}

template <int DIM, int N>
__device__ __forceinline__ int line_node_rt(int o, int t, int a) {
  if constexpr (DIM == 1) {
    return a;
  } else if constexpr (DIM == 2) {
    return (o == 0) ? a + t * N : t + a * N;
  } else {
    const int t1 = t % N, t2 = t / N;
    return (o == 0) ? a + t1 * N + t2 * N * N : (o == 1) ? t1 + a * N + t2 * N * N : t1 + t2 * N + a * N * N;
  }
}

// index of the pair (a, b), a != b, among the N(N-1)/2 pairs of a line
template <int N>
__device__ __forceinline__ int pair_index(int a, int b) {
  const int lo = a < b ? a : b, hi = a < b ? b : a;
  return lo * (2 * N - lo - 1) / 2 + (hi - lo - 1);
}

// (i, m) of pair p, packed 4 bits per pair into one 64-bit constant each
template <int N>
struct PairBits {
  static constexpr unsigned long long pack(bool second) {
    unsigned long long bits = 0;
    int p = 0;
    for (int a = 0; a < N; ++a)
      for (int b = a + 1; b < N; ++b, ++p) bits |= (unsigned long long)(second ? b : a) << (4 * p);
    return bits;
  }
  static constexpr unsigned long long I = pack(false);
  static constexpr unsigned long long M = pack(true);
};

template <int N>
__device__ __forceinline__ void pair_nodes(int p, int &i, int &m) {
  i = (int)((PairBits<N>::I >> (4 * p)) & 0xfull);
  m = (int)((PairBits<N>::M >> (4 * p)) & 0xfull);
}

// Node records of NV values in shared memory: one 16-byte (float) or two
// 16-byte (double) accesses when NV == 4, scalar accesses otherwise.
template <int NV, typename R>
__device__ __forceinline__ void lds_rec(const R *src, R *dst) {
  if constexpr (NV == 4 && sizeof(R) == 4) {
    const float4 t = *reinterpret_cast<const float4 *>(src);
    dst[0] = t.x;
    dst[1] = t.y;
    dst[2] = t.z;
    dst[3] = t.w;
  } else if constexpr (NV == 4 && sizeof(R) == 8) {
    const double2 a = reinterpret_cast<const double2 *>(src)[0], b = reinterpret_cast<const double2 *>(src)[1];
    dst[0] = a.x;
    dst[1] = a.y;
    dst[2] = b.x;
    dst[3] = b.y;
  } else {
#pragma unroll
    for (int v = 0; v < NV; ++v) dst[v] = src[v];
  }
}
template <int NV, typename R>
__device__ __forceinline__ void sts_rec(R *dst, const R *src) {
  if constexpr (NV == 4 && sizeof(R) == 4) {
    *reinterpret_cast<float4 *>(dst) = make_float4(src[0], src[1], src[2], src[3]);
  } else if constexpr (NV == 4 && sizeof(R) == 8) {
    reinterpret_cast<double2 *>(dst)[0] = make_double2(src[0], src[1]);
    reinterpret_cast<double2 *>(dst)[1] = make_double2(src[2], src[3]);
  } else {
#pragma unroll
    for (int v = 0; v < NV; ++v) dst[v] = src[v];
  }
}
// The NV doubles of one node in global memory: two 16-byte accesses when
// NV == 4 and the arrays are 16-byte aligned (vec), scalar accesses otherwise.
template <int NV>
__device__ __forceinline__ void ldg_node(const double *src, double *dst, bool vec) {
  if constexpr (NV == 4) {
    if (vec) {
      const double2 a = __ldg(reinterpret_cast<const double2 *>(src));
      const double2 b = __ldg(reinterpret_cast<const double2 *>(src) + 1);
      dst[0] = a.x;
      dst[1] = a.y;
      dst[2] = b.x;
      dst[3] = b.y;
      return;
    }
  }
#pragma unroll
  for (int v = 0; v < NV; ++v) dst[v] = src[v];
}
template <int NV>
__device__ __forceinline__ void stg_node(double *dst, const double *src, bool vec) {
  if constexpr (NV == 4) {
    if (vec) {
      reinterpret_cast<double2 *>(dst)[0] = make_double2(src[0], src[1]);
      reinterpret_cast<double2 *>(dst)[1] = make_double2(src[2], src[3]);
      return;
    }
  }
#pragma unroll
  for (int v = 0; v < NV; ++v) dst[v] = src[v];
}

// The NV floats of one node record of an FP32 state copy (16-byte records
// when NV == 4: the copies are allocated by the library).
template <int NV>
__device__ __forceinline__ void ldg_rec32(const float *src, float *dst) {
  if constexpr (NV == 4) {
    const float4 t = __ldg(reinterpret_cast<const float4 *>(src));
    dst[0] = t.x;
    dst[1] = t.y;
    dst[2] = t.z;
    dst[3] = t.w;
  } else {
#pragma unroll
    for (int v = 0; v < NV; ++v) dst[v] = __ldg(src + v);
  }
}
template <int NV>
__device__ __forceinline__ void stg_rec32(float *dst, const float *src) {
  if constexpr (NV == 4) {
    *reinterpret_cast<float4 *>(dst) = make_float4(src[0], src[1], src[2], src[3]);
  } else {
#pragma unroll
    for (int v = 0; v < NV; ++v) dst[v] = src[v];
  }
}

constexpr int round_up4(int x) { return (x + 3) & ~3; }

// Asynchronous global -> shared copies (cp.async): the copy needs no
// registers while in flight; cp.async.wait_all makes the executing thread's
// copies complete, a barrier after it makes them visible to the group.
__device__ __forceinline__ void cp_async16(void *dst_smem, const void *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void *dst_smem, const void *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }



// BND = 1: the instantiation for non-periodic meshes and source terms (the
// Dirichlet states of boundary faces in phase A, the source in phase C);
// BND = 0 carries none of that code, so the periodic kernels keep their
// registers.
template <int DIM, int N, int EQ, typename R, int VOL, int VFLUX, int BND = 0>
struct FusedKernel {
  using P = Physics<DIM, EQ, R>;
  static constexpr int NV = P::NV;
  // the HLL family (flux_hll, flux_hlle) as surface / FV flux: in the
  // instantiations with boundary support, and in the flux_shima_etal ones
  // (which have no such twin); left out of the other periodic kernels, whose
  // code it grows by a fifth
  static constexpr int HLL_FAMILY = (BND || VFLUX == FLUX_SHIMA) ? 1 : 0;
  // the entropy-conservative flux (flux_ranocha) as the surface or FV flux
  // of the periodic Euler / advection shock-capturing kernels: likewise left
  // out (a quarter of their code; the reference's shock-capturing set-ups
  // take flux_lax_friedrichs there) and served by the boundary-capable twins
  static constexpr int SC_EC = (HLL_FAMILY || EQ == EQ_MHD || VOL != VOL_SC) ? 1 : 0;
  // nonconservative terms (ideal GLM-MHD in 2D/3D: Powell + GLM transport)
  static constexpr bool NC = (EQ == EQ_MHD && DIM > 1);
  // FV subcell fluxes per interface: one, or with nonconservative terms one
  // per side (fstar_L / fstar_R of src/solvers/dg_2d_kernel.jl:609-707)
  static constexpr int FV_RECS = NC ? 2 : 1;
  // largest block: 16 warps, 8 for the register-heavy MHD kernels
  static constexpr int MAX_WARPS = (EQ == EQ_MHD) ? 8 : 16;
  // double -> compute type of phase A: the FP64 pipe's conversion (hw) or the
  // integer-pipe rounding of dg_convert.cuh; both round to nearest even, so
  // the results are identical.  Splitting the work between the two pipes
  // measured best: the neighbour traces on the FP64 pipe everywhere (3D FP32
  // stage kernels 3.5-5 % faster, 2D unchanged), the owners' states too in 3D
  // (a further 2-3 %; in 2D that costs 6 %).
  static constexpr bool HW_TRACE = true;
  static constexpr bool HW_OWNER = (DIM == 3);
  // the FP32 copy of an RK stage's output (u32_out): narrowed on the integer
  // pipe (measured A/B: 2D Euler step 66.1 -> 65.2 us against the FP64
  // pipe; 3D shock capturing unchanged)
  static constexpr bool HW_OUT = false;
  template <bool HW>
  __device__ __forceinline__ static R narrow(double x) {
    if constexpr (HW) return R(x);
    else return from_double<R>(x);
  }
  static constexpr int NN = ipow(N, DIM);
  static constexpr int NF = ipow(N, DIM - 1);
  static constexpr int NP = N * (N - 1) / 2;
  // staged fluxes per element and direction
  // Linear advection: its volume fluxes (a_d u, and the central pair flux
  // a_d {{u}}) cost a multiply, so phase C forms them from the node records
  // and phase B stages none -- in the weak form, and in flux differencing in
  // FP32 (measured: 3D N=4 FP32 78 -> 53 us; in FP64 the staged pairs were
  // 10 % faster).  The other systems stage one flux per node and direction
  // (weak form) or per pair (flux differencing).
  static constexpr bool LINEAR = (EQ == EQ_ADV) && (VOL == VOL_WEAK || sizeof(R) == 4);
  // Flux differencing in FP32 ("owner pairs"): the thread that owns node i
  // evaluates f#(u_i, u_m) for its N-1 line partners in every direction and
  // sums D_split[i,m] f# straight into its registers -- twice the flux
  // arithmetic of the symmetric pairs, but no pair decoding, no pair staging
  // in shared memory and no gather in phase C.  The FP32 kernels are bound by
  // instruction issue, where the pair bookkeeping cost more than the second
  // evaluation (measured: integer instructions were 42 % of the 2D Euler
  // stage kernel's, FP32 arithmetic 20 %).  FP64 keeps the symmetric pairs:
  // it is bound by GB300's FP64 pipe, where the flux arithmetic is the cost.
  static constexpr bool OWNER_PAIRS = (VOL != VOL_WEAK) && !LINEAR && sizeof(R) == 4;
  // Euler flux_ranocha in FP32: the owner's DIM (N-1) partner fluxes, taken
  // two at a time in the halves of float2 registers (ranocha_x2, packed FP32
  // instructions); partner J of the flattened list is k = 1 + J % (N-1)
  // steps along direction J / (N-1).  Measured on the 2D Euler level-7
  // stage kernel: FP32 instructions -36 %, all instructions -7 % (the pairs
  // cost register moves), 18.35 -> 17.41 us per launch.  2D up to N = 4
  // (the higher-N kernels spill at their register caps with it); 3D for
  // N = 4 without boundary support, and only with u and k staged in shared
  // memory (UK_SMEM below) -- the other 3D kernels still spill with it.
  static constexpr bool PACKED = OWNER_PAIRS && EQ == EQ_EULER && VFLUX == FLUX_RANOCHA &&
                                 ((DIM == 2 && N <= 4) || (DIM == 3 && N == 4 && !BND));
  static constexpr int VOL_PER_DIR = (LINEAR || OWNER_PAIRS) ? 0 : (VOL == VOL_WEAK) ? NN : NF * NP;
  static constexpr int SURF_PER_EL = 2 * DIM * NF;
  static constexpr int FV_PER_DIR = (VOL == VOL_SC) ? NF * (N - 1) : 0;
  static constexpr int ITEMS_PER_EL = DIM * VOL_PER_DIR + SURF_PER_EL + DIM * FV_PER_DIR;
  static constexpr int TRACE_PER_EL = 2 * DIM * NF * NV;  // neighbour face nodes (or mortar fluxes)
  // Thread mapping: one owner thread per node.  A group of WPG warps owns EPG
  // elements and synchronises only among itself (__syncwarp or a named
  // barrier), never block-wide, so groups of a block drift apart and hide
  // each other's latency.
  static constexpr int TPE = NN;  // owner threads per element
  // shared memory of one group of `epg` elements (every array 16-byte aligned)
  static constexpr int n_cons(int epg) { return round_up4(epg * NN * NV); }
  static constexpr int n_vol(int epg) { return round_up4(epg * DIM * VOL_PER_DIR * NV); }
  static constexpr int n_fv(int epg) { return round_up4(epg * DIM * FV_PER_DIR * FV_RECS * NV); }
  static constexpr int n_trace(int epg) { return round_up4(epg * TRACE_PER_EL); }
  static constexpr int n_el(int epg) { return round_up4(epg); }
  static constexpr int N_OPS = round_up4(2 * N * N + N);  // D_split, D_hat, 1/w
  // FP32 RK stages of the packed 3D kernels: the FP64 u and k of the
  // group's nodes are copied into shared memory while phases A and B run
  // (cp.async), so that no thread holds them in registers until phase C.
  // The packed 3D flux_ranocha needs those registers (without the copies it
  // spills at the 64-register cap); measured on the 3D shock-capturing
  // level-5 workload, 1.032 -> 0.990 ms per step.  Without packing the
  // copies cost more than they save (1.070 ms; 2D: 68.2 -> 70.0 us per step).
  static constexpr bool UK_SMEM = PACKED && DIM == 3;
  static constexpr int n_uk(int epg) { return UK_SMEM ? ((epg * NN * NV + 1) & ~1) : 0; }  // doubles
  static constexpr size_t group_smem_core(int epg) {
    // (the surface fluxes overwrite the neighbour traces in place: n_surf is not added)
    return sizeof(R) * (size_t)(2 * n_cons(epg) + n_vol(epg) + n_fv(epg) + n_trace(epg) +
                                2 * n_el(epg) + N_OPS) +
           sizeof(int) * (size_t)round_up4(epg * 2 * DIM);
  }
  static constexpr size_t group_smem(int epg) {
    return group_smem_core(epg) + sizeof(double) * 2 * n_uk(epg);
  }

  static constexpr int warps_for(int epg) { return (epg * TPE + 31) / 32; }
  // Warp passes of phase B for a group of `epg` elements: items are ordered
  // [volume dir 0 | dir 1 | ... | surface dir 0 | ... | FV dir 0 | ...] and a
  // warp executes one pass per section that its 32 items touch.
  static constexpr int phase_b_passes(int epg) {
    int bounds[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    int nb = 0, acc = 0;
    for (int d = 0; d < DIM; ++d) bounds[nb++] = (acc += epg * VOL_PER_DIR);
    for (int d = 0; d < DIM; ++d) bounds[nb++] = (acc += epg * 2 * NF);
    if (FV_PER_DIR > 0)
      for (int d = 0; d < DIM; ++d) bounds[nb++] = (acc += epg * FV_PER_DIR);
    int passes = 0;
    for (int w0 = 0; w0 < acc; w0 += 32) {
      const int w1 = (w0 + 32 < acc) ? w0 + 32 : acc;
      int lo = 0;
      for (int b = 0; b < nb; ++b) {
        if (bounds[b] > lo && lo < w1 && bounds[b] > w0) ++passes;  // section [lo, bounds[b]) meets [w0, w1)
        lo = bounds[b];
      }
    }
    return passes;
  }
  // elements per group: fewest phase-B passes per element, then fewest idle
  // owner lanes, within 8 warps and (beyond one element) 48 KB per group
  static constexpr int epg_pick() {
    int best = 1;
    long best_cost = -1;
    for (int e = 1; e <= 32; e *= 2) {
      if (warps_for(e) > 8) break;
      if (e > 1 && group_smem_core(e) > 48 * 1024) break;
      // cost per element in 1/1000 units: passes plus idle-lane waste of phases A/C
      const long cost = 1000L * phase_b_passes(e) / e + 1000L * (warps_for(e) * 32 - e * TPE) / (32 * e);
      if (best_cost < 0 || cost < best_cost) {
        best = e;
        best_cost = cost;
      }
    }
    return best;
  }
  static constexpr int EPG = epg_pick();  // elements per group
  // Default tile (the tuner may pick others): the warps that own the EPG
  // elements' nodes, and groups up to 8 warps per block within 200 KB of
  // shared memory.  Measured against every valid tile on 14 kernel kinds
  // (2D/3D Euler FD and SC, MHD FD and SC, FP64 and FP32-mixed), this choice
  // is within ~5 % of the fastest; wider groups lost up to 34 %.
  static constexpr int wpg_pick() { return warps_for(EPG); }
  static constexpr int WPG = wpg_pick();
  static constexpr int GT = 32 * WPG;                  // threads per group
  static constexpr int N_CONS = n_cons(EPG);
  static constexpr int N_VOL = n_vol(EPG);
  static constexpr int N_FV = n_fv(EPG);
  static constexpr int N_TRACE = n_trace(EPG);
  static constexpr int N_EL = n_el(EPG);
  static constexpr int N_UK = n_uk(EPG);
  // trace items per thread of phase A at the narrowest group (the owners' warps)
  static constexpr int TR_IT = (EPG * 2 * DIM * NF + 32 * warps_for(EPG) - 1) / (32 * warps_for(EPG));
  static constexpr size_t GROUP_SMEM = group_smem(EPG);
  static constexpr int gpb_pick() {
    int g = 8 / WPG;
    if (g < 1) g = 1;
    while (g > 1 && g * GROUP_SMEM > 200 * 1024) --g;
    return g;
  }
  static constexpr int GPB = gpb_pick();
  static constexpr int BLOCK = GPB * GT;
  static constexpr int EPB = GPB * EPG;  // elements per block
  static_assert(GPB <= 15, "named barrier ids");
  static constexpr size_t smem_for(int) { return GPB * GROUP_SMEM; }
  static size_t smem_bytes() { return smem_for(EPB); }

  struct Smem {
    double *u64, *k64;  // UK_SMEM: the group's u and k, [el][node][v]
    R *cons, *prim, *fvol, *fsurf, *ffv, *trace, *alpha, *scale, *dsplit, *dhat, *invw;
    int *conforming;  // [el][face]: 1 = trace holds the neighbour's node, 0 = a mortar flux
    // node records [el][node][v]
    __device__ __forceinline__ R *c(int el, int n) const { return cons + (el * NN + n) * NV; }
    __device__ __forceinline__ R *w(int el, int n) const { return prim + (el * NN + n) * NV; }
    // record loads and stores (16-byte accesses for 4 variables)
    __device__ __forceinline__ static void ld(const R *base, int q, R *dst) { lds_rec<NV>(base + q * NV, dst); }
    __device__ __forceinline__ static void st(R *base, int q, const R *src) { sts_rec<NV>(base + q * NV, src); }
    __device__ __forceinline__ void ldc(int el, int n, R *dst) const { ld(cons, el * NN + n, dst); }
    __device__ __forceinline__ void ldw(int el, int n, R *dst) const { ld(prim, el * NN + n, dst); }
    __device__ __forceinline__ void stc(int el, int n, const R *src) const { st(cons, el * NN + n, src); }
    __device__ __forceinline__ void stw(int el, int n, const R *src) const { st(prim, el * NN + n, src); }
    // [el][face][t][v]
    __device__ __forceinline__ R *tr(int el, int face, int t) const {
      return trace + ((el * 2 * DIM + face) * NF + t) * NV;
    }
    // [el][dir][slot][v]
    __device__ __forceinline__ R *vol(int el, int d, int slot) const {
      return fvol + ((el * DIM + d) * VOL_PER_DIR + slot) * NV;
    }
    // [el][face][t][v]
    __device__ __forceinline__ R *surf(int el, int face, int t) const {
      return fsurf + ((el * 2 * DIM + face) * NF + t) * NV;
    }
    // [el][dir][t][a][side][v]: side 0 seen from node a (left), 1 from node a+1
    __device__ __forceinline__ R *fv(int el, int d, int t, int a, int side = 0) const {
      return ffv + ((((el * DIM + d) * NF + t) * (N - 1) + a) * FV_RECS + side) * NV;
    }
  };

  // groups of one warp use __syncwarp; larger groups a named barrier (id 1 + gid)
  __device__ __forceinline__ static void group_sync(int gid, int wpg, int gthreads) {
    if (wpg == 1) {
      __syncwarp();
    } else {
      asm volatile("bar.sync %0, %1;" ::"r"(gid + 1), "r"(gthreads) : "memory");
    }
  }

  // volume item: one symmetric pair (FD / SC) or one nodal physical flux (weak form)
  template <int O>
  __device__ __forceinline__ static void volume_item(const FusedParams<R> &p, const Smem &s, int el, int r) {
    R f[NV];
    if constexpr (VOL == VOL_WEAK) {
      R u[NV], w[NV];
      s.ldc(el, r, u);
      s.ldw(el, r, w);
      P::template flux<O>(u, w, f, p.pp);
    } else {
      const int t = r / NP, pp_ = r - (r / NP) * NP;
      int i, m;
      pair_nodes<N>(pp_, i, m);
      const int ni = line_node<DIM, N, O>(t, i), nm = line_node<DIM, N, O>(t, m);
      R ui[NV], wi[NV], um[NV], wm[NV];
      s.ldc(el, ni, ui);
      s.ldw(el, ni, wi);
      s.ldc(el, nm, um);
      s.ldw(el, nm, wm);
      two_point_flux_t<DIM, EQ, R, O, VFLUX>(ui, wi, um, wm, f, p.pp);
    }
    sts_rec<NV>(s.vol(el, O, r), f);
  }

  // surface item: face 2*O + side, face node t (neighbour data staged in phase A)
  template <int O>
  __device__ __forceinline__ static void surface_item(const FusedParams<R> &p, const Smem &s, int el, int side,
                                                      int t) {
    const int face = 2 * O + side;
    R f[NV];
    lds_rec<NV>(s.tr(el, face, t), f);
    if (s.conforming[el * 2 * DIM + face]) {
      const int own = line_node<DIM, N, O>(t, side == 0 ? 0 : N - 1);
      R un[NV], wn[NV], uo[NV], wo[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) un[v] = f[v];
      P::prim(un, wn, p.pp);
      s.ldc(el, own, uo);
      s.ldw(el, own, wo);
      if (side == 0)
        two_point_flux<DIM, EQ, R, O, HLL_FAMILY, SC_EC>(p.surface_flux, un, wn, uo, wo, f, p.pp);
      else
        two_point_flux<DIM, EQ, R, O, HLL_FAMILY, SC_EC>(p.surface_flux, uo, wo, un, wn, f, p.pp);
      // nonconservative terms: each side adds 0.5 Phi(own, other)
      // (interface_flux_kernel!, src/solvers/dg_2d_kernel.jl:1009-1035)
      if constexpr (NC) P::template add_noncons<O>(wo, wn, R(0.5), f);
    }
    sts_rec<NV>(s.surf(el, face, t), f);
  }

  // FV subcell item (shock capturing): flux between nodes a and a+1 of line t
  template <int O>
  __device__ __forceinline__ static void fv_item(const FusedParams<R> &p, const Smem &s, int el, int t, int a) {
    R ul[NV], wl[NV], ur[NV], wr[NV], f[NV];
    const int nl = line_node<DIM, N, O>(t, a), nr = line_node<DIM, N, O>(t, a + 1);
    s.ldc(el, nl, ul);
    s.ldw(el, nl, wl);
    s.ldc(el, nr, ur);
    s.ldw(el, nr, wr);
    two_point_flux<DIM, EQ, R, O, HLL_FAMILY, SC_EC>(p.fv_flux, ul, wl, ur, wr, f, p.pp);
    if constexpr (NC) {
      R g[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) g[v] = f[v];
      P::template add_noncons<O>(wl, wr, R(0.5), f);  // fstar_L: node a's side
      P::template add_noncons<O>(wr, wl, R(0.5), g);  // fstar_R: node a+1's side
      sts_rec<NV>(s.fv(el, O, t, a, 1), g);
    }
    sts_rec<NV>(s.fv(el, O, t, a), f);
  }

  // owner-pair volume term of direction O for node `node` (position ci on
  // its line): acc += sum_{m != ci} D_split[ci, m] f#_O(u_node, u_m), the
  // partners visited as m = ci + 1, ..., ci + N - 1 (mod N) so that every
  // lane of a warp evaluates a flux in every step
  template <int O>
  __device__ __forceinline__ static void owner_volume(const FusedParams<R> &p, const Smem &s, int el, int node,
                                                      int ci, const R *ui, const R *wi, R *acc) {
    constexpr int stride = (O == 0) ? 1 : (O == 1) ? N : N * N;
    const int n0 = node - ci * stride;
    const R *drow = s.dsplit + ci * N;
#pragma unroll
    for (int k = 1; k < N; ++k) {
      int m = ci + k;
      if (m >= N) m -= N;
      R um[NV], wm[NV], f[NV];
      s.ldc(el, n0 + m * stride, um);
      s.ldw(el, n0 + m * stride, wm);
      two_point_flux_t<DIM, EQ, R, O, VFLUX>(ui, wi, um, wm, f, p.pp);
      const R dm = drow[m];
#pragma unroll
      for (int v = 0; v < NV; ++v) acc[v] += dm * f[v];
    }
  }

  template <int J>
  __device__ __forceinline__ static void partner(const Smem &s, int node, const int *coord, int &nm, R &dm) {
    constexpr int O = J / (N - 1), k = 1 + J % (N - 1);
    constexpr int stride = (O == 0) ? 1 : (O == 1) ? N : N * N;
    const int ci = coord[O];
    int m = ci + k;
    if (m >= N) m -= N;
    nm = node + (m - ci) * stride;
    dm = s.dsplit[ci * N + m];
  }
  template <int J>
  __device__ __forceinline__ static void owner_volume_packed(const FusedParams<R> &p, const Smem &s, int el, int node,
                                                             const int *coord, const R *wi, float2 *acc2, R *acc) {
    constexpr int NPART = DIM * (N - 1);
    if constexpr (J + 1 < NPART) {
      int na, nb;
      R da, db;
      partner<J>(s, node, coord, na, da);
      partner<J + 1>(s, node, coord, nb, db);
      R wa[NV], wb[NV];
      s.ldw(el, na, wa);
      s.ldw(el, nb, wb);
      float2 f[NV];
      ranocha_x2<DIM, J / (N - 1), (J + 1) / (N - 1)>(wi, wa, wb, f, p.pp);
      const float2 dd = pk::mk(da, db);
#pragma unroll
      for (int v = 0; v < NV; ++v) acc2[v] = pk::fma2(dd, f[v], acc2[v]);
      owner_volume_packed<J + 2>(p, s, el, node, coord, wi, acc2, acc);
    } else if constexpr (J < NPART) {
      int nm;
      R dm;
      partner<J>(s, node, coord, nm, dm);
      R ui[NV], um[NV], wm[NV], f[NV];
      s.ldc(el, node, ui);
      s.ldc(el, nm, um);
      s.ldw(el, nm, wm);
      two_point_flux_t<DIM, EQ, R, J / (N - 1), VFLUX>(ui, wi, um, wm, f, p.pp);
#pragma unroll
      for (int v = 0; v < NV; ++v) acc[v] += dm * f[v];
    }
  }

  __device__ __forceinline__ static void run(const FusedParams<R> &p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // runtime tile: p.wpg warps per group (>= the owners of EPG elements),
    // p.gpb groups per block (launch_one validates both); the block is
    // (32 * wpg, gpb), so threadIdx.y is the group and the threads of a group
    // are consecutive warps
    const int GTr = 32 * p.wpg;
    const int gid = threadIdx.y;  // group within the block
    const int gt = threadIdx.x;
    Smem s;
    s.u64 = reinterpret_cast<double *>(smem_raw + gid * GROUP_SMEM);
    s.k64 = s.u64 + N_UK;
    s.cons = reinterpret_cast<R *>(s.k64 + N_UK);
    s.prim = s.cons + N_CONS;
    s.fvol = s.prim + N_CONS;
    s.ffv = s.fvol + N_VOL;
    s.trace = s.ffv + N_FV;
    s.fsurf = s.trace;  // each surface item overwrites its own trace record
    s.alpha = s.trace + N_TRACE;
    s.scale = s.alpha + N_EL;
    s.dsplit = s.scale + N_EL;
    s.dhat = s.dsplit + N * N;
    s.invw = s.dhat + N * N;
    s.conforming = reinterpret_cast<int *>(s.dsplit + N_OPS);
    // the operators, staged once per group (first read after phase A's sync)
    for (int q = gt; q < N * N; q += GTr) {
      s.dsplit[q] = p.dsplit[q];
      s.dhat[q] = p.dhat[q];
    }
    if (gt < N) s.invw[gt] = p.invw[gt];
    const int64_t e0 = ((int64_t)blockIdx.x * p.gpb + gid) * EPG;  // first element of the group
    if (e0 >= p.nelements) return;  // whole groups leave together
    const int ne = (int)min((int64_t)EPG, p.nelements - e0);

    const int mode = p.mode;
    const bool surface = (mode != MODE_VOLUME);
    const bool vec = p.vec16 != 0;
    const bool use_k = (mode == MODE_RK) && p.use_k;
    // The connectivity and the geometry are constant: their loads go out
    // before the wait for the previous kernel below, so that the neighbour
    // traces of phase A need one global round trip after it, not two (face
    // table, then the neighbour's node).  nbp[it]: the face-table entry of
    // this thread's trace item it (items j = gt + it * GTr).
    constexpr int PER_EL = 2 * DIM * NF;
    const int n_trace = surface ? ne * PER_EL : 0;
    int32_t nbp[TR_IT];
#pragma unroll
    for (int it = 0; it < TR_IT; ++it) {
      const int j = gt + it * GTr;
      nbp[it] = 0;
      if (j < n_trace) {
        const int el = j / PER_EL, face = (j - el * PER_EL) / NF;
        nbp[it] = __ldg(p.face_table + (e0 + el) * (2 * DIM) + face);
      }
    }
    const int my_el = gt / NN, my_node = gt - (gt / NN) * NN;
    const bool has_node = (gt < EPG * NN) && (my_el < ne);
    double inv_jac_el = 0.0, dt_el = p.dt;  // the owner's element's J^{-1} and time step
    if (has_node) {
      inv_jac_el = __ldg(p.inv_jac + e0 + my_el);
      if (p.dt_elem) dt_el = __ldg(p.dt_elem + e0 + my_el);
    }
    if (p.pdl) {
      // programmatic dependent launch: the next kernel in the stream may start
      // launching now (it waits below before its own reads), and this grid
      // waits until the previous kernel has completed and its writes are
      // visible before reading u, k, mortar fluxes or alpha
      asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
      asm volatile("griddepcontrol.wait;" ::: "memory");
    }

    // phase A: every global read of the group is issued here.  Owner thread
    // (el, node) keeps its node's u and k in registers until phase C; all
    // threads stage the neighbours' face nodes (or the mortar fluxes) of the
    // group's faces in shared memory.
    const int64_t g0 = ((e0 + my_el) * NN + my_node) * NV;
    // FP32 copy of u_in (FP32 kernels inside trixi_rk_steps), else null
    const float *sh_in = nullptr;
    if constexpr (sizeof(R) == 4) sh_in = p.u32_in;
    double ureg[NV], kreg[NV];
    R uown[NV];
    if constexpr (UK_SMEM) {
      if (mode == MODE_RK) {
        // the group's u (and k) spans, contiguous in global memory
        const int nval = ne * NN * NV;
        const double *gu = p.u_in + e0 * NN * NV, *gk = p.k + e0 * NN * NV;
        const bool a16 = vec && ((e0 * NN * NV) & 1) == 0;  // 16-byte aligned span starts
        if (a16) {
          const int nc = nval >> 1;
          for (int c = gt; c < nc; c += GTr) {
            cp_async16(s.u64 + 2 * c, gu + 2 * c);
            if (use_k) cp_async16(s.k64 + 2 * c, gk + 2 * c);
          }
          if ((nval & 1) && gt == 0) {
            cp_async8(s.u64 + nval - 1, gu + nval - 1);
            if (use_k) cp_async8(s.k64 + nval - 1, gk + nval - 1);
          }
        } else {
          for (int c = gt; c < nval; c += GTr) {
            cp_async8(s.u64 + c, gu + c);
            if (use_k) cp_async8(s.k64 + c, gk + c);
          }
        }
      }
      if (has_node) {
        if (sh_in != nullptr) {
          if constexpr (sizeof(R) == 4) ldg_rec32<NV>(sh_in + g0, uown);
        } else {
          ldg_node<NV>(p.u_in + g0, ureg, vec);
        }
      }
    } else if (has_node) {
      ldg_node<NV>(p.u_in + g0, ureg, vec);
      if (use_k) ldg_node<NV>(p.k + g0, kreg, vec);
      if constexpr (sizeof(R) == 4)
        if (sh_in) ldg_rec32<NV>(sh_in + g0, uown);
    }
    if (surface) {
#pragma unroll
      for (int it = 0; it < TR_IT; ++it) {
        const int j = gt + it * GTr;
        if (j >= n_trace) break;
        const int el = j / PER_EL, r = j - (j / PER_EL) * PER_EL;
        const int face = r / NF, t = r - (r / NF) * NF;
        const int32_t nb = nbp[it];
        R tr[NV];
        if (sh_in != nullptr && nb >= 0) {
          // the neighbour's node from the FP32 copy: no conversion
          const int other = line_node_rt<DIM, N>(face >> 1, t, (face & 1) ? 0 : N - 1);
          if constexpr (sizeof(R) == 4) ldg_rec32<NV>(sh_in + ((int64_t)nb * NN + other) * NV, tr);
        } else {
          double tv[NV];
          if (nb >= 0) {
            const int o = face >> 1;
            const int other = line_node_rt<DIM, N>(o, t, (face & 1) ? 0 : N - 1);
            ldg_node<NV>(p.u_in + ((int64_t)nb * NN + other) * NV, tv, vec);
          } else if (BND && nb == FACE_BOUNDARY) {
            // Dirichlet boundary: the boundary function's state at the face node
            // plays the neighbour's trace (the surface flux then follows the
            // interface convention: inner state on the left of an upper face)
            if constexpr (BND) {
              const int o = face >> 1;
              const int own = line_node_rt<DIM, N>(o, t, (face & 1) ? N - 1 : 0);
              eval_ic<DIM, EQ>(p.bc_kind, p.coords + ((e0 + el) * NN + own) * DIM, p.t, p.bc, tv);
            }
          } else {
            ldg_node<NV>(p.mortar_flux + ((int64_t)(-nb - 1) * NF + t) * NV, tv, vec);
          }
#pragma unroll
          for (int v = 0; v < NV; ++v) tr[v] = narrow<HW_TRACE>(tv[v]);
        }
        sts_rec<NV>(s.tr(el, face, t), tr);
        if (t == 0) s.conforming[el * 2 * DIM + face] = (nb >= 0 || (BND && nb == FACE_BOUNDARY));
      }
    }
    if (has_node) {
      R uu[NV], ww[NV];
      if (sh_in != nullptr) {
#pragma unroll
        for (int v = 0; v < NV; ++v) uu[v] = uown[v];
      } else {
#pragma unroll
        for (int v = 0; v < NV; ++v) uu[v] = narrow<HW_OWNER>(ureg[v]);
      }
      P::prim(uu, ww, p.pp);
      s.stc(my_el, my_node, uu);
      s.stw(my_el, my_node, ww);
      if (my_node == 0) {
        if constexpr (VOL == VOL_SC) {
          const double a = p.alpha[e0 + my_el];
          s.alpha[my_el] = (fabs(a) <= p.atol) ? R(0) : from_double<R>(a);
        }
        // per-element factor of the node phase: -J^{-1} (rhs) or -J^{-1} dt (RK)
        const double f = -inv_jac_el * (mode == MODE_RK ? dt_el : 1.0);
        s.scale[my_el] = from_double<R>(f);
      }
    }
    group_sync(gid, p.wpg, GTr);

    // phase B: every flux of the group, sections [volume | surface | FV],
    // each ordered [direction][element][item] so warps stay on one direction
    constexpr int PER_VOL = EPG * VOL_PER_DIR;
    constexpr int PER_SURF = EPG * 2 * NF;
    constexpr int PER_FV = EPG * FV_PER_DIR;
    constexpr int NVOL_ITEMS = DIM * PER_VOL;
    const int n_surf = surface ? DIM * PER_SURF : 0;
    const int n_all = NVOL_ITEMS + n_surf + DIM * PER_FV;
    for (int w = gt; w < n_all; w += GTr) {
      if (w < NVOL_ITEMS) {
        // (the divisors are never 0 where this runs; the guards only keep the
        // kernels without volume items, LINEAR, free of a constant division by 0)
        constexpr int PV = PER_VOL > 0 ? PER_VOL : 1, VD = VOL_PER_DIR > 0 ? VOL_PER_DIR : 1;
        const int dir = w / PV;
        const int r0 = w - dir * PV;
        const int el = r0 / VD, r = r0 - (r0 / VD) * VD;
        if (el >= ne) continue;
        if (dir == 0) volume_item<0>(p, s, el, r);
        if constexpr (DIM > 1) if (dir == 1) volume_item<1>(p, s, el, r);
        if constexpr (DIM > 2) if (dir == 2) volume_item<2>(p, s, el, r);
      } else if (w < NVOL_ITEMS + n_surf) {
        const int w2 = w - NVOL_ITEMS;
        const int dir = w2 / PER_SURF;
        const int r0 = w2 - dir * PER_SURF;
        const int el = r0 / (2 * NF);
        const int r1 = r0 - el * (2 * NF);
        const int side = r1 / NF, t = r1 - (r1 / NF) * NF;
        if (el >= ne) continue;
        if (dir == 0) surface_item<0>(p, s, el, side, t);
        if constexpr (DIM > 1) if (dir == 1) surface_item<1>(p, s, el, side, t);
        if constexpr (DIM > 2) if (dir == 2) surface_item<2>(p, s, el, side, t);
      } else if constexpr (VOL == VOL_SC) {
        const int w2 = w - NVOL_ITEMS - n_surf;
        const int dir = w2 / PER_FV;
        const int r0 = w2 - dir * PER_FV;
        const int el = r0 / FV_PER_DIR;
        const int r1 = r0 - el * FV_PER_DIR;
        const int t = r1 / (N - 1), a = r1 - (r1 / (N - 1)) * (N - 1);
        if (el >= ne || s.alpha[el] == R(0)) continue;
        if (dir == 0) fv_item<0>(p, s, el, t, a);
        if constexpr (DIM > 1) if (dir == 1) fv_item<1>(p, s, el, t, a);
        if constexpr (DIM > 2) if (dir == 2) fv_item<2>(p, s, el, t, a);
      }
    }

    // node coordinates of the owner thread, and the face index of its line
    // through each face
    const int el = my_el, node = my_node;
    int coord[3] = {0, 0, 0}, tface[3] = {0, 0, 0};
    {
      int qq = node;
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        coord[d] = qq % N;
        qq /= N;
      }
      if constexpr (DIM == 2) {
        tface[0] = coord[1];
        tface[1] = coord[0];
      } else if constexpr (DIM == 3) {
        tface[0] = coord[1] + N * coord[2];
        tface[1] = coord[0] + N * coord[2];
        tface[2] = coord[0] + N * coord[1];
      }
    }
    R acc[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) acc[v] = R(0);
    if constexpr (OWNER_PAIRS) {
      // the owner-pair volume term needs only the node records, already
      // visible after phase A's barrier
      if (has_node) {
        R ui[NV], wi[NV];
        s.ldc(el, node, ui);
        s.ldw(el, node, wi);
        if constexpr (PACKED) {
          float2 acc2[NV];
#pragma unroll
          for (int v = 0; v < NV; ++v) acc2[v] = pk::bc(0.0f);
          owner_volume_packed<0>(p, s, el, node, coord, wi, acc2, acc);
#pragma unroll
          for (int v = 0; v < NV; ++v) acc[v] += acc2[v].x + acc2[v].y;
        } else {
          owner_volume<0>(p, s, el, node, coord[0], ui, wi, acc);
          if constexpr (DIM > 1) owner_volume<1>(p, s, el, node, coord[1], ui, wi, acc);
          if constexpr (DIM > 2) owner_volume<2>(p, s, el, node, coord[2], ui, wi, acc);
        }
      }
    }
    if constexpr (UK_SMEM) cp_async_wait_all();
    group_sync(gid, p.wpg, GTr);

    // phase C: the thread that loaded node q finishes it
    if (!has_node) return;
    if constexpr (UK_SMEM) {
      if (mode == MODE_RK) {
        const int q = (el * NN + node) * NV;
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          ureg[v] = s.u64[q + v];
          if (use_k) kreg[v] = s.k64[q + v];
        }
      }
    }
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      const int ci = coord[d];
      if constexpr (OWNER_PAIRS) {
        // (the volume term is in acc already)
      } else if constexpr (LINEAR) {
        // linear advection: sum_m D_hat[i,m] a_d u_m (weak form) or
        // sum_m D_split[i,m] a_d (u_i + u_m)/2 (flux differencing), with a_d
        // taken out of the sum: one multiply per direction (FP64 multiplies
        // occupy GB300's narrow FP64 pipe)
        constexpr int strides[3] = {1, N, N * N};
        const int n0 = node - ci * strides[d];
        R sum = R(0);
        if constexpr (VOL == VOL_WEAK) {
#pragma unroll
          for (int m = 0; m < N; ++m) sum += s.dhat[ci * N + m] * s.c(el, n0 + m * strides[d])[0];
          acc[0] += p.pp.a[d] * sum;
        } else {
          const R ui = s.c(el, node)[0];
#pragma unroll
          for (int m = 0; m < N; ++m) {
            if (m == ci) continue;
            sum += s.dsplit[ci * N + m] * (ui + s.c(el, n0 + m * strides[d])[0]);
          }
          acc[0] += (R(0.5) * p.pp.a[d]) * sum;
        }
      } else if constexpr (VOL == VOL_WEAK) {
        constexpr int strides[3] = {1, N, N * N};
        const int n0 = node - ci * strides[d];
#pragma unroll
        for (int m = 0; m < N; ++m) {
          const R dm = s.dhat[ci * N + m];
          R F[NV];
          lds_rec<NV>(s.vol(el, d, n0 + m * strides[d]), F);
#pragma unroll
          for (int v = 0; v < NV; ++v) acc[v] += dm * F[v];
        }
      } else {
#pragma unroll
        for (int m = 0; m < N; ++m) {
          if (m == ci) continue;
          const R dm = s.dsplit[ci * N + m];
          R F[NV];
          lds_rec<NV>(s.vol(el, d, tface[d] * NP + pair_index<N>(ci, m)), F);
#pragma unroll
          for (int v = 0; v < NV; ++v) acc[v] += dm * F[v];
        }
      }
    }
    if constexpr (NC) {
      // nonconservative volume term 0.5 sum_d sum_m D_split[i_d, m] Phi_d(u_i, u_m)
      // (src/solvers/dg_2d_kernel.jl:269-292).  Phi_d(u_i, u_m) is linear in
      // u_m's (B_d, psi), so the sum is Phi_d(u_i, .) of sum_m D_split[i_d, m] (B_d, psi)_m.
      R wo[NV];
      s.ldw(el, node, wo);
      constexpr int strides[3] = {1, N, N * N};
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        const int ci = coord[d];
        const int n0 = node - ci * strides[d];
        R g[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) g[v] = R(0);
#pragma unroll
        for (int m = 0; m < N; ++m) {
          if (m == ci) continue;
          const R dm = s.dsplit[ci * N + m];
          const R *wm = s.w(el, n0 + m * strides[d]);
          g[5 + d] += dm * wm[5 + d];
          g[8] += dm * wm[8];
        }
        if (d == 0) P::template add_noncons<0>(wo, g, R(0.5), acc);
        if constexpr (DIM > 1) if (d == 1) P::template add_noncons<1>(wo, g, R(0.5), acc);
        if constexpr (DIM > 2) if (d == 2) P::template add_noncons<2>(wo, g, R(0.5), acc);
      }
    }
    if constexpr (VOL == VOL_SC) {
      const R alpha = s.alpha[el];
      if (alpha != R(0)) {
        R fv[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) fv[v] = R(0);
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
          const int ci = coord[d];
          const R iw = s.invw[ci];
          if (ci + 1 < N) {
            R F[NV];
            lds_rec<NV>(s.fv(el, d, tface[d], ci), F);
#pragma unroll
            for (int v = 0; v < NV; ++v) fv[v] += iw * F[v];
          }
          if (ci > 0) {
            R F[NV];
            lds_rec<NV>(s.fv(el, d, tface[d], ci - 1, NC ? 1 : 0), F);
#pragma unroll
            for (int v = 0; v < NV; ++v) fv[v] -= iw * F[v];
          }
        }
#pragma unroll
        for (int v = 0; v < NV; ++v) acc[v] = (R(1) - alpha) * acc[v] + alpha * fv[v];
      }
    }
    if (surface) {
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        if (coord[d] == 0) {
          R F[NV];
          lds_rec<NV>(s.surf(el, 2 * d, tface[d]), F);
#pragma unroll
          for (int v = 0; v < NV; ++v) acc[v] -= p.lhat_l * F[v];
        }
        if (coord[d] == N - 1) {
          R F[NV];
          lds_rec<NV>(s.surf(el, 2 * d + 1, tface[d]), F);
#pragma unroll
          for (int v = 0; v < NV; ++v) acc[v] += p.lhat_r * F[v];
        }
      }
    }
    double o[NV], kk[NV];
    if (mode == MODE_VOLUME) {
#pragma unroll
      for (int v = 0; v < NV; ++v) o[v] = to_double(acc[v]);
      stg_node<NV>(p.out + g0, o, vec);
    } else if constexpr (sizeof(R) == sizeof(double)) {
      const double sc = -inv_jac_el;
      const double dte = dt_el;
      double src[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) src[v] = 0.0;
      if constexpr (BND) {
        if (p.src_kind != SRC_NONE)
          source_convergence<DIM, EQ>(p.src, p.bc.gamma, p.coords + ((e0 + el) * NN + node) * DIM, p.t, src,
                                      p.src_kind);
      }
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        double du;
        if constexpr (BND) du = double(acc[v]) * sc + src[v];
        else du = double(acc[v]) * sc;
        if (mode == MODE_RHS) {
          o[v] = du;
        } else {
          kk[v] = (use_k ? p.rk_a * kreg[v] : 0.0) + dte * du;
          o[v] = ureg[v] + p.rk_b * kk[v];
        }
      }
      if (mode == MODE_RK) stg_node<NV>(p.k + g0, kk, vec);
      stg_node<NV>(p.out + g0, o, vec);
    } else {
      // mixed precision: scale in FP32, widen exactly, accumulate the RK
      // register and the state in FP64 (two FMAs on the FP64 pipe)
      const R sc = s.scale[el];
      double src[NV];  // FP64 source term, times dt in the RK form (sc holds -J^{-1} dt there)
#pragma unroll
      for (int v = 0; v < NV; ++v) src[v] = 0.0;
      if constexpr (BND) {
        if (p.src_kind != SRC_NONE) {
          source_convergence<DIM, EQ>(p.src, p.bc.gamma, p.coords + ((e0 + el) * NN + node) * DIM, p.t, src,
                                      p.src_kind);
          const double f = (mode == MODE_RK) ? dt_el : 1.0;
#pragma unroll
          for (int v = 0; v < NV; ++v) src[v] *= f;
        }
      }
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        // (x + 0.0 is not x for x = -0: without sources the FP64 add is not emitted)
        double dd = to_double(acc[v] * sc);
        if constexpr (BND) dd += src[v];
        if (mode == MODE_RHS) {
          o[v] = dd;
        } else {
          kk[v] = use_k ? fma(p.rk_a, kreg[v], dd) : dd;
          o[v] = fma(p.rk_b, kk[v], ureg[v]);
        }
      }
      if (mode == MODE_RK) stg_node<NV>(p.k + g0, kk, vec);
      stg_node<NV>(p.out + g0, o, vec);
      if (p.u32_out) {
        // the next stage's flux states: u_out narrowed as phase A would narrow it
        R f[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) f[v] = narrow<HW_OUT>(o[v]);
        stg_rec32<NV>(p.u32_out + g0, f);
      }
    }
  }
};

template <int DIM, int N, int EQ, typename R, int VOL, int VFLUX, int BND>
__global__ void __launch_bounds__(512) dg_fused_kernel(const FusedParams<R> p) {
  FusedKernel<DIM, N, EQ, R, VOL, VFLUX, BND>::run(p);
}

// the ideal GLM-MHD kernels: blocks of at most 256 threads, so that a thread
// may hold up to 255 registers (9-variable states)
template <int DIM, int N, int EQ, typename R, int VOL, int VFLUX, int BND>
__global__ void __launch_bounds__(256, 1) dg_fused_kernel_wide(const FusedParams<R> p) {
  FusedKernel<DIM, N, EQ, R, VOL, VFLUX, BND>::run(p);
}

// the kernel entry of an instantiation
template <int DIM, int N, int EQ, typename R, int VOL, int VFLUX, int BND>
constexpr auto fused_entry() {
  if constexpr (EQ == EQ_MHD) return &dg_fused_kernel_wide<DIM, N, EQ, R, VOL, VFLUX, BND>;
  else return &dg_fused_kernel<DIM, N, EQ, R, VOL, VFLUX, BND>;
}

}  // namespace trixi
