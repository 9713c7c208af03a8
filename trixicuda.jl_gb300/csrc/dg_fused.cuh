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
// Work decomposition: one thread per two-point flux.  Phase A stages the
// tile's states in shared memory (conservative and primitive variables, in
// the compute precision).  Phase B evaluates every flux the tile needs, each
// exactly once per element: the symmetric volume fluxes f#(u_i, u_m), i < m,
// on every line (N(N-1)/2 per line instead of the reference's N^2), the
// surface fluxes on the element's 2*ndims faces (the neighbour's adjacent
// node is read straight from u -- "owner computes", no interfaces.u or
// surface_flux_values round trip through HBM; mortar faces read the flux
// prepared by the mortar kernel), and for shock capturing the LGL subcell
// FV fluxes.  Phase C gives one thread per (node, variable): it sums
// D_split / D_hat times the staged fluxes along each dimension, adds the
// surface terms, scales by -J^{-1}, and stores du or performs the RK update,
// with coalesced global accesses in the reference layout.
#pragma once
#include "dg_convert.cuh"
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
  int epb;                                  // elements per block
  int mode;
  int surface_flux, fv_flux;
  double rk_a, rk_b, dt;
  double atol;                              // dg-only test for alpha
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

template <int DIM, int N, int EQ, typename R, int VOL, int VFLUX>
struct FusedKernel {
  using P = Physics<DIM, EQ, R>;
  static constexpr int NV = P::NV;
  static constexpr int NN = ipow(N, DIM);
  static constexpr int NF = ipow(N, DIM - 1);
  static constexpr int NP = N * (N - 1) / 2;
  // staged fluxes per element and direction
  static constexpr int VOL_PER_DIR = (VOL == VOL_WEAK) ? NN : NF * NP;
  static constexpr int SURF_PER_EL = 2 * DIM * NF;
  static constexpr int FV_PER_DIR = (VOL == VOL_SC) ? NF * (N - 1) : 0;
  static constexpr int ITEMS_PER_EL = DIM * VOL_PER_DIR + SURF_PER_EL + DIM * FV_PER_DIR;
  static constexpr int F_PER_EL = ITEMS_PER_EL * NV;
  static constexpr int BLOCK = 256;
  static constexpr int TRACE_PER_EL = 2 * DIM * NF * NV;  // neighbour face nodes (or mortar fluxes)
  static constexpr size_t smem_for(int epb) {
    return sizeof(R) * ((size_t)epb * (2 * NV * NN + F_PER_EL + TRACE_PER_EL) + 2 * epb + 2 * N * N + N) +
           sizeof(int) * (size_t)epb * 2 * DIM;
  }
  // elements per block: ~2 flux items per thread, <= 48 KB of shared memory
  static constexpr int epb_pick() {
    int e = (2 * BLOCK + ITEMS_PER_EL - 1) / ITEMS_PER_EL;
    if (e < 1) e = 1;
    if (e > 32) e = 32;
    while (e > 1 && smem_for(e) > 48 * 1024) --e;
    while (e > 1 && e * NN > BLOCK) --e;  // one node per thread in phases A and C
    return e;
  }
  static constexpr int EPB = epb_pick();
  static_assert(EPB * NN <= BLOCK, "one node per thread");
  static size_t smem_bytes() { return smem_for(EPB); }

  struct Smem {
    R *cons, *prim, *fvol, *fsurf, *ffv, *alpha, *scale, *dsplit, *dhat, *invw, *trace;
    int *conforming;  // [el][face]: 1 = trace holds the neighbour's node, 0 = a mortar flux
    // [el][face][t][v]
    __device__ __forceinline__ R *tr(int el, int face, int t) const {
      return trace + ((el * 2 * DIM + face) * NF + t) * NV;
    }
    // [el][v][node]
    __device__ __forceinline__ R &c(int el, int v, int n) const { return cons[(el * NV + v) * NN + n]; }
    __device__ __forceinline__ R &w(int el, int v, int n) const { return prim[(el * NV + v) * NN + n]; }
    // [el][dir][slot][v]
    __device__ __forceinline__ R *vol(int el, int d, int slot) const {
      return fvol + ((el * DIM + d) * VOL_PER_DIR + slot) * NV;
    }
    // [el][face][t][v]
    __device__ __forceinline__ R *surf(int el, int face, int t) const {
      return fsurf + ((el * 2 * DIM + face) * NF + t) * NV;
    }
    // [el][dir][t][a][v]
    __device__ __forceinline__ R *fv(int el, int d, int t, int a) const {
      return ffv + (((el * DIM + d) * NF + t) * (N - 1) + a) * NV;
    }
  };

  __device__ __forceinline__ static void load_node(const Smem &s, int el, int n, R *u, R *w) {
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      u[v] = s.c(el, v, n);
      w[v] = s.w(el, v, n);
    }
  }

  // volume item: one symmetric pair (FD / SC) or one nodal physical flux (weak form)
  template <int O>
  __device__ __forceinline__ static void volume_item(const FusedParams<R> &p, const Smem &s, int el, int r) {
    R f[NV];
    if constexpr (VOL == VOL_WEAK) {
      R u[NV], w[NV];
      load_node(s, el, r, u, w);
      P::template flux<O>(u, w, f, p.pp);
    } else {
      const int t = r / NP, pp_ = r - (r / NP) * NP;
      int i, m;
      pair_nodes<N>(pp_, i, m);
      R ui[NV], wi[NV], um[NV], wm[NV];
      load_node(s, el, line_node<DIM, N, O>(t, i), ui, wi);
      load_node(s, el, line_node<DIM, N, O>(t, m), um, wm);
      two_point_flux_t<DIM, EQ, R, O, VFLUX>(ui, wi, um, wm, f, p.pp);
    }
    R *dst = s.vol(el, O, r);
#pragma unroll
    for (int v = 0; v < NV; ++v) dst[v] = f[v];
  }

  // surface item: face 2*O + side, face node t (neighbour data staged in phase A)
  template <int O>
  __device__ __forceinline__ static void surface_item(const FusedParams<R> &p, const Smem &s, int el, int side,
                                                      int t) {
    const int face = 2 * O + side;
    const R *src = s.tr(el, face, t);
    R f[NV];
    if (s.conforming[el * 2 * DIM + face]) {
      const int own = line_node<DIM, N, O>(t, side == 0 ? 0 : N - 1);
      R un[NV], wn[NV], uo[NV], wo[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) un[v] = src[v];
      P::prim(un, wn, p.pp);
      load_node(s, el, own, uo, wo);
      if (side == 0)
        two_point_flux<DIM, EQ, R, O>(p.surface_flux, un, wn, uo, wo, f, p.pp);
      else
        two_point_flux<DIM, EQ, R, O>(p.surface_flux, uo, wo, un, wn, f, p.pp);
    } else {
#pragma unroll
      for (int v = 0; v < NV; ++v) f[v] = src[v];
    }
    R *dst = s.surf(el, face, t);
#pragma unroll
    for (int v = 0; v < NV; ++v) dst[v] = f[v];
  }

  // FV subcell item (shock capturing): flux between nodes a and a+1 of line t
  template <int O>
  __device__ __forceinline__ static void fv_item(const FusedParams<R> &p, const Smem &s, int el, int t, int a) {
    R ul[NV], wl[NV], ur[NV], wr[NV], f[NV];
    load_node(s, el, line_node<DIM, N, O>(t, a), ul, wl);
    load_node(s, el, line_node<DIM, N, O>(t, a + 1), ur, wr);
    two_point_flux<DIM, EQ, R, O>(p.fv_flux, ul, wl, ur, wr, f, p.pp);
    R *dst = s.fv(el, O, t, a);
#pragma unroll
    for (int v = 0; v < NV; ++v) dst[v] = f[v];
  }

  __device__ __forceinline__ static void run(const FusedParams<R> &p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int epb = EPB;
    Smem s;
    s.cons = reinterpret_cast<R *>(smem_raw);
    s.prim = s.cons + epb * NV * NN;
    s.fvol = s.prim + epb * NV * NN;
    s.fsurf = s.fvol + epb * DIM * VOL_PER_DIR * NV;
    s.ffv = s.fsurf + epb * SURF_PER_EL * NV;
    s.alpha = s.ffv + epb * DIM * FV_PER_DIR * NV;
    s.scale = s.alpha + epb;
    s.dsplit = s.scale + epb;
    s.dhat = s.dsplit + N * N;
    s.invw = s.dhat + N * N;
    s.trace = s.invw + N;
    s.conforming = reinterpret_cast<int *>(s.trace + epb * TRACE_PER_EL);

    const int64_t e0 = (int64_t)blockIdx.x * epb;
    if (e0 >= p.nelements) return;
    const int ne = (int)min((int64_t)epb, p.nelements - e0);
    const int mode = p.mode;
    const bool surface = (mode != MODE_VOLUME);

    // phase A: every global read of the tile is issued here.  Thread q < epb*NN
    // owns node q for the whole kernel (its u and k stay in registers until
    // the node phase); the other threads stage the neighbours' face nodes
    // (or the mortar fluxes) of the tile's faces in shared memory.
    const int tid = threadIdx.x;
    const bool use_k = (mode == MODE_RK) && (p.rk_a != 0.0);
    const int my_el = tid / NN, my_node = tid - (tid / NN) * NN;
    const bool has_node = (tid < epb * NN) && (my_el < ne);
    const int64_t g0 = ((e0 + my_el) * NN + my_node) * NV;
    double ureg[NV], kreg[NV];
    if (has_node) {
#pragma unroll
      for (int v = 0; v < NV; ++v) ureg[v] = p.u_in[g0 + v];
      if (use_k) {
#pragma unroll
        for (int v = 0; v < NV; ++v) kreg[v] = p.k[g0 + v];
      }
    }
    if (surface) {
      constexpr int PER_EL = 2 * DIM * NF;
      const int n_trace = ne * PER_EL;
      for (int j = (tid - epb * NN + BLOCK) % BLOCK; j < n_trace; j += BLOCK) {
        const int el = j / PER_EL, r = j - (j / PER_EL) * PER_EL;
        const int face = r / NF, t = r - (r / NF) * NF;
        const int32_t nb = p.face_table[(e0 + el) * (2 * DIM) + face];
        const double *src;
        if (nb >= 0) {
          const int o = face >> 1;
          const int other = line_node_rt<DIM, N>(o, t, (face & 1) ? 0 : N - 1);
          src = p.u_in + ((int64_t)nb * NN + other) * NV;
        } else {
          src = p.mortar_flux + ((int64_t)(-nb - 1) * NF + t) * NV;
        }
        R *dst = s.tr(el, face, t);
#pragma unroll
        for (int v = 0; v < NV; ++v) dst[v] = from_double<R>(src[v]);
        if (t == 0) s.conforming[el * 2 * DIM + face] = (nb >= 0);
      }
    }
    if (has_node) {
      R uu[NV], ww[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) uu[v] = from_double<R>(ureg[v]);
      P::prim(uu, ww, p.pp);
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        s.c(my_el, v, my_node) = uu[v];
        s.w(my_el, v, my_node) = ww[v];
      }
    }
    if (threadIdx.x < epb && threadIdx.x < ne) {
      const int el = threadIdx.x;
      if constexpr (VOL == VOL_SC) {
        const double a = p.alpha[e0 + el];
        s.alpha[el] = (fabs(a) <= p.atol) ? R(0) : from_double<R>(a);
      }
      // per-element factor of the node phase: -J^{-1} (rhs) or -J^{-1} dt (RK)
      const double dte = p.dt_elem ? p.dt_elem[e0 + el] : p.dt;
      const double f = -p.inv_jac[e0 + el] * (mode == MODE_RK ? dte : 1.0);
      s.scale[el] = from_double<R>(f);
    }
    for (int q = threadIdx.x; q < N * N; q += BLOCK) {
      s.dsplit[q] = p.dsplit[q];
      s.dhat[q] = p.dhat[q];
    }
    if (threadIdx.x < N) s.invw[threadIdx.x] = p.invw[threadIdx.x];
    __syncthreads();

    // phase B: every flux of the tile, sections [volume | surface | FV],
    // each ordered [direction][element][item] so warps stay on one direction
    constexpr int PER_VOL = epb * VOL_PER_DIR;
    constexpr int PER_SURF = epb * 2 * NF;
    constexpr int PER_FV = epb * FV_PER_DIR;
    constexpr int N_VOL = DIM * PER_VOL;
    const int n_surf = surface ? DIM * PER_SURF : 0;
    const int n_all = N_VOL + n_surf + DIM * PER_FV;
    for (int w = threadIdx.x; w < n_all; w += BLOCK) {
      if (w < N_VOL) {
        const int dir = w / PER_VOL;
        const int r0 = w - dir * PER_VOL;
        const int el = r0 / VOL_PER_DIR, r = r0 - (r0 / VOL_PER_DIR) * VOL_PER_DIR;
        if (el >= ne) continue;
        if (dir == 0) volume_item<0>(p, s, el, r);
        if constexpr (DIM > 1) if (dir == 1) volume_item<1>(p, s, el, r);
        if constexpr (DIM > 2) if (dir == 2) volume_item<2>(p, s, el, r);
      } else if (w < N_VOL + n_surf) {
        const int w2 = w - N_VOL;
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
        const int w2 = w - N_VOL - n_surf;
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
    __syncthreads();

    // phase C: the thread that loaded node q finishes it
    if (has_node) {
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
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        const int ci = coord[d];
        if constexpr (VOL == VOL_WEAK) {
          constexpr int strides[3] = {1, N, N * N};
          const int n0 = node - ci * strides[d];
#pragma unroll
          for (int m = 0; m < N; ++m) {
            const R dm = s.dhat[ci * N + m];
            const R *F = s.vol(el, d, n0 + m * strides[d]);
#pragma unroll
            for (int v = 0; v < NV; ++v) acc[v] += dm * F[v];
          }
        } else {
#pragma unroll
          for (int m = 0; m < N; ++m) {
            if (m == ci) continue;
            const R dm = s.dsplit[ci * N + m];
            const R *F = s.vol(el, d, tface[d] * NP + pair_index<N>(ci, m));
#pragma unroll
            for (int v = 0; v < NV; ++v) acc[v] += dm * F[v];
          }
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
              const R *F = s.fv(el, d, tface[d], ci);
#pragma unroll
              for (int v = 0; v < NV; ++v) fv[v] += iw * F[v];
            }
            if (ci > 0) {
              const R *F = s.fv(el, d, tface[d], ci - 1);
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
            const R *F = s.surf(el, 2 * d, tface[d]);
#pragma unroll
            for (int v = 0; v < NV; ++v) acc[v] -= p.lhat_l * F[v];
          }
          if (coord[d] == N - 1) {
            const R *F = s.surf(el, 2 * d + 1, tface[d]);
#pragma unroll
            for (int v = 0; v < NV; ++v) acc[v] += p.lhat_r * F[v];
          }
        }
      }
      if (mode == MODE_VOLUME) {
#pragma unroll
        for (int v = 0; v < NV; ++v) p.out[g0 + v] = to_double(acc[v]);
      } else if constexpr (sizeof(R) == sizeof(double)) {
        const double sc = -p.inv_jac[e0 + el];
        const double dte = p.dt_elem ? p.dt_elem[e0 + el] : p.dt;
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          const double du = double(acc[v]) * sc;
          if (mode == MODE_RHS) {
            p.out[g0 + v] = du;
          } else {
            const double kk = (use_k ? p.rk_a * kreg[v] : 0.0) + dte * du;
            p.k[g0 + v] = kk;
            p.out[g0 + v] = ureg[v] + p.rk_b * kk;
          }
        }
      } else {
        // mixed precision: scale in FP32, widen exactly, accumulate the RK
        // register and the state in FP64 (two FMAs on the FP64 pipe)
        const R sc = s.scale[el];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          const double dd = to_double(acc[v] * sc);
          if (mode == MODE_RHS) {
            p.out[g0 + v] = dd;
          } else {
            const double kk = use_k ? fma(p.rk_a, kreg[v], dd) : dd;
            p.k[g0 + v] = kk;
            p.out[g0 + v] = fma(p.rk_b, kk, ureg[v]);
          }
        }
      }
    }
  }
};

template <int DIM, int N, int EQ, typename R, int VOL, int VFLUX>
__global__ void __launch_bounds__(256) dg_fused_kernel(const FusedParams<R> p) {
  FusedKernel<DIM, N, EQ, R, VOL, VFLUX>::run(p);
}

}  // namespace trixi
