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
// Work decomposition ("lines"): a tensor-product element is a set of 1D lines
// of N nodes along each dimension.  One thread owns one line: it keeps the N
// nodal states in registers, evaluates each symmetric two-point flux once
// (N(N-1)/2 pairs instead of the reference's N^2), and computes the two
// surface fluxes at the line's ends itself, reading the neighbouring
// element's adjacent node straight from u ("owner computes": no
// interfaces.u or surface_flux_values round trip through HBM).  Faces on a
// mortar take their flux from a small per-mortar buffer filled by
// dg_mortar_kernel.  Each line writes its partial du for its direction to
// shared memory; the node phase sums the directions, scales by -J^{-1} and
// either stores du or performs the RK update with coalesced global accesses.
#pragma once
#include "dg_physics.cuh"

namespace trixi {

constexpr int NMAXT = 6;        // largest N = polydeg + 1 compiled

template <typename R>
struct FusedParams {
  const double *__restrict__ u_in;          // [E][NN][NV]
  double *__restrict__ out;                 // du (VOLUME/RHS) or u_out (RK)
  double *__restrict__ k;                   // RK register (RK)
  const int32_t *__restrict__ face_table;   // [E][2*DIM]: >=0 neighbour element, <0: -(slot+1)
  const double *__restrict__ mortar_flux;   // [slot][NF][NV]
  const double *__restrict__ inv_jac;       // [E]
  const double *__restrict__ alpha;         // [E] (shock capturing)
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

// Offset of the first node of line t (face index t) along orientation O.
template <int DIM, int N, int O>
__device__ __forceinline__ int line_offset(int t) {
  if constexpr (DIM == 1) {
    return 0;
  } else if constexpr (DIM == 2) {
    return (O == 0) ? t * N : t;
  } else {
    const int t1 = t % N, t2 = t / N;
    if constexpr (O == 0) return t1 * N + t2 * N * N;
    else if constexpr (O == 1) return t1 + t2 * N * N;
    else return t1 + t2 * N;
  }
}

template <int DIM, int N, int EQ, typename R, int VOL, int VFLUX>
struct FusedKernel {
  using P = Physics<DIM, EQ, R>;
  static constexpr int NV = P::NV;
  static constexpr int NN = ipow(N, DIM);
  static constexpr int NF = ipow(N, DIM - 1);
  static constexpr int LINES = DIM * NF;

  static size_t smem_bytes(int epb) {
    return sizeof(R) * ((size_t)(2 + DIM) * epb * NV * NN + epb);
  }

  template <int O>
  __device__ __forceinline__ static void line(const FusedParams<R> &p, int el, int t, int64_t e0, const R *s_cons,
                                              const R *s_prim, R *s_du, const R *s_alpha) {
    constexpr int S = ipow(N, O);
    const int off = line_offset<DIM, N, O>(t);
    const int64_t e = e0 + el;
    const PhysParams<R> &pp = p.pp;
    const bool surface = (p.mode != MODE_VOLUME);

    // issue the neighbour-trace loads first; their latency overlaps the volume work
    int32_t nbl = 0, nbr = 0;
    double gl[NV], gr[NV];
    if (surface) {
      nbl = p.face_table[e * (2 * DIM) + 2 * O];
      nbr = p.face_table[e * (2 * DIM) + 2 * O + 1];
      if (nbl >= 0) {
        const double *src = p.u_in + ((int64_t)nbl * NN + off + (N - 1) * S) * NV;
#pragma unroll
        for (int v = 0; v < NV; ++v) gl[v] = src[v];
      } else {
        const double *src = p.mortar_flux + ((int64_t)(-nbl - 1) * NF + t) * NV;
#pragma unroll
        for (int v = 0; v < NV; ++v) gl[v] = src[v];
      }
      if (nbr >= 0) {
        const double *src = p.u_in + ((int64_t)nbr * NN + off) * NV;
#pragma unroll
        for (int v = 0; v < NV; ++v) gr[v] = src[v];
      } else {
        const double *src = p.mortar_flux + ((int64_t)(-nbr - 1) * NF + t) * NV;
#pragma unroll
        for (int v = 0; v < NV; ++v) gr[v] = src[v];
      }
    }

    R w[N][NV];
    R acc[N][NV];
#pragma unroll
    for (int a = 0; a < N; ++a)
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        w[a][v] = s_prim[(el * NV + v) * NN + off + a * S];
        acc[a][v] = R(0);
      }

    if constexpr (VOL == VOL_WEAK) {
      // du_i = sum_m dhat[i,m] f_O(u_m)
      R f[N][NV];
#pragma unroll
      for (int a = 0; a < N; ++a) {
        R ua[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) ua[v] = s_cons[(el * NV + v) * NN + off + a * S];
        P::template flux<O>(ua, w[a], f[a], pp);
      }
#pragma unroll
      for (int i = 0; i < N; ++i)
#pragma unroll
        for (int m = 0; m < N; ++m)
#pragma unroll
          for (int v = 0; v < NV; ++v) acc[i][v] += p.dhat[i * N + m] * f[m][v];
    } else {
      // symmetric flux differencing: each pair (i<m) evaluated once,
      // du_i += dsplit[i,m] f#, du_m += dsplit[m,i] f#
      constexpr bool need_cons = (VFLUX != FLUX_RANOCHA) || (EQ == EQ_ADV);
      R uc[need_cons ? N : 1][NV];
      if constexpr (need_cons) {
#pragma unroll
        for (int a = 0; a < N; ++a)
#pragma unroll
          for (int v = 0; v < NV; ++v) uc[a][v] = s_cons[(el * NV + v) * NN + off + a * S];
      }
#pragma unroll
      for (int i = 0; i < N; ++i)
#pragma unroll
        for (int m = i + 1; m < N; ++m) {
          R f[NV];
          two_point_flux_t<DIM, EQ, R, O, VFLUX>(need_cons ? uc[need_cons ? i : 0] : w[i], w[i],
                                                 need_cons ? uc[need_cons ? m : 0] : w[m], w[m], f, pp);
          const R dim_ = p.dsplit[i * N + m], dmi = p.dsplit[m * N + i];
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            acc[i][v] += dim_ * f[v];
            acc[m][v] += dmi * f[v];
          }
        }
      if constexpr (VOL == VOL_SC) {
        const R alpha = s_alpha[el];
        if (!(dev_fabs(alpha) <= R(p.atol))) {
          // (1 - alpha) * DG + alpha * FV with LGL subcell fluxes on the line
#pragma unroll
          for (int a = 0; a < N; ++a)
#pragma unroll
            for (int v = 0; v < NV; ++v) acc[a][v] *= (R(1) - alpha);
#pragma unroll
          for (int a = 0; a + 1 < N; ++a) {
            R ul[NV], ur[NV], g[NV];
#pragma unroll
            for (int v = 0; v < NV; ++v) {
              ul[v] = s_cons[(el * NV + v) * NN + off + a * S];
              ur[v] = s_cons[(el * NV + v) * NN + off + (a + 1) * S];
            }
            two_point_flux<DIM, EQ, R, O>(p.fv_flux, ul, w[a], ur, w[a + 1], g, pp);
#pragma unroll
            for (int v = 0; v < NV; ++v) {
              acc[a][v] += alpha * p.invw[a] * g[v];
              acc[a + 1][v] -= alpha * p.invw[a + 1] * g[v];
            }
          }
        }
      }
    }

    if (surface) {
      // left end: face -O, u_ll = neighbour, u_rr = own node 0
      R fs[NV];
      if (nbl >= 0) {
        R un[NV], wn[NV], u0[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          un[v] = R(gl[v]);
          u0[v] = s_cons[(el * NV + v) * NN + off];
        }
        P::prim(un, wn, pp);
        two_point_flux<DIM, EQ, R, O>(p.surface_flux, un, wn, u0, w[0], fs, pp);
      } else {
#pragma unroll
        for (int v = 0; v < NV; ++v) fs[v] = R(gl[v]);
      }
#pragma unroll
      for (int v = 0; v < NV; ++v) acc[0][v] -= p.lhat_l * fs[v];
      // right end: face +O, u_ll = own node N-1, u_rr = neighbour
      if (nbr >= 0) {
        R un[NV], wn[NV], u1[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          un[v] = R(gr[v]);
          u1[v] = s_cons[(el * NV + v) * NN + off + (N - 1) * S];
        }
        P::prim(un, wn, pp);
        two_point_flux<DIM, EQ, R, O>(p.surface_flux, u1, w[N - 1], un, wn, fs, pp);
      } else {
#pragma unroll
        for (int v = 0; v < NV; ++v) fs[v] = R(gr[v]);
      }
#pragma unroll
      for (int v = 0; v < NV; ++v) acc[N - 1][v] += p.lhat_r * fs[v];
    }

    R *dst = s_du + (size_t)O * p.epb * NV * NN;
#pragma unroll
    for (int a = 0; a < N; ++a)
#pragma unroll
      for (int v = 0; v < NV; ++v) dst[(el * NV + v) * NN + off + a * S] = acc[a][v];
  }

  __device__ __forceinline__ static void run(const FusedParams<R> &p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int epb = p.epb;
    R *s_cons = reinterpret_cast<R *>(smem_raw);
    R *s_prim = s_cons + (size_t)epb * NV * NN;
    R *s_du = s_prim + (size_t)epb * NV * NN;
    R *s_alpha = s_du + (size_t)DIM * epb * NV * NN;

    const int64_t e0 = (int64_t)blockIdx.x * epb;
    if (e0 >= p.nelements) return;
    const int ne = (int)min((int64_t)epb, p.nelements - e0);
    const int64_t base = e0 * NN * NV;
    const int nval = ne * NN * NV;

    // phase A: coalesced load of the tile (elements are contiguous in u)
    for (int i = threadIdx.x; i < nval; i += blockDim.x) {
      const int el = i / (NN * NV);
      const int r = i - el * (NN * NV);
      const int node = r / NV;
      const int v = r - node * NV;
      s_cons[(el * NV + v) * NN + node] = R(p.u_in[base + i]);
    }
    if constexpr (VOL == VOL_SC) {
      for (int el = threadIdx.x; el < ne; el += blockDim.x) s_alpha[el] = R(p.alpha[e0 + el]);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < ne * NN; i += blockDim.x) {
      const int el = i / NN, node = i - el * NN;
      R uu[NV], ww[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) uu[v] = s_cons[(el * NV + v) * NN + node];
      P::prim(uu, ww, p.pp);
#pragma unroll
      for (int v = 0; v < NV; ++v) s_prim[(el * NV + v) * NN + node] = ww[v];
    }
    __syncthreads();

    // phase B: one thread per line, items ordered [direction][element][line]
    const int per_dir = ne * NF;
    for (int w = threadIdx.x; w < DIM * per_dir; w += blockDim.x) {
      const int dir = w / per_dir;
      const int r = w - dir * per_dir;
      const int el = r / NF, t = r - el * NF;
      if (dir == 0) line<0>(p, el, t, e0, s_cons, s_prim, s_du, s_alpha);
      if constexpr (DIM > 1) if (dir == 1) line<1>(p, el, t, e0, s_cons, s_prim, s_du, s_alpha);
      if constexpr (DIM > 2) if (dir == 2) line<2>(p, el, t, e0, s_cons, s_prim, s_du, s_alpha);
    }
    __syncthreads();

    // phase C: sum directions, -J^{-1}, store du or RK update (coalesced)
    const size_t dstride = (size_t)epb * NV * NN;
    for (int i = threadIdx.x; i < nval; i += blockDim.x) {
      const int el = i / (NN * NV);
      const int r = i - el * (NN * NV);
      const int node = r / NV;
      const int v = r - node * NV;
      const int si = (el * NV + v) * NN + node;
      R s = s_du[si];
      if constexpr (DIM > 1) s += s_du[dstride + si];
      if constexpr (DIM > 2) s += s_du[2 * dstride + si];
      double d = double(s);
      if (p.mode == MODE_VOLUME) {
        p.out[base + i] = d;
      } else {
        d *= -p.inv_jac[e0 + el];
        if (p.mode == MODE_RHS) {
          p.out[base + i] = d;
        } else {
          const double kk = (p.rk_a != 0.0 ? p.rk_a * p.k[base + i] : 0.0) + p.dt * d;
          p.k[base + i] = kk;
          p.out[base + i] = p.u_in[base + i] + p.rk_b * kk;
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
