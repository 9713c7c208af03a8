// dg_adv.cuh -- the rhs / RK-stage kernel of linear scalar advection on
// periodic and mortar meshes (weak form or flux differencing with the
// central flux; every surface flux of the reference's advection set-ups).
//
// The generic fused kernel (dg_fused.cuh) stages neighbour traces, surface
// flux items and node records per element group with group barriers and a
// tile that the tuner picks; ncu counted 510 thread instructions per node on
// its 3D N = 6 weak-form stage kernel, whose arithmetic is ~20 multiply-adds.
// Here a block holds floor(512 / N^d) whole elements, each thread two of
// its nodes (tid and tid + blockDim), and three phases separated by block
// barriers:
//   A. thread = node: load u (and k), store the narrowed value; thread =
//      face node of the block's element faces (2 d N^(d-1) per element):
//      load the neighbour's adjacent value (or the mortar kernel's flux);
//   B. thread = face node: the surface flux from its own node's value and the
//      neighbour's -- linear in both, a few operations -- to shared memory;
//   C. thread = node: the volume term over its lines (D_hat for the weak
//      form: a_d sum_m D_hat[i,m] u_m; D_split for flux differencing:
//      a_d/2 sum_m D_split[i,m] (u_i + u_m)), the surface terms -/+ lhat f*,
//      -J^{-1} and du or the 2N RK update, as phase C of the generic kernel.
// Every phase maps threads to uniform work (no per-node face branches in
// the loads).  Boundary conditions are not handled here: non-periodic meshes
// use the generic kernel's boundary-capable instantiations.
#pragma once
#include "dg_fused.cuh"

namespace trixi {

// Index tables of one element shape, built at compile time into device
// memory (every block reads the same few hundred bytes, which stay in L1):
// per node its coordinates (4 bits each) and the face index of its line
// through each face direction (6 bits each); per face node (face f, node t
// of the face) the element's own node on that face, the neighbour's adjacent
// node, f and t.  They replace per-thread divisions and branches.
template <int DIM, int N>
struct AdvTables {
  static constexpr int NN = ipow(N, DIM), NF = ipow(N, DIM - 1), FPE = 2 * DIM * NF;
  uint32_t node[NN];
  uint32_t face[FPE];
  static constexpr int lnode(int o, int t, int a) {
    return DIM == 1 ? a
           : DIM == 2 ? (o == 0 ? a + t * N : t + a * N)
                      : (o == 0 ? a + (t % N) * N + (t / N) * N * N
                                : o == 1 ? (t % N) + a * N + (t / N) * N * N : (t % N) + (t / N) * N + a * N * N);
  }
  static constexpr AdvTables make() {
    AdvTables tb{};
    for (int q = 0; q < NN; ++q) {
      int c[3] = {0, 0, 0}, tf[3] = {0, 0, 0}, qq = q;
      for (int d = 0; d < DIM; ++d) {
        c[d] = qq % N;
        qq /= N;
      }
      if (DIM == 2) {
        tf[0] = c[1];
        tf[1] = c[0];
      } else if (DIM == 3) {
        tf[0] = c[1] + N * c[2];
        tf[1] = c[0] + N * c[2];
        tf[2] = c[0] + N * c[1];
      }
      tb.node[q] = (uint32_t)(c[0] | (c[1] << 4) | (c[2] << 8) | (tf[0] << 12) | (tf[1] << 18) | (tf[2] << 24));
    }
    for (int r = 0; r < FPE; ++r) {
      const int f = r / NF, t = r % NF, o = f / 2;
      const int own = lnode(o, t, (f & 1) ? N - 1 : 0), other = lnode(o, t, (f & 1) ? 0 : N - 1);
      tb.face[r] = (uint32_t)(own | (other << 8) | (f << 16) | (t << 19));
    }
    return tb;
  }
};
template <int DIM, int N>
__device__ const AdvTables<DIM, N> g_adv_tables = AdvTables<DIM, N>::make();

template <int DIM, int N, typename R, int VOL>
struct AdvKernel {
  static constexpr int NN = ipow(N, DIM);
  static constexpr int NF = ipow(N, DIM - 1);
  static constexpr int EPB = (512 / NN) > 0 ? 512 / NN : 1;  // elements per block
  // nodes per thread: thread tid holds nodes tid, tid + BLOCK, ... of the
  // block (coalesced loads; twice the independent loads in flight per
  // thread).  Measured on the batched ensemble, FP32-mixed: 5.66 ms per step
  // with one node per thread, 5.44 ms with two (FP64: 45.6 -> 44.9 ms).
  static constexpr int NPT = 2;
  static constexpr int NODES = EPB * NN;
  static constexpr int BLOCK = (((NODES + NPT - 1) / NPT) + 31) / 32 * 32;

  // the surface flux kinds of linear advection: central and flux_ranocha
  // (the arithmetic mean), Lax-Friedrichs (speed |a|) and HLL (lmin = lmax =
  // a: the upwind value), as the generic kernel's two_point_flux forms them
  __device__ __forceinline__ static R face_flux(int kind, R a, R ul, R ur) {
    if (kind == FLUX_HLL || kind == FLUX_HLLE) return a >= R(0) ? a * ul : a * ur;
    R f = R(0.5) * (a * ul + a * ur);
    if (kind == FLUX_LLF || kind == FLUX_LLF_NAIVE) f += -R(0.5) * dev_fabs(a) * (ur - ul);
    return f;
  }

  // the neighbour's value narrowed on the FP64 pipe (as the generic kernel's
  // neighbour traces); the owner's own value on the integer pipe
  __device__ __forceinline__ static R narrow_hw(double x) { return R(x); }

  static constexpr int FPE = 2 * DIM * NF;                    // face nodes per element
  static constexpr int ITEMS = EPB * FPE;                      // face nodes per block
  static constexpr int IPT = (ITEMS + BLOCK - 1) / BLOCK;      // face nodes per thread

  __device__ __forceinline__ static void run(const FusedParams<R> &p) {
    __shared__ R s_u[EPB * NN];
    __shared__ R s_f[ITEMS];   // [element][face][face node]
    __shared__ R s_op[N * N];  // D_hat (weak form) or D_split (flux differencing), row-major
    __shared__ R s_scale[EPB];  // FP32 path: -J^{-1} (rhs) or -J^{-1} dt (RK) per element
    const int tid = threadIdx.x;
    for (int q = tid; q < N * N; q += BLOCK) s_op[q] = (VOL == VOL_WEAK) ? p.dhat[q] : p.dsplit[q];
    const int64_t e0 = (int64_t)blockIdx.x * EPB;
    const int mode = p.mode;
    const bool surface = mode != MODE_VOLUME;
    const bool use_k = mode == MODE_RK && p.use_k;
    // the block's nodes (and face nodes) are contiguous from element e0 on:
    // block-relative 32-bit indices against block base pointers
    const int nvalid = (int)min((int64_t)NODES, (p.nelements - e0) * NN);
    const int ivalid = surface ? (int)min((int64_t)ITEMS, (p.nelements - e0) * FPE) : 0;
    const double *ub = p.u_in + e0 * NN;
    double *const ob = p.out + e0 * NN;
    double *const kb = (mode == MODE_RK) ? p.k + e0 * NN : nullptr;  // (k is absent outside RK stages)
    int el[NPT], node[NPT];
    bool has[NPT];
#pragma unroll
    for (int i = 0; i < NPT; ++i) {
      const int q = tid + i * BLOCK;
      el[i] = q / NN;
      node[i] = q - el[i] * NN;
      has[i] = q < nvalid;
    }
    // the connectivity, the face-node tables and the geometry are constant:
    // loaded before the wait for the previous kernel, so that the neighbour
    // values need one global round trip after it
    const AdvTables<DIM, N> &tab = g_adv_tables<DIM, N>;
    R outer[IPT];
    bool conforming[IPT];
    uint32_t item[IPT];
    int32_t nbs[IPT];
    const int32_t *ftb = p.face_table + e0 * (2 * DIM);
#pragma unroll
    for (int i = 0; i < IPT; ++i) {
      item[i] = 0;
      nbs[i] = 0;
      const int j = tid + i * BLOCK;
      if (j >= ivalid) continue;
      const int fe = j / FPE, r = j - fe * FPE;
      item[i] = __ldg(&tab.face[r]);
      nbs[i] = __ldg(ftb + fe * (2 * DIM) + ((item[i] >> 16) & 7));
    }
    double inv_jac_e[NPT], dt_e[NPT];
#pragma unroll
    for (int i = 0; i < NPT; ++i) {
      inv_jac_e[i] = 0.0;
      dt_e[i] = p.dt;
      if (has[i]) {
        inv_jac_e[i] = __ldg(p.inv_jac + e0 + el[i]);
        if (p.dt_elem) dt_e[i] = __ldg(p.dt_elem + e0 + el[i]);
      }
    }
    if (p.pdl) {
      asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
      asm volatile("griddepcontrol.wait;" ::: "memory");
    }
    // phase A: node values, and the outer values of the block's face nodes
    double ureg[NPT], kreg[NPT];
    R ui[NPT];
#pragma unroll
    for (int i = 0; i < NPT; ++i) {
      ureg[i] = 0.0;
      kreg[i] = 0.0;
      ui[i] = R(0);
      if (has[i]) {
        const int q = tid + i * BLOCK;
        ureg[i] = ub[q];
        if (use_k) kreg[i] = kb[q];
      }
    }
#pragma unroll
    for (int i = 0; i < IPT; ++i) {
      outer[i] = R(0);
      conforming[i] = true;
      const int j = tid + i * BLOCK;
      if (j >= ivalid) continue;
      const int32_t nb = nbs[i];
      if (nb >= 0) {
        outer[i] = narrow_hw(p.u_in[(int64_t)nb * NN + ((item[i] >> 8) & 255)]);
      } else {
        outer[i] = narrow_hw(p.mortar_flux[(int64_t)(-nb - 1) * NF + (item[i] >> 19)]);
        conforming[i] = false;
      }
    }
#pragma unroll
    for (int i = 0; i < NPT; ++i) {
      if (!has[i]) continue;
      // the FP64 pipe carries the neighbours' narrowing and the RK update
      // here, so the owner's value narrows on the integer pipe
      ui[i] = from_double<R>(ureg[i]);
      s_u[tid + i * BLOCK] = ui[i];
      if constexpr (sizeof(R) == 4) {
        // the element's scale, once per element (as phase A of the generic kernel)
        if (node[i] == 0) s_scale[el[i]] = from_double<R>(-inv_jac_e[i] * (mode == MODE_RK ? dt_e[i] : 1.0));
      }
    }
    __syncthreads();
    // phase B: the surface flux of every face node (the element's own value
    // on the inner side; a mortar face's flux comes from the mortar kernel)
    if (surface) {
      const int kind = p.surface_flux;
#pragma unroll
      for (int i = 0; i < IPT; ++i) {
        const int j = tid + i * BLOCK;
        if (j >= ivalid) continue;
        const int fe = j / FPE;
        R f = outer[i];
        if (conforming[i]) {
          const int face = (item[i] >> 16) & 7;
          const R own = s_u[fe * NN + (item[i] & 255)];
          const R a = p.pp.a[face >> 1];
          f = (face & 1) ? face_flux(kind, a, own, outer[i]) : face_flux(kind, a, outer[i], own);
        }
        s_f[j] = f;
      }
    }
    __syncthreads();
    // phase C, node by node
#pragma unroll
    for (int i = 0; i < NPT; ++i) {
      if (!has[i]) continue;
      constexpr int strides[3] = {1, N, N * N};
      int coord[3], tface[3];
      {
        const uint32_t nd = __ldg(&tab.node[node[i]]);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          coord[d] = (nd >> (4 * d)) & 15;
          tface[d] = (nd >> (12 + 6 * d)) & 63;
        }
      }
      R acc = R(0);
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        const int ci = coord[d];
        const R *row = s_op + ci * N;
        const R *line = s_u + (tid + i * BLOCK) - ci * strides[d];
        R sum = R(0);
        if constexpr (VOL == VOL_WEAK) {
#pragma unroll
          for (int m = 0; m < N; ++m) sum += row[m] * line[m * strides[d]];
          acc += p.pp.a[d] * sum;
        } else {
#pragma unroll
          for (int m = 0; m < N; ++m) {
            if (m == ci) continue;
            sum += row[m] * (ui[i] + line[m * strides[d]]);
          }
          acc += (R(0.5) * p.pp.a[d]) * sum;
        }
      }
      if (surface) {
        const R *fel = s_f + el[i] * FPE;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
          if (coord[d] == 0) acc -= p.lhat_l * fel[(2 * d) * NF + tface[d]];
          if (coord[d] == N - 1) acc += p.lhat_r * fel[(2 * d + 1) * NF + tface[d]];
        }
      }
      const int g = tid + i * BLOCK;  // block-relative node index
      if (mode == MODE_VOLUME) {
        ob[g] = to_double(acc);
        continue;
      }
      if constexpr (sizeof(R) == sizeof(double)) {
        const double du = double(acc) * -inv_jac_e[i];
        if (mode == MODE_RHS) {
          ob[g] = du;
        } else {
          const double kk = (use_k ? p.rk_a * kreg[i] : 0.0) + dt_e[i] * du;
          kb[g] = kk;
          ob[g] = ureg[i] + p.rk_b * kk;
        }
      } else {
        // mixed precision: scale in FP32, widen exactly, accumulate in FP64
        const double dd = to_double(acc * s_scale[el[i]]);
        if (mode == MODE_RHS) {
          ob[g] = dd;
        } else {
          const double kk = use_k ? fma(p.rk_a, kreg[i], dd) : dd;
          kb[g] = kk;
          ob[g] = fma(p.rk_b, kk, ureg[i]);
        }
      }
    }
  }
};

template <int DIM, int N, typename R, int VOL>
__global__ void __launch_bounds__(AdvKernel<DIM, N, R, VOL>::BLOCK) dg_adv_kernel(const FusedParams<R> p) {
  AdvKernel<DIM, N, R, VOL>::run(p);
}

// FP32-mixed: at least six resident blocks per SM (40 registers for the
// ~256-thread blocks; without the bound the polydeg-5 3D kind took 42 and lost
// a block): batched ensemble 5.25 -> 5.14 ms per step.  The FP64 kernels keep
// the plain bound (with six blocks they spill; no gain measured).
template <int DIM, int N, typename R, int VOL>
__global__ void __launch_bounds__(AdvKernel<DIM, N, R, VOL>::BLOCK, 6) dg_adv_kernel_f32(const FusedParams<R> p) {
  AdvKernel<DIM, N, R, VOL>::run(p);
}

template <int DIM, int N, typename R, int VOL>
constexpr auto adv_entry() {
  if constexpr (sizeof(R) == 4) return &dg_adv_kernel_f32<DIM, N, R, VOL>;
  else return &dg_adv_kernel<DIM, N, R, VOL>;
}

}  // namespace trixi
