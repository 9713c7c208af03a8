// dg_adjoint.cuh -- discrete adjoint of the fused rhs (FP64).
//
// The reference has no adjoint; this is the differentiation capability of the
// GB300 library.  For a reverse CarpenterKennedy2N54 stage s the kernel
// computes, with lam~ = lam_k + B_s lam_u,
//     lam_u_out = lam_u_in + dt * J_L(u)^T lam~,     lam_k_out = A_s lam~,
// i.e. the exact transpose of  k <- A_s k + dt L(u);  u <- u + B_s k.
// J_L(u)^T is applied with the forward kernel's structure: one thread per
// symmetric volume pair (reverse-mode derivative of the two-point flux with
// respect to both states) and one per element face, where the interface
// flux's cotangent gathers the adjoint of both elements that use it (the
// owning element only writes its own nodes: no scatter, no atomics).
//
// Supported: Euler with flux differencing (flux_ranocha / flux_central
// volume and surface fluxes) and linear advection (weak form or central flux
// differencing, LLF / central surface fluxes), conforming periodic meshes.
#pragma once
#include "dg_fused.cuh"

namespace trixi {

// ---- derivatives of the logarithmic means (same series / branches as forward)
__device__ __forceinline__ void ln_mean_grad(double x, double y, double r, double &L, double &dx, double &dy) {
  const double s = x + y, d = x - y, f = d * r, u = f * f;
  if (u < LnMeanThreshold<double>::value) {
    const double h = series_h(u);
    const double hp = series_h_du(u);
    L = 0.5 * s * h;
    dx = 0.5 * h + 2.0 * f * y * hp * r;
    dy = 0.5 * h - 2.0 * f * x * hp * r;
  } else {
    const double l = log(x * rcp_newton(y)), il = rcp_newton(l);
    L = d * il;
    dx = (1.0 - L * rcp_newton(x)) * il;
    dy = (L * rcp_newton(y) - 1.0) * il;
  }
}

__device__ __forceinline__ void inv_ln_mean_grad(double x, double y, double r, double &Q, double &dx, double &dy) {
  const double d = x - y, f = d * r, u = f * f;
  if (u < LnMeanThreshold<double>::value) {
    const double g = series_g(u);
    const double gp = series_g_du(u);
    Q = 2.0 * r * g;
    dx = -2.0 * r * r * g + 8.0 * f * y * r * r * r * gp;
    dy = -2.0 * r * r * g - 8.0 * f * x * r * r * r * gp;
  } else {
    const double l = log(x * rcp_newton(y)), id = rcp_newton(d);
    Q = l * id;
    dx = (rcp_newton(x) - Q) * id;
    dy = (Q - rcp_newton(y)) * id;
  }
}

template <int DIM, int EQ>
struct Adjoint;

// Linear advection: all Jacobians are constant.
template <int DIM>
struct Adjoint<DIM, EQ_ADV> {
  static constexpr int NV = 1;
  // cotangents of a two-point flux f(u_l, u_r) with respect to u_l and u_r
  template <int O>
  __device__ __forceinline__ static void two_point_vjp(int kind, const double *, const double *, double,
                                                      const double *, const double *, double, const double *g,
                                                      double *ul_bar, double *ur_bar, const PhysParams<double> &pp) {
    const double a = pp.a[O];
    // LLF with |a| and HLL with the signal speeds lmin = lmax = a are both the
    // upwind flux a u_upwind, so they share the upwind cotangents
    if (kind == FLUX_LLF || kind == FLUX_LLF_NAIVE || kind == FLUX_HLL) {
      ul_bar[0] = 0.5 * (a + fabs(a)) * g[0];
      ur_bar[0] = 0.5 * (a - fabs(a)) * g[0];
    } else {
      ul_bar[0] = 0.5 * a * g[0];
      ur_bar[0] = 0.5 * a * g[0];
    }
  }
  template <int O>
  __device__ __forceinline__ static void flux_vjp(const double *, const double *, const double *g, double *ubar,
                                                  const PhysParams<double> &pp) {
    ubar[0] = pp.a[O] * g[0];
  }
};

template <int DIM>
struct Adjoint<DIM, EQ_EULER> {
  static constexpr int NV = DIM + 2;

  // cotangent of the primitive state (rho, v, p) -> conservative state
  __device__ __forceinline__ static void prim_vjp(const double *w, double inv_rho, const double *wb, double *ub,
                                                  const PhysParams<double> &pp) {
    double kin = 0.0, vbv = 0.0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      kin += w[1 + d] * w[1 + d];
      vbv += wb[1 + d] * w[1 + d];
    }
    const double pb = wb[DIM + 1];
    ub[0] = wb[0] - vbv * inv_rho + pb * pp.gm1 * 0.5 * kin;
#pragma unroll
    for (int d = 0; d < DIM; ++d) ub[1 + d] = wb[1 + d] * inv_rho - pb * pp.gm1 * w[1 + d];
    ub[DIM + 1] = pb * pp.gm1;
  }

  // reverse mode of flux_ranocha in primitive variables
  template <int O>
  __device__ __forceinline__ static void ranocha_vjp(const double *wl, const double *wr, const double *g, double *wlb,
                                                     double *wrb, const PhysParams<double> &pp) {
    const double rl = wl[0], rr = wr[0], pl = wl[DIM + 1], pr = wr[DIM + 1];
    double L, dLl, dLr, Q, dQx, dQy;
    const double x2 = rl * pr, y2 = rr * pl;
    const double s1 = rl + rr, s2 = x2 + y2, qq = rcp_newton(s1 * s2);  // one reciprocal for both means
    ln_mean_grad(rl, rr, s2 * qq, L, dLl, dLr);
    inv_ln_mean_grad(x2, y2, s1 * qq, Q, dQx, dQy);
    const double ipm = pl * pr * Q;
    double va[DIM], v2 = 0.0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      va[d] = 0.5 * (wl[1 + d] + wr[1 + d]);
      v2 += wl[1 + d] * wr[1 + d];
    }
    v2 *= 0.5;
    const double f0 = L * va[O];
    const double gE = g[DIM + 1];
    double f0b = g[0] + gE * (v2 + ipm * pp.inv_gm1);
#pragma unroll
    for (int d = 0; d < DIM; ++d) f0b += g[1 + d] * va[d];
    double vab[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) vab[d] = g[1 + d] * f0;
    vab[O] += f0b * L;
    const double pab = g[1 + O];
    const double v2b = gE * f0;
    const double ipmb = gE * f0 * pp.inv_gm1;
    const double Lb = f0b * va[O];
    const double Qb = ipmb * pl * pr;
    const double x2b = Qb * dQx, y2b = Qb * dQy;
    wlb[0] = Lb * dLl + x2b * pr;
    wrb[0] = Lb * dLr + y2b * pl;
    wlb[DIM + 1] = 0.5 * gE * wr[1 + O] + 0.5 * pab + ipmb * pr * Q + y2b * rr;
    wrb[DIM + 1] = 0.5 * gE * wl[1 + O] + 0.5 * pab + ipmb * pl * Q + x2b * rl;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      wlb[1 + d] = 0.5 * vab[d] + 0.5 * v2b * wr[1 + d];
      wrb[1 + d] = 0.5 * vab[d] + 0.5 * v2b * wl[1 + d];
    }
    wlb[1 + O] += 0.5 * gE * pr;
    wrb[1 + O] += 0.5 * gE * pl;
  }

  // reverse mode of the physical flux f_O(u) with respect to u
  template <int O>
  __device__ __forceinline__ static void flux_vjp(const double *u, const double *w, const double *g, double *ub,
                                                  const PhysParams<double> &pp) {
    const double rho = w[0], p = w[DIM + 1], E = u[DIM + 1];
    double kin = 0.0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) kin += w[1 + d] * w[1 + d];
    const double p_rho = pp.gm1 * 0.5 * kin, p_E = pp.gm1;
    const double vo = w[1 + O];
    const double gE = g[DIM + 1];
    // f0 = m_o
    double ubr = 0.0, ubE = 0.0, ubm[DIM];
#pragma unroll
    for (int k = 0; k < DIM; ++k) ubm[k] = 0.0;
    ubm[O] += g[0];
    // f_{1+d} = m_o v_d + delta_{do} p
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      const double gd = g[1 + d];
      ubr += gd * (-vo * w[1 + d] + (d == O ? p_rho : 0.0));
      ubm[O] += gd * w[1 + d];
      ubm[d] += gd * vo;
      if (d == O) {
#pragma unroll
        for (int k = 0; k < DIM; ++k) ubm[k] += gd * (-pp.gm1 * w[1 + k]);
        ubE += gd * p_E;
      }
    }
    // f_E = (E + p) v_o
    ubr += gE * (p_rho * vo - (E + p) * vo / rho);
#pragma unroll
    for (int k = 0; k < DIM; ++k) ubm[k] += gE * (-pp.gm1 * w[1 + k] * vo);
    ubm[O] += gE * (E + p) / rho;
    ubE += gE * (1.0 + p_E) * vo;
    ub[0] = ubr;
#pragma unroll
    for (int k = 0; k < DIM; ++k) ub[1 + k] = ubm[k];
    ub[DIM + 1] = ubE;
  }

  // ul/ur: conservative, wl/wr: primitive states; irl/irr: 1/rho of each state
  template <int O>
  __device__ __forceinline__ static void two_point_vjp(int kind, const double *ul, const double *wl, double irl,
                                                      const double *ur, const double *wr, double irr,
                                                      const double *g, double *ulb, double *urb,
                                                      const PhysParams<double> &pp) {
    if (kind == FLUX_RANOCHA) {
      double wlb[NV], wrb[NV];
      ranocha_vjp<O>(wl, wr, g, wlb, wrb, pp);
      prim_vjp(wl, irl, wlb, ulb, pp);
      prim_vjp(wr, irr, wrb, urb, pp);
    } else {  // central: 1/2 (f(u_l) + f(u_r))
      double gh[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) gh[v] = 0.5 * g[v];
      flux_vjp<O>(ul, wl, gh, ulb, pp);
      flux_vjp<O>(ur, wr, gh, urb, pp);
    }
  }
};

struct AdjointParams {
  const double *__restrict__ u;        // state the stage's rhs was evaluated at
  const double *__restrict__ lu_in;    // lambda_u
  const double *__restrict__ lk_in;    // lambda_k
  double *__restrict__ lu_out;
  double *__restrict__ lk_out;
  const int32_t *__restrict__ face_table;
  const double *__restrict__ inv_jac;
  int64_t nelements;
  int surface_flux, volume_flux;
  double rk_a, rk_b, dt;               // mode VJP: rk_a = 0, rk_b = 0, dt = 1, lk_in = lambda
  PhysParams<double> pp;
  double dsplit[NMAXT * NMAXT];        // row-major, diagonal zeroed
  double dhat[NMAXT * NMAXT];
  double lhat_l, lhat_r;
  int pdl;      // launched as a programmatic dependent launch
  int u_ready;  // u does not depend on the previous kernel: read before griddepcontrol.wait
};

template <int DIM, int N, int EQ, int VOL>
struct AdjointKernel {
  using A = Adjoint<DIM, EQ>;
  using P = Physics<DIM, EQ, double>;
  static constexpr int NV = A::NV;
  static constexpr int NN = ipow(N, DIM);
  static constexpr int NF = ipow(N, DIM - 1);
  static constexpr int NP = N * (N - 1) / 2;
  static constexpr int VOL_PER_DIR = (VOL == VOL_WEAK) ? NN : NF * NP;
  static constexpr int VOL_BAR = (VOL == VOL_WEAK) ? 1 : 2;  // cotangent slots per volume item
  static constexpr int BLOCK = 256;
  static constexpr int ITEMS_PER_EL = DIM * VOL_PER_DIR + 2 * DIM * NF;
  static constexpr size_t smem_for(int epb) {
    return sizeof(double) * ((size_t)epb * (3 * NV * NN + NN + (DIM * VOL_PER_DIR * VOL_BAR + 2 * DIM * NF) * NV) +
                             epb + N * N);
  }
  static constexpr int epb_pick() {
    int e = (2 * BLOCK + ITEMS_PER_EL - 1) / ITEMS_PER_EL;
    if (e < 1) e = 1;
    if (e > 32) e = 32;
    while (e > 1 && smem_for(e) > 64 * 1024) --e;
    return e;
  }
  static constexpr int EPB = epb_pick();

  __device__ static void run(const AdjointParams &p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int epb = EPB;
    double *s_u = reinterpret_cast<double *>(smem_raw);      // [el][v][n]
    double *s_w = s_u + epb * NV * NN;
    double *s_l = s_w + epb * NV * NN;                         // lambda~ [el][v][n]
    double *s_vb = s_l + epb * NV * NN;                        // [el][dir][slot][VOL_BAR][v]
    double *s_sb = s_vb + epb * DIM * VOL_PER_DIR * VOL_BAR * NV;  // [el][face][t][v]
    double *s_ij = s_sb + epb * 2 * DIM * NF * NV;
    double *s_ir = s_ij + epb;                                 // 1/rho per node [el][n]
    double *s_D = s_ir + epb * NN;                             // D_hat (weak form) or D_split, row-major
    // the operator is read with a different (i, m) per lane: shared memory, not
    // the parameter (constant) bank, which serialises divergent reads
    for (int q = threadIdx.x; q < N * N; q += BLOCK) s_D[q] = (VOL == VOL_WEAK) ? p.dhat[q] : p.dsplit[q];
    const int64_t e0 = (int64_t)blockIdx.x * epb;
    if (e0 >= p.nelements) return;
    const int ne = (int)min((int64_t)epb, p.nelements - e0);
    auto U = [&](int el, int v, int n) -> double & { return s_u[(el * NV + v) * NN + n]; };
    auto W = [&](int el, int v, int n) -> double & { return s_w[(el * NV + v) * NN + n]; };
    auto Lm = [&](int el, int v, int n) -> double & { return s_l[(el * NV + v) * NN + n]; };

    // the stage's state, its primitive variables and 1/rho
    auto load_u = [&]() {
      for (int q = threadIdx.x; q < epb * NN; q += BLOCK) {
        const int el = q / NN, n = q - (q / NN) * NN;
        if (el >= ne) continue;
        const int64_t g0 = ((e0 + el) * NN + n) * NV;
        double uu[NV], ww[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) uu[v] = p.u[g0 + v];
        P::prim(uu, ww, p.pp);
        s_ir[el * NN + n] = rcp_newton(uu[0]);
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          U(el, v, n) = uu[v];
          W(el, v, n) = ww[v];
        }
      }
    };
    if (threadIdx.x < ne) s_ij[threadIdx.x] = p.inv_jac[e0 + threadIdx.x];
    if (p.pdl) {
      // programmatic dependent launch: the next stage kernel may start
      // launching; the cotangents (the previous kernel's output) are read
      // only after the wait.  A stored stage state (u_ready) does not depend
      // on the previous kernel, so its loads and FP64 work overlap that
      // kernel's tail.
      asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
      if (p.u_ready) load_u();
      asm volatile("griddepcontrol.wait;" ::: "memory");
      if (!p.u_ready) load_u();
    } else {
      load_u();
    }
    for (int q = threadIdx.x; q < epb * NN; q += BLOCK) {
      const int el = q / NN, n = q - (q / NN) * NN;
      if (el >= ne) continue;
      const int64_t g0 = ((e0 + el) * NN + n) * NV;
#pragma unroll
      for (int v = 0; v < NV; ++v) Lm(el, v, n) = p.lk_in[g0 + v] + (p.lu_in ? p.rk_b * p.lu_in[g0 + v] : 0.0);
    }
    __syncthreads();

    constexpr int PER_VOL = epb * VOL_PER_DIR;
    constexpr int PER_SURF = epb * 2 * NF;
    constexpr int N_VOL = DIM * PER_VOL;
    constexpr int N_ALL = N_VOL + DIM * PER_SURF;
    for (int w = threadIdx.x; w < N_ALL; w += BLOCK) {
      if (w < N_VOL) {
        const int dir = w / PER_VOL;
        const int r0 = w - dir * PER_VOL;
        const int el = r0 / VOL_PER_DIR, r = r0 - (r0 / VOL_PER_DIR) * VOL_PER_DIR;
        if (el >= ne) continue;
        if (dir == 0) vol_item<0>(p, el, r, s_u, s_w, s_l, s_vb, s_ij, s_ir);
        if constexpr (DIM > 1) if (dir == 1) vol_item<1>(p, el, r, s_u, s_w, s_l, s_vb, s_ij, s_ir);
        if constexpr (DIM > 2) if (dir == 2) vol_item<2>(p, el, r, s_u, s_w, s_l, s_vb, s_ij, s_ir);
      } else {
        const int w2 = w - N_VOL;
        const int dir = w2 / PER_SURF;
        const int r0 = w2 - dir * PER_SURF;
        const int el = r0 / (2 * NF);
        const int r1 = r0 - el * (2 * NF);
        const int side = r1 / NF, t = r1 - (r1 / NF) * NF;
        if (el >= ne) continue;
        if (dir == 0) surf_item<0>(p, e0, el, side, t, s_u, s_w, s_l, s_sb, s_ij, s_ir);
        if constexpr (DIM > 1) if (dir == 1) surf_item<1>(p, e0, el, side, t, s_u, s_w, s_l, s_sb, s_ij, s_ir);
        if constexpr (DIM > 2) if (dir == 2) surf_item<2>(p, e0, el, side, t, s_u, s_w, s_l, s_sb, s_ij, s_ir);
      }
    }
    __syncthreads();

    for (int q = threadIdx.x; q < epb * NN; q += BLOCK) {
      const int el = q / NN, node = q - (q / NN) * NN;
      if (el >= ne) continue;
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
      // cotangents of the node: conservative (ub) and primitive-variable (pb,
      // from flux_ranocha items, mapped to conservative once below)
      double ub[NV], pb[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) ub[v] = pb[v] = 0.0;
      double *vacc = ub, *sacc = ub;
      if constexpr (EQ == EQ_EULER) {
        if (VOL != VOL_WEAK && p.volume_flux == FLUX_RANOCHA) vacc = pb;
        if (p.surface_flux == FLUX_RANOCHA) sacc = pb;
      }
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        const int ci = coord[d];
        if constexpr (VOL == VOL_WEAK) {
          const double *B = s_vb + ((el * DIM + d) * VOL_PER_DIR + node) * NV;
#pragma unroll
          for (int v = 0; v < NV; ++v) vacc[v] += B[v];
        } else {
#pragma unroll
          for (int m = 0; m < N; ++m) {
            if (m == ci) continue;
            const int pidx = tface[d] * NP + pair_index<N>(ci, m);
            // the pair stores (i<m): slot 0 = cotangent of its left state, 1 = right
            const double *B = s_vb + (((el * DIM + d) * VOL_PER_DIR + pidx) * 2 + (ci < m ? 0 : 1)) * NV;
#pragma unroll
            for (int v = 0; v < NV; ++v) vacc[v] += B[v];
          }
        }
        if (ci == 0) {
          const double *B = s_sb + ((el * 2 * DIM + 2 * d) * NF + tface[d]) * NV;
#pragma unroll
          for (int v = 0; v < NV; ++v) sacc[v] += B[v];
        }
        if (ci == N - 1) {
          const double *B = s_sb + ((el * 2 * DIM + 2 * d + 1) * NF + tface[d]) * NV;
#pragma unroll
          for (int v = 0; v < NV; ++v) sacc[v] += B[v];
        }
      }
      if constexpr (EQ == EQ_EULER) {
        if (vacc == pb || sacc == pb) {
          double w[NV], cb[NV];
#pragma unroll
          for (int v = 0; v < NV; ++v) w[v] = W(el, v, node);
          A::prim_vjp(w, s_ir[el * NN + node], pb, cb, p.pp);
#pragma unroll
          for (int v = 0; v < NV; ++v) ub[v] += cb[v];
        }
      }
      const int64_t g0 = ((e0 + el) * NN + node) * NV;
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        const double lt = Lm(el, v, node);
        p.lu_out[g0 + v] = (p.lu_in ? p.lu_in[g0 + v] : 0.0) + p.dt * ub[v];
        if (p.lk_out) p.lk_out[g0 + v] = p.rk_a * lt;
      }
    }
  }

  template <int O>
  __device__ __forceinline__ static void vol_item(const AdjointParams &p, int el, int r, double *s_u, double *s_w,
                                                  double *s_l, double *s_vb, const double *s_ij, const double *s_ir) {
    const double scale = -s_ij[el];
    const double *s_D = s_ir + EPB * NN;
    if constexpr (VOL == VOL_WEAK) {
      // du_i = -J^{-1} sum_m dhat[i,m] f(u_m): cotangent of f(u_r) gathers the column r of dhat
      const int ci = (r / ipow(N, O)) % N;
      const int stride = ipow(N, O);
      const int n0 = r - ci * stride;
      double g[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        double a = 0.0;
#pragma unroll
        for (int i = 0; i < N; ++i) a += s_D[i * N + ci] * s_l[(el * NV + v) * NN + n0 + i * stride];
        g[v] = scale * a;
      }
      double u[NV], w[NV], ub[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        u[v] = s_u[(el * NV + v) * NN + r];
        w[v] = s_w[(el * NV + v) * NN + r];
      }
      A::template flux_vjp<O>(u, w, g, ub, p.pp);
      double *dst = s_vb + ((el * DIM + O) * VOL_PER_DIR + r) * NV;
#pragma unroll
      for (int v = 0; v < NV; ++v) dst[v] = ub[v];
    } else {
      const int t = r / NP, pp_ = r - (r / NP) * NP;
      int i, m;
      pair_nodes<N>(pp_, i, m);
      const int ni = line_node<DIM, N, O>(t, i), nm = line_node<DIM, N, O>(t, m);
      const double dim_ = s_D[i * N + m], dmi = s_D[m * N + i];
      double g[NV], ui[NV], wi[NV], um[NV], wm[NV], bi[NV], bm[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        g[v] = scale * (dim_ * s_l[(el * NV + v) * NN + ni] + dmi * s_l[(el * NV + v) * NN + nm]);
        ui[v] = s_u[(el * NV + v) * NN + ni];
        wi[v] = s_w[(el * NV + v) * NN + ni];
        um[v] = s_u[(el * NV + v) * NN + nm];
        wm[v] = s_w[(el * NV + v) * NN + nm];
      }
      if constexpr (EQ == EQ_EULER) {
        if (p.volume_flux == FLUX_RANOCHA) {
          // primitive-variable cotangents: the node phase sums them over the
          // pairs and maps the sum to conservative variables once per node
          // (the map is linear in the cotangent)
          A::template ranocha_vjp<O>(wi, wm, g, bi, bm, p.pp);
        } else {
          A::template two_point_vjp<O>(p.volume_flux, ui, wi, s_ir[el * NN + ni], um, wm, s_ir[el * NN + nm], g, bi,
                                       bm, p.pp);
        }
      } else {
        A::template two_point_vjp<O>(p.volume_flux, ui, wi, s_ir[el * NN + ni], um, wm, s_ir[el * NN + nm], g, bi, bm,
                                     p.pp);
      }
      double *dst = s_vb + ((el * DIM + O) * VOL_PER_DIR + r) * 2 * NV;
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        dst[v] = bi[v];
        dst[NV + v] = bm[v];
      }
    }
  }

  template <int O>
  __device__ __forceinline__ static void surf_item(const AdjointParams &p, int64_t e0, int el, int side, int t,
                                                   double *s_u, double *s_w, double *s_l, double *s_sb,
                                                   const double *s_ij, const double *s_ir) {
    const int64_t e = e0 + el;
    const int32_t nb = p.face_table[e * (2 * DIM) + 2 * O + side];
    const int own = line_node<DIM, N, O>(t, side == 0 ? 0 : N - 1);
    const int other = line_node<DIM, N, O>(t, side == 0 ? N - 1 : 0);
    const double *un_g = p.u + ((int64_t)nb * NN + other) * NV;
    const double *lk_g = p.lk_in + ((int64_t)nb * NN + other) * NV;
    const double ij_own = s_ij[el], ij_nb = p.inv_jac[nb];
    double un[NV], wn[NV], uo[NV], wo[NV], g[NV], bl[NV], br[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      un[v] = un_g[v];
      uo[v] = s_u[(el * NV + v) * NN + own];
      wo[v] = s_w[(el * NV + v) * NN + own];
      const double lnb = lk_g[v] + (p.lu_in ? p.rk_b * p.lu_in[((int64_t)nb * NN + other) * NV + v] : 0.0);
      const double lown = s_l[(el * NV + v) * NN + own];
      // side 0: du_own += J_own lhat_l f*, du_nb(other) -= J_nb lhat_r f*
      // side 1: du_own -= J_own lhat_r f*, du_nb(other) += J_nb lhat_l f*
      g[v] = (side == 0) ? (ij_own * p.lhat_l * lown - ij_nb * p.lhat_r * lnb)
                         : (-ij_own * p.lhat_r * lown + ij_nb * p.lhat_l * lnb);
    }
    P::prim(un, wn, p.pp);
    const double irn = rcp_newton(un[0]), iro = s_ir[el * NN + own];
    double *dst = s_sb + ((el * 2 * DIM + 2 * O + side) * NF + t) * NV;
    if constexpr (EQ == EQ_EULER) {
      if (p.surface_flux == FLUX_RANOCHA) {
        // the owner's primitive-variable cotangent (mapped once per node)
        if (side == 0)
          A::template ranocha_vjp<O>(wn, wo, g, bl, br, p.pp);
        else
          A::template ranocha_vjp<O>(wo, wn, g, bl, br, p.pp);
#pragma unroll
        for (int v = 0; v < NV; ++v) dst[v] = side == 0 ? br[v] : bl[v];
        return;
      }
    }
    if (side == 0) {
      A::template two_point_vjp<O>(p.surface_flux, un, wn, irn, uo, wo, iro, g, bl, br, p.pp);
#pragma unroll
      for (int v = 0; v < NV; ++v) dst[v] = br[v];
    } else {
      A::template two_point_vjp<O>(p.surface_flux, uo, wo, iro, un, wn, irn, g, bl, br, p.pp);
#pragma unroll
      for (int v = 0; v < NV; ++v) dst[v] = bl[v];
    }
  }
};

template <int DIM, int N, int EQ, int VOL>
__global__ void __launch_bounds__(256) dg_adjoint_kernel(const AdjointParams p) {
  AdjointKernel<DIM, N, EQ, VOL>::run(p);
}

}  // namespace trixi
