// dg_analysis.cu -- GPU replacements of the reference's host-side callback
// loops and of its initial-condition kernel:
//   max_dt            src/callbacks_step/stepsize_dg_{1,2,3}d.jl (copies u to the host every step)
//   integrals         src/callbacks_step/analysis_dg_2d.jl:1-40 (integrate_via_indices)
//   calc_error_norms  src/callbacks_step/analysis_dg_2d.jl:44-89 (interpolation to
//                     2*polydeg+1 LGL analysis nodes, L2 and Linf)
//   initial condition src/solvers/dg.jl:46-160 (compute_coefficients_kernel!,
//                     including the 1D endpoint nudge of dg.jl:54-57)
// Reductions are deterministic: per-element partials, then one block that
// sums them in a fixed order.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <mutex>

#include "../../include/trixi_b200.h"
#include "basis.h"
#include "dg_analysis.h"
#include "dg_host.h"
#include "dg_ic.cuh"
#include "dg_physics.cuh"

namespace trixi {

namespace {

template <int DIM>
__device__ __forceinline__ int nodes_per_elem(int N) {
  return DIM == 1 ? N : (DIM == 2 ? N * N : N * N * N);
}

// ---------------------------------------------------------------------------
// max_dt: 2 / (N * max_e invJ_e * sum_d max_nodes lambda_d)
// ---------------------------------------------------------------------------
template <int DIM, int EQ>
__global__ void max_speed_kernel(int N, int64_t E, const double *__restrict__ u, const double *__restrict__ inv_jac,
                                 double gamma, double a0, double a1, double a2,
                                 unsigned long long *__restrict__ acc) {
  constexpr int NV = NVarsOf<DIM, EQ>::value;
  const int64_t e = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (e >= E) return;
  const int NN = nodes_per_elem<DIM>(N);
  double lam[3] = {0.0, 0.0, 0.0};
  if (EQ == EQ_ADV) {
    lam[0] = fabs(a0);
    lam[1] = fabs(a1);
    lam[2] = fabs(a2);
  } else if (EQ == EQ_MHD) {
    // ideal GLM-MHD: |v_d| + the fast magnetosonic speed along d
    for (int n = lane; n < NN; n += 32) {
      const double *un = u + (e * NN + n) * NV;
      const double rho = un[0];
      double kin = 0.0, mag = 0.0, v[3];
      for (int d = 0; d < 3; ++d) {
        v[d] = un[1 + d] / rho;
        kin += un[1 + d] * v[d];
        mag += un[5 + d] * un[5 + d];
      }
      const double psi2 = (NV == 9) ? un[NV - 1] * un[NV - 1] : 0.0;
      const double p = (gamma - 1.0) * (un[4] - 0.5 * kin - 0.5 * mag - 0.5 * psi2);
      const double a2 = gamma * p / rho, b2 = mag / rho;
      for (int d = 0; d < DIM; ++d) {
        const double bd2 = un[5 + d] * un[5 + d] / rho;
        const double cf = sqrt(0.5 * (a2 + b2 + sqrt((a2 + b2) * (a2 + b2) - 4.0 * a2 * bd2)));
        lam[d] = fmax(lam[d], fabs(v[d]) + cf);
      }
    }
    for (int off = 16; off > 0; off >>= 1)
      for (int d = 0; d < DIM; ++d) lam[d] = fmax(lam[d], __shfl_xor_sync(0xffffffffu, lam[d], off));
  } else {
    for (int n = lane; n < NN; n += 32) {
      const double *un = u + (e * NN + n) * NV;
      const double rho = un[0];
      double kin = 0.0, v[3];
      for (int d = 0; d < DIM; ++d) {
        v[d] = un[1 + d] / rho;
        kin += un[1 + d] * v[d];
      }
      const double p = (gamma - 1.0) * (un[DIM + 1] - 0.5 * kin);
      const double c = sqrt(gamma * p / rho);
      for (int d = 0; d < DIM; ++d) lam[d] = fmax(lam[d], fabs(v[d]) + c);
    }
    for (int off = 16; off > 0; off >>= 1)
      for (int d = 0; d < DIM; ++d) lam[d] = fmax(lam[d], __shfl_xor_sync(0xffffffffu, lam[d], off));
  }
  if (lane == 0) {
    double s = 0.0;
    for (int d = 0; d < DIM; ++d) s += lam[d];
    const double scaled = inv_jac[e] * s;
    // non-negative doubles order like their bit patterns
    atomicMax(acc, (unsigned long long)__double_as_longlong(scaled));
  }
}

__global__ void max_dt_finalize(int N, const unsigned long long *acc, double *dt) {
  double m = __longlong_as_double((long long)*acc);
  if (!(m > 0.0)) m = 4.9406564584124654e-324;  // nextfloat(0): no division by zero
  *dt = 2.0 / (N * m);
}

// ---------------------------------------------------------------------------
// integrals: per element sum_nodes (prod_d w) * J * q(u, du)
// ---------------------------------------------------------------------------
template <int DIM, int EQ>
__device__ void quantity(int which, const double *un, const double *dun, double gamma, double *q) {
  constexpr int NV = NVarsOf<DIM, EQ>::value;
  if (which == 0) {  // conserved variables
    for (int v = 0; v < NV; ++v) q[v] = un[v];
    return;
  }
  if (which == 3) {  // du
    for (int v = 0; v < NV; ++v) q[v] = dun[v];
    return;
  }
  if (EQ == EQ_ADV) {
    if (which == 1) q[0] = 0.5 * un[0] * un[0];  // entropy 1/2 u^2
    else q[0] = un[0] * dun[0];                  // entropy variable u times du
    return;
  }
  if (EQ == EQ_MHD) {
    // ideal GLM-MHD: S = -rho s/(gamma-1) with the MHD pressure; entropy
    // variables ((gamma-s)/(gamma-1) - beta|v|^2, 2 beta v, -2 beta, 2 beta B,
    // 2 beta psi), beta = rho/(2p) (Derigs et al., JCP 364 (2018))
    const double rho = un[0];
    double kin = 0.0, mag = 0.0, v[3];
    for (int d = 0; d < 3; ++d) {
      v[d] = un[1 + d] / rho;
      kin += un[1 + d] * v[d];
      mag += un[5 + d] * un[5 + d];
    }
    const double psi = (NV == 9) ? un[NV - 1] : 0.0;
    const double p = (gamma - 1.0) * (un[4] - 0.5 * kin - 0.5 * mag - 0.5 * psi * psi);
    const double s = log(p) - gamma * log(rho);
    if (which == 1) {
      q[0] = -rho * s / (gamma - 1.0);
      return;
    }
    const double rho_p = rho / p;  // 2 beta
    double acc = ((gamma - s) / (gamma - 1.0) - 0.5 * rho_p * kin / rho) * dun[0];
    for (int d = 0; d < 3; ++d) acc += rho_p * (v[d] * dun[1 + d] + un[5 + d] * dun[5 + d]);
    acc += -rho_p * dun[4];
    if (NV == 9) acc += rho_p * psi * dun[NV - 1];
    q[0] = acc;
    return;
  }
  const double rho = un[0];
  double kin = 0.0, v[3];
  for (int d = 0; d < DIM; ++d) {
    v[d] = un[1 + d] / rho;
    kin += un[1 + d] * v[d];
  }
  const double p = (gamma - 1.0) * (un[DIM + 1] - 0.5 * kin);
  const double s = log(p) - gamma * log(rho);
  if (which == 1) {  // mathematical entropy -rho s / (gamma - 1)
    q[0] = -rho * s / (gamma - 1.0);
    return;
  }
  // entropy production: w(u) . du with the entropy variables w
  const double rho_p = rho / p;
  double wv = (gamma - s) / (gamma - 1.0) - 0.5 * rho_p * kin / rho;
  double acc = wv * dun[0];
  for (int d = 0; d < DIM; ++d) acc += rho_p * v[d] * dun[1 + d];
  acc += -rho_p * dun[DIM + 1];
  q[0] = acc;
}

// Compensated (double-double) accumulation for the quadrature integrals:
// error-free TwoSum (Knuth) and TwoProduct (by FMA) keep the rounding errors
// of every product and partial sum in a second word, so conservation and
// entropy integrals, sums of terms that cancel, come out correct to the last
// bits instead of to the size of the largest term (Ogita, Rump, Oishi, "Accurate
// sum and dot product", SIAM J. Sci. Comput. 26 (2005)).
struct Dd {
  double hi, lo;
};
__device__ __forceinline__ void two_sum(double a, double b, double &s, double &e) {
  s = __dadd_rn(a, b);
  const double bp = __dsub_rn(s, a);
  e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bp)), __dsub_rn(b, bp));
}
__device__ __forceinline__ void dd_add(Dd &acc, double x) {  // acc += x
  double s, e;
  two_sum(acc.hi, x, s, e);
  acc.hi = s;
  acc.lo = __dadd_rn(acc.lo, e);
}
__device__ __forceinline__ void dd_add_prod(Dd &acc, double a, double b) {  // acc += a b
  const double p = __dmul_rn(a, b);
  const double pe = fma(a, b, -p);  // exact error of the product
  dd_add(acc, p);
  acc.lo = __dadd_rn(acc.lo, pe);
}
__device__ __forceinline__ void dd_merge(Dd &acc, const Dd &o) {
  double s, e;
  two_sum(acc.hi, o.hi, s, e);
  acc.hi = s;
  acc.lo = __dadd_rn(__dadd_rn(acc.lo, o.lo), e);
}
// a warp-wide compensated sum, the result in every lane
__device__ __forceinline__ Dd dd_warp_sum(Dd v) {
  for (int off = 16; off > 0; off >>= 1) {
    Dd o;
    o.hi = __shfl_xor_sync(0xffffffffu, v.hi, off);
    o.lo = __shfl_xor_sync(0xffffffffu, v.lo, off);
    dd_merge(v, o);
  }
  return v;
}

template <int DIM, int EQ>
__global__ void integrate_kernel(int N, int64_t E, const double *__restrict__ u, const double *__restrict__ du,
                                 const double *__restrict__ inv_jac, const double *__restrict__ w, int which,
                                 int nq, double gamma, double *__restrict__ partial) {
  constexpr int NV = NVarsOf<DIM, EQ>::value;
  const int64_t e = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (e >= E) return;
  const int NN = nodes_per_elem<DIM>(N);
  Dd acc[NV];
  for (int k = 0; k < NV; ++k) acc[k] = Dd{0.0, 0.0};
  for (int n = lane; n < NN; n += 32) {
    int r = n;
    double wt = 1.0;
    for (int d = 0; d < DIM; ++d) {
      wt *= w[r % N];
      r /= N;
    }
    double q[NV];
    quantity<DIM, EQ>(which, u + (e * NN + n) * NV, du ? du + (e * NN + n) * NV : nullptr, gamma, q);
    for (int k = 0; k < nq; ++k) dd_add_prod(acc[k], wt, q[k]);
  }
  double J = 1.0;
  for (int d = 0; d < DIM; ++d) J /= inv_jac[e];
  for (int k = 0; k < nq; ++k) {
    const Dd v = dd_warp_sum(acc[k]);
    if (lane == 0) partial[e * nq + k] = fma(J, v.hi, J * v.lo);
  }
}

struct WeightsArg {
  double w[16];
};

// integrate_kernel with the quadrature weights passed by value (no device copy of them needed)
template <int DIM, int EQ>
__global__ void integrate_w_kernel(int N, int64_t E, const double *__restrict__ u, const double *__restrict__ du,
                                   const double *__restrict__ inv_jac, WeightsArg wa, int which, int nq, double gamma,
                                   double *__restrict__ partial) {
  constexpr int NV = NVarsOf<DIM, EQ>::value;
  const int64_t e = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (e >= E) return;
  const int NN = nodes_per_elem<DIM>(N);
  Dd acc[NV];
  for (int k = 0; k < NV; ++k) acc[k] = Dd{0.0, 0.0};
  for (int n = lane; n < NN; n += 32) {
    int r = n;
    double wt = 1.0;
    for (int d = 0; d < DIM; ++d) {
      wt *= wa.w[r % N];
      r /= N;
    }
    double q[NV];
    quantity<DIM, EQ>(which, u + (e * NN + n) * NV, du ? du + (e * NN + n) * NV : nullptr, gamma, q);
    for (int k = 0; k < nq; ++k) dd_add_prod(acc[k], wt, q[k]);
  }
  double J = 1.0;
  for (int d = 0; d < DIM; ++d) J /= inv_jac[e];
  for (int k = 0; k < nq; ++k) {
    const Dd v = dd_warp_sum(acc[k]);
    if (lane == 0) partial[e * nq + k] = fma(J, v.hi, J * v.lo);
  }
}

// one block: deterministic compensated sum (op 0) or max (op 1) of
// partial[E][nq] per column
__global__ void reduce_columns(int64_t E, int nq, const double *__restrict__ partial, int op, double *__restrict__ out) {
  __shared__ double sm_hi[1024], sm_lo[1024];
  for (int k = 0; k < nq; ++k) {
    Dd v{0.0, 0.0};
    for (int64_t e = threadIdx.x; e < E; e += blockDim.x) {
      const double x = partial[e * nq + k];
      if (op == 0) dd_add(v, x);
      else v.hi = fmax(v.hi, x);
    }
    sm_hi[threadIdx.x] = v.hi;
    sm_lo[threadIdx.x] = v.lo;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) {
        if (op == 0) {
          Dd a{sm_hi[threadIdx.x], sm_lo[threadIdx.x]};
          dd_merge(a, Dd{sm_hi[threadIdx.x + s], sm_lo[threadIdx.x + s]});
          sm_hi[threadIdx.x] = a.hi;
          sm_lo[threadIdx.x] = a.lo;
        } else {
          sm_hi[threadIdx.x] = fmax(sm_hi[threadIdx.x], sm_hi[threadIdx.x + s]);
        }
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) out[k] = (op == 0) ? sm_hi[0] + sm_lo[0] : sm_hi[0];
    __syncthreads();
  }
}

// initial conditions: eval_ic (dg_ic.cuh)
// one ulp towards +inf / -inf for finite x (IEEE-754 bit-pattern order)
__device__ __forceinline__ double next_up(double x) {
  if (x == 0.0) return 4.9406564584124654e-324;
  const long long b = __double_as_longlong(x);
  return __longlong_as_double(x > 0.0 ? b + 1 : b - 1);
}
__device__ __forceinline__ double next_down(double x) { return -next_up(-x); }

template <int DIM, int EQ>
__global__ void ic_kernel(int N, int64_t E, const double *__restrict__ coords, int kind, IcParams ip, double t,
                          double *__restrict__ u) {
  constexpr int NV = NVarsOf<DIM, EQ>::value;
  const int NN = nodes_per_elem<DIM>(N);
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= E * NN) return;
  double x[3] = {0.0, 0.0, 0.0};
  for (int d = 0; d < DIM; ++d) x[d] = coords[idx * DIM + d];
  if (DIM == 1) {
    // the reference moves the element end points one ulp inwards (dg.jl:54-57)
    const int n = (int)(idx % NN);
    if (n == 0) x[0] = next_up(x[0]);
    if (n == N - 1) x[0] = next_down(x[0]);
  }
  double uu[NV];
  eval_ic<DIM, EQ>(kind, x, t, ip, uu);
  for (int v = 0; v < NV; ++v) u[idx * NV + v] = uu[v];
}

// ---------------------------------------------------------------------------
// error norms: one block per element, interpolation to NA analysis nodes
// ---------------------------------------------------------------------------
template <int DIM, int EQ>
__global__ void error_norms_kernel(int N, int NA, int64_t E, const double *__restrict__ u,
                                   const double *__restrict__ uref, const double *__restrict__ coords, int kind,
                                   IcParams ip, double t, const double *__restrict__ vdm /* [NA][N] */,
                                   const double *__restrict__ wa, const double *__restrict__ inv_jac,
                                   double *__restrict__ l2p, double *__restrict__ linfp) {
  constexpr int NV = NVarsOf<DIM, EQ>::value;
  extern __shared__ __align__(16) double sm[];
  const int64_t e = blockIdx.x;
  if (e >= E) return;
  const int NN = nodes_per_elem<DIM>(N);
  int NNA = NA;
  for (int d = 1; d < DIM; ++d) NNA *= NA;
  // buffers sized for the largest intermediate, NA^DIM * NV each:
  // b0 = u at the analysis nodes, b1 = reference state there, b2 = scratch
  double *b0 = sm, *b1 = sm + NNA * NV, *b2 = sm + 2 * NNA * NV;
  double *sl2 = b2 + NNA * NV;         // [blockDim][NV]
  double *slinf = sl2 + blockDim.x * NV;
  // element geometry (affine): first and last node coordinates
  double xlo[3], xhi[3];
  for (int d = 0; d < DIM; ++d) {
    xlo[d] = coords[(e * NN) * DIM + d];
    int stride = 1;
    for (int dd = 0; dd < d; ++dd) stride *= N;
    xhi[d] = coords[(e * NN + (N - 1) * stride) * DIM + d];
  }
  for (int pass = 0; pass < (uref ? 2 : 1); ++pass) {
    const double *src = pass == 0 ? u : uref;
    double *dst = pass == 0 ? b0 : b1;
    // stage element values in scratch as [v][n] (n over N^DIM)
    double *tmp = b2;
    for (int i = threadIdx.x; i < NN * NV; i += blockDim.x) {
      const int n = i / NV, v = i - (i / NV) * NV;
      tmp[v * NNA + n] = src[(e * NN + n) * NV + v];
    }
    __syncthreads();
    // dimension by dimension: sizes go from N^DIM to NA^DIM
    int cur[3] = {N, N, N};
    double *in = tmp, *outp = dst;
    for (int d = 0; d < DIM; ++d) {
      int nin = 1, nout = 1;
      for (int dd = 0; dd < DIM; ++dd) {
        nin *= cur[dd];
        nout *= (dd == d ? NA : cur[dd]);
      }
      int stride = 1;
      for (int dd = 0; dd < d; ++dd) stride *= cur[dd];
      for (int i = threadIdx.x; i < nout * NV; i += blockDim.x) {
        const int v = i / nout, n = i - (i / nout) * nout;
        const int c = (n / stride) % NA;
        const int hi = n / (stride * NA), lo = n % stride;
        double s = 0.0;
        for (int m = 0; m < N; ++m) s += vdm[c * N + m] * in[v * NNA + lo + stride * (m + cur[d] * hi)];
        outp[v * NNA + n] = s;
      }
      __syncthreads();
      cur[d] = NA;
      double *sw = in;
      in = outp;
      outp = sw;
    }
    if (in != dst) {
      for (int i = threadIdx.x; i < NNA * NV; i += blockDim.x) dst[i] = in[i];
      __syncthreads();
    }
  }
  double J = 1.0;
  for (int d = 0; d < DIM; ++d) J /= inv_jac[e];
  double l2[NV], linf[NV];
  for (int v = 0; v < NV; ++v) l2[v] = linf[v] = 0.0;
  for (int n = threadIdx.x; n < NNA; n += blockDim.x) {
    double x[3] = {0, 0, 0};
    double wt = J;
    int r = n;
    for (int d = 0; d < DIM; ++d) {
      const int c = r % NA;
      r /= NA;
      wt *= wa[c];
      // affine position of analysis node c (nodes on [-1, 1] come from vdm's row sums)
      x[d] = xlo[d] + 0.5 * (xhi[d] - xlo[d]) * (ip.xa[c] + 1.0);
    }
    double ex[NV];
    if (uref) {
      for (int v = 0; v < NV; ++v) ex[v] = b1[v * NNA + n];
    } else {
      eval_ic<DIM, EQ>(kind, x, t, ip, ex);
    }
    for (int v = 0; v < NV; ++v) {
      const double diff = ex[v] - b0[v * NNA + n];
      l2[v] += diff * diff * wt;
      linf[v] = fmax(linf[v], fabs(diff));
    }
  }
  for (int v = 0; v < NV; ++v) {
    sl2[threadIdx.x * NV + v] = l2[v];
    slinf[threadIdx.x * NV + v] = linf[v];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int v = 0; v < NV; ++v) {
      double a = 0.0, b = 0.0;
      for (int i = 0; i < (int)blockDim.x; ++i) {
        a += sl2[i * NV + v];
        b = fmax(b, slinf[i * NV + v]);
      }
      l2p[e * NV + v] = a;
      linfp[e * NV + v] = b;
    }
  }
}

template <int DIM, int EQ>
cudaError_t launch_error_norms(const ErrorNormHost &h, cudaStream_t s) {
  constexpr int NV = NVarsOf<DIM, EQ>::value;
  int NNA = h.NA;
  for (int d = 1; d < DIM; ++d) NNA *= h.NA;
  const int block = 128;
  const size_t smem = sizeof(double) * ((size_t)3 * NNA * NV + (size_t)2 * block * NV);
  static const cudaError_t attr = cudaFuncSetAttribute(error_norms_kernel<DIM, EQ>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  if (attr != cudaSuccess) return attr;
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  error_norms_kernel<DIM, EQ><<<(unsigned)h.E, block, smem, s>>>(h.N, h.NA, h.E, h.u, h.uref, h.coords, h.kind,
                                                                 h.ip, h.t, h.vdm, h.wa, h.inv_jac, h.l2p, h.linfp);
  return cudaGetLastError();
}

}  // namespace

#define TRIXI_DISPATCH(dim, eq, call)                                 \
  do {                                                                \
    if ((dim) == 1) {                                                 \
      if ((eq) == EQ_ADV) { constexpr int D_ = 1, Q_ = EQ_ADV; call; } \
      else { constexpr int D_ = 1, Q_ = EQ_EULER; call; }             \
    } else if ((dim) == 2) {                                          \
      if ((eq) == EQ_ADV) { constexpr int D_ = 2, Q_ = EQ_ADV; call; } \
      else { constexpr int D_ = 2, Q_ = EQ_EULER; call; }             \
    } else {                                                          \
      if ((eq) == EQ_ADV) { constexpr int D_ = 3, Q_ = EQ_ADV; call; } \
      else { constexpr int D_ = 3, Q_ = EQ_EULER; call; }             \
    }                                                                 \
  } while (0)

// the same with ideal GLM-MHD (max_dt and the integrals)
#define TRIXI_DISPATCH_MHD(dim, eq, call)                                                   \
  do {                                                                                      \
    if ((eq) == EQ_MHD) {                                                                   \
      if ((dim) == 1) { constexpr int D_ = 1, Q_ = EQ_MHD; call; }                          \
      else if ((dim) == 2) { constexpr int D_ = 2, Q_ = EQ_MHD; call; }                     \
      else { constexpr int D_ = 3, Q_ = EQ_MHD; call; }                                     \
    } else {                                                                                \
      TRIXI_DISPATCH(dim, eq, call);                                                        \
    }                                                                                       \
  } while (0)

cudaError_t launch_max_dt(const MaxDtHost &h, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(h.acc, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  const int per_block = 8;  // one warp per element
  const unsigned grid = (unsigned)((h.E + per_block - 1) / per_block);
  TRIXI_DISPATCH_MHD(h.dim, h.eq,
                 (max_speed_kernel<D_, Q_><<<grid, 32 * per_block, 0, s>>>(h.N, h.E, h.u, h.inv_jac, h.gamma, h.a[0],
                                                                           h.a[1], h.a[2], h.acc)));
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  max_dt_finalize<<<1, 1, 0, s>>>(h.N, h.acc, h.dt);
  return cudaGetLastError();
}

cudaError_t launch_integrate(const IntegrateHost &h, cudaStream_t s) {
  const int per_block = 8;
  const unsigned grid = (unsigned)((h.E + per_block - 1) / per_block);
  TRIXI_DISPATCH_MHD(h.dim, h.eq,
                 (integrate_kernel<D_, Q_><<<grid, 32 * per_block, 0, s>>>(h.N, h.E, h.u, h.du, h.inv_jac, h.w, h.which,
                                                                           h.nq, h.gamma, h.partial)));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  reduce_columns<<<1, 1024, 0, s>>>(h.E, h.nq, h.partial, 0, h.out);
  return cudaGetLastError();
}

cudaError_t launch_initial_condition(const IcHost &h, cudaStream_t s) {
  int NN = h.N;
  for (int d = 1; d < h.dim; ++d) NN *= h.N;
  const int64_t n = h.E * NN;
  const unsigned grid = (unsigned)((n + 255) / 256);
  TRIXI_DISPATCH_MHD(h.dim, h.eq, (ic_kernel<D_, Q_><<<grid, 256, 0, s>>>(h.N, h.E, h.coords, h.kind, h.ip, h.t, h.u)));
  return cudaGetLastError();
}

cudaError_t launch_error_norms_all(const ErrorNormHost &h, cudaStream_t s) {
  cudaError_t e = cudaSuccess;
  TRIXI_DISPATCH_MHD(h.dim, h.eq, (e = launch_error_norms<D_, Q_>(h, s)));
  if (e != cudaSuccess) return e;
  reduce_columns<<<1, 1024, 0, s>>>(h.E, h.nv, h.l2p, 0, h.l2_out);
  reduce_columns<<<1, 1024, 0, s>>>(h.E, h.nv, h.linfp, 1, h.linf_out);
  return cudaGetLastError();
}

}  // namespace trixi

// ===========================================================================
// trixi_integrate_noalloc: the quadrature integrals of trixi_integrate (linear
// advection and compressible Euler; ideal GLM-MHD only through
// trixi_integrate) for callers that cannot allocate device memory -- for example an application
// whose device memory is owned entirely by another allocator (a Julia
// CUDA.jl or PyTorch caching pool that has reserved the GPU), or a
// time-critical loop that must not pay for the device-wide synchronisation
// that cudaMalloc / cudaFree imply.  Its per-element partial sums live in the
// file-scope device array below instead of a handle-owned buffer, and it
// needs no handle (trixi_create allocates).  Limits and sharing rules:
//   * at most kNoallocMaxPartials = 2^20 partial sums per call, i.e.
//     nelements * nq <= 1,048,576 (nq = nvars for STATE and DU, 1 otherwise);
//     larger calls are rejected with TRIXI_ERR_INVALID_ARGUMENT;
//   * the array (8 MiB) is reserved on every GPU that loads the library, until
//     the process exits;
//   * all calls share it and it keeps the last call's contents.  Every slot a
//     call reads it has written itself first, so nothing needs clearing, but
//     two calls whose kernels overlap on the GPU (different streams, or
//     different host threads on the same device) race on it;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current, and caches it per
//     device.
// ===========================================================================
// file-scope scratch shared by every call on a device (see above)
static constexpr int64_t kNoallocMaxPartials = int64_t(1) << 20;
static __device__ __align__(256) double g_noalloc_partials[kNoallocMaxPartials];

namespace {

// device address of g_noalloc_partials per device ordinal; filled at the first
// call on that device, with that device current
constexpr int kMaxDevices = 64;
std::atomic<double *> g_noalloc_ptr[kMaxDevices];

int noalloc_scratch(double **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return TRIXI_ERR_CUDA;
  double *p = g_noalloc_ptr[dev].load(std::memory_order_acquire);
  if (!p) {
    cudaError_t e = cudaGetSymbolAddress((void **)&p, g_noalloc_partials);
    if (e != cudaSuccess || !p) return TRIXI_ERR_CUDA;
    g_noalloc_ptr[dev].store(p, std::memory_order_release);
  }
  *out = p;
  return TRIXI_OK;
}

// LGL quadrature weights per polydeg, computed once per process:
// lgl_weights_fixed runs a long-double Newton iteration per node, which a
// per-call entry point meant for time-critical loops should not repeat
const double *noalloc_weights(int polydeg) {
  constexpr int kMaxDeg = 15;
  static std::once_flag once[kMaxDeg + 1];
  static double table[kMaxDeg + 1][16];
  static bool ok[kMaxDeg + 1];
  if (polydeg < 1 || polydeg > kMaxDeg) return nullptr;
  std::call_once(once[polydeg], [polydeg] { ok[polydeg] = trixi::lgl_weights_fixed(polydeg, table[polydeg]); });
  return ok[polydeg] ? table[polydeg] : nullptr;
}

}  // namespace
extern "C" int trixi_integrate_noalloc(int ndims, int polydeg, int equation, double gamma, const double *u,
                                       const double *du, const double *inverse_jacobian, int64_t nelements,
                                       int which, double *out_dev, void *stream) {
  using namespace trixi;
  char msg[256];
  auto reject = [&](int status, const char *text) {
    set_last_error(status, text);
    return status;
  };
  if (ndims < 1 || ndims > 3) return reject(TRIXI_ERR_INVALID_ARGUMENT, "integrate_noalloc: ndims");
  if (polydeg < 1 || polydeg > 15) return reject(TRIXI_ERR_INVALID_ARGUMENT, "integrate_noalloc: polydeg");
  if (equation != EQ_ADV && equation != EQ_EULER) return reject(TRIXI_ERR_INVALID_ARGUMENT, "integrate_noalloc: equation");
  if (which < 0 || which > 3) return reject(TRIXI_ERR_INVALID_ARGUMENT, "integrate_noalloc: integral kind");
  if (!u || !inverse_jacobian || !out_dev || nelements <= 0 || ((which == 2 || which == 3) && !du))
    return reject(TRIXI_ERR_INVALID_ARGUMENT, "integrate_noalloc: null pointer or empty mesh");
  const int nv = (equation == EQ_ADV) ? 1 : ndims + 2;
  const int nq = (which == 0 || which == 3) ? nv : 1;
  if (nelements > kNoallocMaxPartials / nq) {
    snprintf(msg, sizeof(msg),
             "integrate_noalloc: %lld elements x %d values exceed the %lld partial sums of its static scratch",
             (long long)nelements, nq, (long long)kNoallocMaxPartials);
    return reject(TRIXI_ERR_INVALID_ARGUMENT, msg);
  }
  double *partials = nullptr;
  if (noalloc_scratch(&partials) != TRIXI_OK)
    return reject(TRIXI_ERR_CUDA, "integrate_noalloc: cudaGetSymbolAddress of the scratch array failed");
  WeightsArg wa{};
  const double *w = noalloc_weights(polydeg);
  if (!w) return reject(TRIXI_ERR_INVALID_ARGUMENT, "integrate_noalloc: weights");
  for (int j = 0; j <= polydeg; ++j) wa.w[j] = w[j];
  cudaStream_t s = (cudaStream_t)stream;
  const int per_block = 8;
  const unsigned grid = (unsigned)((nelements + per_block - 1) / per_block);
  const int N = polydeg + 1;
  TRIXI_DISPATCH(ndims, equation,
                 (integrate_w_kernel<D_, Q_><<<grid, 32 * per_block, 0, s>>>(N, nelements, u, du, inverse_jacobian, wa,
                                                                             which, nq, gamma, partials)));
  if (cudaGetLastError() != cudaSuccess) return reject(TRIXI_ERR_CUDA, "integrate_noalloc: kernel launch");
  reduce_columns<<<1, 1024, 0, s>>>(nelements, nq, partials, 0, out_dev);
  if (cudaGetLastError() != cudaSuccess) return reject(TRIXI_ERR_CUDA, "integrate_noalloc: reduction launch");
  return TRIXI_OK;
}
