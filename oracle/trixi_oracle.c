/*
 * trixi_oracle.c -- CPU restatement (C11 + OpenMP) of the TreeMesh DGSEM
 * semidiscretization rhs! of TrixiCUDA.jl, stage by stage.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU library, never shipped
 * in or called by the product path.  Parity is UNPINNED at the Trixi.jl
 * boundary (Trixi.jl, which owns the arithmetic, is not vendored and Julia is
 * absent); the oracle is pinned by analytic known answers and discrete
 * invariants checked in tests/.
 *
 * Stage structure, signs and scalings follow the reference kernels:
 *   volume integral (weak form)     src/solvers/dg_2d_kernel.jl:55-105 (1D L42, 3D L65)
 *   volume integral (flux diff.)    src/solvers/dg_2d_kernel.jl:164-225 (1D L132, 3D L188)
 *   DG-FV shock capturing blend     src/solvers/dg_2d_kernel.jl:496-606, dg_3d_kernel.jl:589-728,
 *                                   atol from src/solvers/dg_2d.jl:173
 *   prolong2interfaces              src/solvers/dg_2d_kernel.jl:907-935, dg_3d_kernel.jl:1121-1152
 *   interface flux + scatter        src/solvers/dg_2d_kernel.jl:938-1006, dg_3d_kernel.jl:1155-1230
 *   prolong2mortars                 src/solvers/dg_2d_kernel.jl:1167-1259, dg_3d_kernel.jl:1361-1500
 *   mortar flux + L2 back-projection src/solvers/dg_2d_kernel.jl:1262-1397, dg_3d_kernel.jl:1503-1770
 *   surface integral                src/solvers/dg_2d_kernel.jl:1400-1421, dg_3d_kernel.jl:1773-1799
 *   apply jacobian                  src/solvers/dg_2d_kernel.jl:1424-1437
 *   HG indicator parameters         src/solvers/indicators.jl:7-42
 *   rhs stage order                 src/solvers/dg_2d.jl:760-790
 *
 * The mathematics owned by Trixi.jl / OrdinaryDiffEq is restated from the
 * published methods, not from their sources:
 *   LGL nodes/weights, barycentric Lagrange, derivative matrix: Kopriva (2009),
 *     "Implementing Spectral Methods for PDEs", Alg. 22-25, 30-31, 37.
 *   Split-form operator D_split = 2D - M^{-1}B: Gassner, Winters, Kopriva (2016), JCP 327.
 *   Weak-form operator D_hat = -M^{-1} D^T M.
 *   flux_ranocha: Ranocha (2018) thesis / Ranocha (2020), entropy-conserving,
 *     kinetic-energy-preserving flux with logarithmic means.
 *   Logarithmic mean: Ismail & Roe (2009), JCP 228, appendix B series in
 *     u = ((x-y)/(x+y))^2, used below 1e-4.
 *   Local Lax-Friedrichs (Rusanov) flux with Davis wave-speed estimate.
 *   Hennemann, Rueda-Ramirez, Hindenlang, Gassner (2021), JCP 426: modal
 *     energy indicator, threshold 0.5*10^(-1.8 N^0.25), logistic blending.
 *   L2 mortars: Kopriva (1996), exact L2 projection.
 *   CarpenterKennedy2N54: Carpenter & Kennedy (1994), NASA TM-109112, 2N storage.
 */
#include "trixi_oracle.h"

#define ORC_PI 3.14159265358979323846

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NMAX 16
#define NVMAX 9

typedef long double ld;

/* ------------------------------------------------------------------------ */
/* Basis (Kopriva 2009)                                                     */
/* ------------------------------------------------------------------------ */

/* Legendre polynomial L_n and its derivative by the three-term recurrence. */
static void legendre(int n, ld x, ld *L, ld *dL) {
  if (n == 0) { *L = 1; *dL = 0; return; }
  if (n == 1) { *L = x; *dL = 1; return; }
  ld Lm2 = 1, Lm1 = x, dLm2 = 0, dLm1 = 1, Lk = 0, dLk = 0;
  for (int k = 2; k <= n; ++k) {
    Lk = ((ld)(2 * k - 1) * x * Lm1 - (ld)(k - 1) * Lm2) / (ld)k;
    dLk = dLm2 + (ld)(2 * k - 1) * Lm1;
    Lm2 = Lm1; Lm1 = Lk; dLm2 = dLm1; dLm1 = dLk;
  }
  *L = Lk; *dL = dLk;
}

static const ld PI_L = 3.141592653589793238462643383279502884L;

/* Gauss-Lobatto nodes/weights for n nodes (degree p = n-1): endpoints plus the
 * roots of L_p', found by Newton's method from Chebyshev-Lobatto guesses. */
static void lgl_nodes_weights(int n, ld *x, ld *w) {
  int p = n - 1;
  if (p == 0) { x[0] = 0; w[0] = 2; return; }
  x[0] = -1; x[p] = 1;
  for (int j = 1; j < p; ++j) {
    ld xj = -cosl(PI_L * (ld)j / (ld)p);
    for (int it = 0; it < 100; ++it) {
      ld L, dL;
      legendre(p, xj, &L, &dL);
      ld d2L = (2 * xj * dL - (ld)p * (ld)(p + 1) * L) / (1 - xj * xj);
      ld dx = dL / d2L;
      xj -= dx;
      if (fabsl(dx) < 1e-30L) break;
    }
    x[j] = xj;
  }
  /* enforce exact symmetry */
  for (int j = 0; j < n / 2; ++j) { ld s = 0.5L * (x[n - 1 - j] - x[j]); x[j] = -s; x[n - 1 - j] = s; }
  if (n % 2 == 1) x[n / 2] = 0;
  for (int j = 0; j < n; ++j) {
    ld L, dL;
    legendre(p, x[j], &L, &dL);
    w[j] = 2.0L / ((ld)p * (ld)(p + 1) * L * L);
  }
}

/* Gauss-Legendre nodes/weights (roots of L_n). */
static void gauss_nodes_weights(int n, ld *x, ld *w) {
  for (int j = 0; j < n; ++j) {
    ld xj = -cosl(PI_L * ((ld)j + 0.75L) / ((ld)n + 0.5L));
    for (int it = 0; it < 100; ++it) {
      ld L, dL;
      legendre(n, xj, &L, &dL);
      ld dx = L / dL;
      xj -= dx;
      if (fabsl(dx) < 1e-30L) break;
    }
    ld L, dL;
    legendre(n, xj, &L, &dL);
    x[j] = xj;
    w[j] = 2.0L / ((1 - xj * xj) * dL * dL);
  }
}

static void barycentric_weights(int n, const ld *x, ld *lam) {
  for (int j = 0; j < n; ++j) {
    ld p = 1;
    for (int k = 0; k < n; ++k)
      if (k != j) p *= (x[j] - x[k]);
    lam[j] = 1 / p;
  }
}

/* Lagrange basis values at xi (barycentric form; exact delta at a node). */
static void lagrange_at(int n, const ld *x, const ld *lam, ld xi, ld *ell) {
  for (int j = 0; j < n; ++j)
    if (xi == x[j]) {
      for (int k = 0; k < n; ++k) ell[k] = (k == j);
      return;
    }
  ld s = 0;
  for (int j = 0; j < n; ++j) { ell[j] = lam[j] / (xi - x[j]); s += ell[j]; }
  for (int j = 0; j < n; ++j) ell[j] /= s;
}

/* Orthonormal Legendre polynomial sqrt(n+1/2) L_n(x). */
static ld legendre_normalized(int n, ld x) {
  ld L, dL;
  legendre(n, x, &L, &dL);
  return L * sqrtl((ld)n + 0.5L);
}

static int invert(int n, ld *a /* n x n column-major, overwritten */, ld *inv) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) inv[i + n * j] = (i == j);
  for (int c = 0; c < n; ++c) {
    int piv = c;
    for (int r = c + 1; r < n; ++r)
      if (fabsl(a[r + n * c]) > fabsl(a[piv + n * c])) piv = r;
    if (a[piv + n * c] == 0) return -1;
    if (piv != c)
      for (int j = 0; j < n; ++j) {
        ld t = a[c + n * j]; a[c + n * j] = a[piv + n * j]; a[piv + n * j] = t;
        t = inv[c + n * j]; inv[c + n * j] = inv[piv + n * j]; inv[piv + n * j] = t;
      }
    ld d = a[c + n * c];
    for (int j = 0; j < n; ++j) { a[c + n * j] /= d; inv[c + n * j] /= d; }
    for (int r = 0; r < n; ++r)
      if (r != c) {
        ld f = a[r + n * c];
        if (f != 0)
          for (int j = 0; j < n; ++j) { a[r + n * j] -= f * a[c + n * j]; inv[r + n * j] -= f * inv[c + n * j]; }
      }
  }
  return 0;
}

int oracle_basis(int polydeg, double *nodes, double *weights, double *dmat,
                 double *dsplit, double *dhat, double *inv_vandermonde,
                 double *forward_upper, double *forward_lower,
                 double *reverse_upper, double *reverse_lower) {
  int n = polydeg + 1;
  if (n < 2 || n > NMAX) return -1;
  ld x[NMAX], w[NMAX], lam[NMAX], D[NMAX * NMAX];
  lgl_nodes_weights(n, x, w);
  barycentric_weights(n, x, lam);
  /* derivative matrix, Kopriva Alg. 37 (negative-sum diagonal) */
  for (int i = 0; i < n; ++i) {
    ld s = 0;
    for (int j = 0; j < n; ++j)
      if (j != i) { D[i + n * j] = (lam[j] / lam[i]) / (x[i] - x[j]); s += D[i + n * j]; }
    D[i + n * i] = -s;
  }
  for (int i = 0; i < n; ++i) {
    if (nodes) nodes[i] = (double)x[i];
    if (weights) weights[i] = (double)w[i];
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      if (dmat) dmat[i + n * j] = (double)D[i + n * j];
      if (dsplit) {
        ld v = 2 * D[i + n * j];
        if (i == j && i == 0) v += 1 / w[0];
        if (i == j && i == n - 1) v -= 1 / w[n - 1];
        dsplit[i + n * j] = (double)v;
      }
      if (dhat) dhat[i + n * j] = (double)(-D[j + n * i] * w[j] / w[i]);
    }
  if (inv_vandermonde) {
    ld V[NMAX * NMAX], Vi[NMAX * NMAX];
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) V[i + n * j] = legendre_normalized(j, x[i]);
    if (invert(n, V, Vi)) return -2;
    for (int i = 0; i < n * n; ++i) inv_vandermonde[i] = (double)Vi[i];
  }
  /* forward (large -> small) interpolation: F_up[j,i] = l_i((x_j+1)/2) */
  for (int j = 0; j < n; ++j) {
    ld ell[NMAX];
    lagrange_at(n, x, lam, 0.5L * (x[j] + 1), ell);
    if (forward_upper)
      for (int i = 0; i < n; ++i) forward_upper[j + n * i] = (double)ell[i];
    lagrange_at(n, x, lam, 0.5L * (x[j] - 1), ell);
    if (forward_lower)
      for (int i = 0; i < n; ++i) forward_lower[j + n * i] = (double)ell[i];
  }
  /* reverse (small -> large) exact L2 projection onto P_{n-1} of the large
   * face, in the LGL nodal basis; Gauss quadrature with n+1 points is exact
   * for the degree 2n-2 integrands. */
  {
    int nq = n + 1;
    ld g[NMAX + 1], gw[NMAX + 1];
    gauss_nodes_weights(nq, g, gw);
    for (int half = 0; half < 2; ++half) {
      double *R = half ? reverse_upper : reverse_lower;
      if (!R) continue;
      ld shift = half ? 1 : -1;
      for (int j = 0; j < n; ++j) {
        ld c[NMAX];
        for (int m = 0; m < n; ++m) {
          ld s = 0;
          for (int q = 0; q < nq; ++q) {
            ld ell[NMAX];
            lagrange_at(n, x, lam, g[q], ell);
            s += gw[q] * legendre_normalized(m, 0.5L * (g[q] + shift)) * ell[j];
          }
          c[m] = 0.5L * s;
        }
        for (int k = 0; k < n; ++k) {
          ld v = 0;
          for (int m = 0; m < n; ++m) v += legendre_normalized(m, x[k]) * c[m];
          R[k + n * j] = (double)v;
        }
      }
    }
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Physics                                                                  */
/* ------------------------------------------------------------------------ */

typedef struct {
  int dim, nv, eq;
  double gamma;
  double a[3];
  double c_h;    /* GLM cleaning speed (ideal GLM-MHD) */
  int noncons;   /* ORC_NONCONS_* */
} phys_t;

/* ---- ideal GLM-MHD --------------------------------------------------------
 * IdealGlmMhdEquations{1,2,3}D.  State (rho, rho v1, rho v2, rho v3, E, B1, B2,
 * B3, psi) in 2D/3D; 1D has no psi (8 variables).  Velocities and magnetic
 * fields always have three components.  The GLM formulation follows Derigs,
 * Winters, Gassner, Walch, Bohm, "Ideal GLM-MHD: about the entropy consistent
 * nine-wave magnetic field divergence diminishing ideal magnetohydrodynamics
 * equations", JCP 364 (2018): E = p/(gamma-1) + rho|v|^2/2 + |B|^2/2 + psi^2/2,
 * the conservative flux carries c_h psi and c_h B_o for the cleaning, and the
 * transport of psi (v . grad psi) sits in the nonconservative term with the
 * Powell source. */
static int mhd_has_psi(const phys_t *P) { return P->nv == 9; }

/* primitive (rho, v1, v2, v3, p, B1, B2, B3, psi) */
static void mhd_prim(const phys_t *P, const double *u, double *w) {
  const double rho = u[0];
  const double v1 = u[1] / rho, v2 = u[2] / rho, v3 = u[3] / rho;
  const double psi = mhd_has_psi(P) ? u[8] : 0.0;
  const double kin = 0.5 * rho * (v1 * v1 + v2 * v2 + v3 * v3);
  const double mag = 0.5 * (u[5] * u[5] + u[6] * u[6] + u[7] * u[7]);
  w[0] = rho; w[1] = v1; w[2] = v2; w[3] = v3;
  w[4] = (P->gamma - 1) * (u[4] - kin - mag - 0.5 * psi * psi);
  w[5] = u[5]; w[6] = u[6]; w[7] = u[7]; w[8] = psi;
}

/* physical flux along o of ideal GLM-MHD */
static void mhd_flux(const phys_t *P, const double *u, int o, double *f) {
  double w[9];
  mhd_prim(P, u, w);
  const double rho = w[0], p = w[4], psi = w[8];
  const double *v = w + 1, *B = w + 5;
  const double mag = 0.5 * (B[0] * B[0] + B[1] * B[1] + B[2] * B[2]);
  const double kin = 0.5 * rho * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  const double vB = v[0] * B[0] + v[1] * B[1] + v[2] * B[2];
  const double ch = mhd_has_psi(P) ? P->c_h : 0.0;
  f[0] = rho * v[o];
  for (int d = 0; d < 3; ++d) f[1 + d] = rho * v[o] * v[d] - B[o] * B[d] + (d == o ? p + mag : 0.0);
  f[4] = (kin + P->gamma * p / (P->gamma - 1) + 2 * mag) * v[o] - B[o] * vB + ch * psi * B[o];
  for (int d = 0; d < 3; ++d) f[5 + d] = (d == o) ? ch * psi : v[o] * B[d] - v[d] * B[o];
  if (mhd_has_psi(P)) f[8] = ch * B[o];
}

/* Hindenlang & Gassner (2019), "A new entropy conservative two-point flux for
 * ideal MHD equations derived from first principles" (HONOM 2019): the
 * logarithmic mean of rho and of rho/p (Ismail-Roe), arithmetic means of v,
 * p, psi, product means of the magnetic terms, and the energy flux fixed by
 * the entropy-conservation condition with the nonconservative Powell term. */
static double ln_mean(double x, double y);
static double inv_ln_mean(double x, double y);
static void mhd_flux_hindenlang_gassner(const phys_t *P, const double *ul, const double *ur, int o, double *f) {
  double wl[9], wr[9];
  mhd_prim(P, ul, wl);
  mhd_prim(P, ur, wr);
  const double rl = wl[0], rr = wr[0], pl = wl[4], pr = wr[4];
  const double *vl = wl + 1, *vr = wr + 1, *Bl = wl + 5, *Br = wr + 5;
  const double psil = wl[8], psir = wr[8];
  const double ch = mhd_has_psi(P) ? P->c_h : 0.0;
  const double rho_mean = ln_mean(rl, rr);
  const double inv_rho_p_mean = pl * pr * inv_ln_mean(rl * pr, rr * pl);
  double vavg[3];
  for (int d = 0; d < 3; ++d) vavg[d] = 0.5 * (vl[d] + vr[d]);
  const double pavg = 0.5 * (pl + pr), psiavg = 0.5 * (psil + psir);
  const double v2avg = 0.5 * (vl[0] * vr[0] + vl[1] * vr[1] + vl[2] * vr[2]);
  const double b2avg = 0.5 * (Bl[0] * Br[0] + Bl[1] * Br[1] + Bl[2] * Br[2]);
  const double f0 = rho_mean * vavg[o];
  f[0] = f0;
  for (int d = 0; d < 3; ++d)
    f[1 + d] = f0 * vavg[d] + (d == o ? pavg + b2avg : 0.0) - 0.5 * (Bl[o] * Br[d] + Br[o] * Bl[d]);
  for (int d = 0; d < 3; ++d)
    f[5 + d] = (d == o) ? ch * psiavg : 0.5 * (vl[o] * Bl[d] - vl[d] * Bl[o] + vr[o] * Br[d] - vr[d] * Br[o]);
  if (mhd_has_psi(P)) f[8] = ch * 0.5 * (Bl[o] + Br[o]);
  double e = pl * vr[o] + pr * vl[o];
  for (int d = 0; d < 3; ++d) {
    if (d == o) continue;
    e += vl[o] * Bl[d] * Br[d] + vr[o] * Br[d] * Bl[d];
    e -= vl[d] * Bl[o] * Br[d] + vr[d] * Br[o] * Bl[d];
  }
  e += ch * (Bl[o] * psir + Br[o] * psil);
  f[4] = f0 * (v2avg + inv_rho_p_mean / (P->gamma - 1)) + 0.5 * e;
}

/* fast magnetosonic speed along o */
static double mhd_fast_speed(const phys_t *P, const double *w, int o) {
  const double rho = w[0], p = w[4];
  const double a2 = P->gamma * p / rho;
  const double b2 = (w[5] * w[5] + w[6] * w[6] + w[7] * w[7]) / rho;
  const double bo2 = w[5 + o] * w[5 + o] / rho;
  const double s = a2 + b2;
  return sqrt(0.5 * (s + sqrt(s * s - 4.0 * a2 * bo2)));
}

/* Powell + GLM (Galilean) nonconservative two-point term along o with the
 * local state u_l (Derigs et al. 2018, Bohm et al. JCP 422 (2020)):
 * phi_Powell(u_l) B_o(u_r) + v_o(u_l) phi_GLM(u_l) psi(u_r), with
 * phi_Powell = (0, B, v.B, v, 0) and phi_GLM = (0, 0, 0, 0, psi, 0, 0, 0, 1). */
static void mhd_noncons_powell(const phys_t *P, const double *ul, const double *ur, int o, double *f) {
  double wl[9], wr[9];
  mhd_prim(P, ul, wl);
  mhd_prim(P, ur, wr);
  const double *vl = wl + 1, *Bl = wl + 5;
  const double Bo = wr[5 + o], psir = wr[8];
  const double vB = vl[0] * Bl[0] + vl[1] * Bl[1] + vl[2] * Bl[2];
  f[0] = 0.0;
  for (int d = 0; d < 3; ++d) f[1 + d] = Bl[d] * Bo;
  f[4] = vB * Bo + vl[o] * wl[8] * psir;
  for (int d = 0; d < 3; ++d) f[5 + d] = vl[d] * Bo;
  f[8] = vl[o] * psir;
}

static void cons2prim(const phys_t *P, const double *u, double *rho, double *v, double *p) {
  if (P->eq == ORC_EQ_MHD) {
    double w[9];
    mhd_prim(P, u, w);
    *rho = w[0];
    for (int d = 0; d < 3; ++d) v[d] = w[1 + d];
    *p = w[4];
    return;
  }
  double r = u[0], kin = 0;
  for (int d = 0; d < P->dim; ++d) { v[d] = u[1 + d] / r; kin += u[1 + d] * v[d]; }
  *rho = r;
  *p = (P->gamma - 1) * (u[P->dim + 1] - 0.5 * kin);
}

/* physical flux f_o(u) */
static void flux_phys(const phys_t *P, const double *u, int o, double *f) {
  if (P->eq == ORC_EQ_ADVECTION) { f[0] = P->a[o] * u[0]; return; }
  if (P->eq == ORC_EQ_MHD) { mhd_flux(P, u, o, f); return; }
  double rho, v[3], p;
  cons2prim(P, u, &rho, v, &p);
  f[0] = u[1 + o];
  for (int d = 0; d < P->dim; ++d) f[1 + d] = u[1 + o] * v[d] + (d == o ? p : 0.0);
  f[P->dim + 1] = (u[P->dim + 1] + p) * v[o];
}

/* Ismail-Roe logarithmic mean and its inverse (series below 1e-4). */
static double ln_mean(double x, double y) {
  double f2 = (x * (x - 2 * y) + y * y) / (x * (x + 2 * y) + y * y);
  if (f2 < 1.0e-4) return (x + y) * 52.5 / (105 + f2 * (35 + f2 * (21 + f2 * 15)));
  return (y - x) / log(y / x);
}
static double inv_ln_mean(double x, double y) {
  double f2 = (x * (x - 2 * y) + y * y) / (x * (x + 2 * y) + y * y);
  if (f2 < 1.0e-4) return (105 + f2 * (35 + f2 * (21 + f2 * 15))) / (52.5 * (x + y));
  return log(y / x) / (y - x);
}

static void flux_ranocha(const phys_t *P, const double *ul, const double *ur, int o, double *f) {
  if (P->eq == ORC_EQ_ADVECTION) { /* EC flux of linear advection = central */
    f[0] = 0.5 * (P->a[o] * ul[0] + P->a[o] * ur[0]);
    return;
  }
  int dim = P->dim;
  double rl, rr, vl[3], vr[3], pl, pr;
  cons2prim(P, ul, &rl, vl, &pl);
  cons2prim(P, ur, &rr, vr, &pr);
  double rho_mean = ln_mean(rl, rr);
  double inv_rho_p_mean = pl * pr * inv_ln_mean(rl * pr, rr * pl);
  double vavg[3], v2avg = 0;
  for (int d = 0; d < dim; ++d) { vavg[d] = 0.5 * (vl[d] + vr[d]); v2avg += vl[d] * vr[d]; }
  v2avg *= 0.5;
  double pavg = 0.5 * (pl + pr);
  double f0 = rho_mean * vavg[o];
  f[0] = f0;
  for (int d = 0; d < dim; ++d) f[1 + d] = f0 * vavg[d] + (d == o ? pavg : 0.0);
  f[dim + 1] = f0 * (v2avg + inv_rho_p_mean / (P->gamma - 1)) + 0.5 * (pl * vr[o] + pr * vl[o]);
}

static void flux_central(const phys_t *P, const double *ul, const double *ur, int o, double *f) {
  double fl[NVMAX], fr[NVMAX];
  flux_phys(P, ul, o, fl);
  flux_phys(P, ur, o, fr);
  for (int v = 0; v < P->nv; ++v) f[v] = 0.5 * (fl[v] + fr[v]);
}

static double max_abs_speed(const phys_t *P, const double *ul, const double *ur, int o, int naive) {
  if (P->eq == ORC_EQ_ADVECTION) return fabs(P->a[o]);
  if (P->eq == ORC_EQ_MHD) {
    double wl[9], wr[9];
    mhd_prim(P, ul, wl);
    mhd_prim(P, ur, wr);
    const double cl = mhd_fast_speed(P, wl, o), cr = mhd_fast_speed(P, wr, o);
    if (naive) return fmax(fabs(wl[1 + o]), fabs(wr[1 + o])) + fmax(cl, cr);
    return fmax(fabs(wl[1 + o]) + cl, fabs(wr[1 + o]) + cr);
  }
  double rl, rr, vl[3], vr[3], pl, pr;
  cons2prim(P, ul, &rl, vl, &pl);
  cons2prim(P, ur, &rr, vr, &pr);
  double cl = sqrt(P->gamma * pl / rl), cr = sqrt(P->gamma * pr / rr);
  if (naive) return fmax(fabs(vl[o]), fabs(vr[o])) + fmax(cl, cr);
  return fmax(fabs(vl[o]) + cl, fabs(vr[o]) + cr);
}

static void flux_llf(const phys_t *P, const double *ul, const double *ur, int o, int naive, double *f) {
  flux_central(P, ul, ur, o, f);
  double lam = max_abs_speed(P, ul, ur, o, naive);
  for (int v = 0; v < P->nv; ++v) f[v] += -0.5 * lam * (ur[v] - ul[v]);
}

/* Shima, Kuya, Tamaki, Kawai (2021), JCP 427: kinetic-energy and pressure-
 * equilibrium preserving flux (Euler). */
static void flux_shima(const phys_t *P, const double *ul, const double *ur, int o, double *f) {
  const int dim = P->dim;
  double rl, rr, vl[3], vr[3], pl, pr;
  cons2prim(P, ul, &rl, vl, &pl);
  cons2prim(P, ur, &rr, vr, &pr);
  const double rho_avg = 0.5 * (rl + rr), p_avg = 0.5 * (pl + pr);
  double vavg[3], kin = 0;
  for (int d = 0; d < dim; ++d) { vavg[d] = 0.5 * (vl[d] + vr[d]); kin += vl[d] * vr[d]; }
  kin *= 0.5;
  const double f0 = rho_avg * vavg[o];
  f[0] = f0;
  for (int d = 0; d < dim; ++d) f[1 + d] = f0 * vavg[d] + (d == o ? p_avg : 0.0);
  f[dim + 1] = p_avg * vavg[o] / (P->gamma - 1) + f0 * kin + 0.5 * (pl * vr[o] + pr * vl[o]);
}

/* HLL (Harten, Lax, van Leer 1983) with the naive signal-speed estimates
 * min(v_l - c_l, v_r - c_r), max(v_l + c_l, v_r + c_r) (fast magnetosonic c
 * for MHD, the advection speed for linear advection). */
static void flux_hll(const phys_t *P, const double *ul, const double *ur, int o, double *f) {
  double lmin, lmax;
  if (P->eq == ORC_EQ_ADVECTION) {
    lmin = lmax = P->a[o];
  } else if (P->eq == ORC_EQ_MHD) {
    double wl[9], wr[9];
    mhd_prim(P, ul, wl);
    mhd_prim(P, ur, wr);
    const double cl = mhd_fast_speed(P, wl, o), cr = mhd_fast_speed(P, wr, o);
    lmin = fmin(wl[1 + o] - cl, wr[1 + o] - cr);
    lmax = fmax(wl[1 + o] + cl, wr[1 + o] + cr);
  } else {
    double rl, rr, vl[3], vr[3], pl, pr;
    cons2prim(P, ul, &rl, vl, &pl);
    cons2prim(P, ur, &rr, vr, &pr);
    const double cl = sqrt(P->gamma * pl / rl), cr = sqrt(P->gamma * pr / rr);
    lmin = fmin(vl[o] - cl, vr[o] - cr);
    lmax = fmax(vl[o] + cl, vr[o] + cr);
  }
  double fl[NVMAX], fr[NVMAX];
  flux_phys(P, ul, o, fl);
  flux_phys(P, ur, o, fr);
  for (int v = 0; v < P->nv; ++v) {
    if (lmin >= 0) f[v] = fl[v];
    else if (lmax <= 0) f[v] = fr[v];
    else f[v] = (lmax * fl[v] - lmin * fr[v] + lmin * lmax * (ur[v] - ul[v])) / (lmax - lmin);
  }
}

/* Einfeldt's signal speeds for flux_hlle (Trixi.jl's min_max_speed_einfeldt,
 * outside the reference repository; restated from the publications):
 *  Euler (Einfeldt, Munz, Roe, Sjogreen, JCP 92 (1991)): Roe averages with
 *    sqrt(rho) weights of v and H = (E + p)/rho, c~ = sqrt((gamma-1)(H~ -
 *    |v~|^2/2)), beta = sqrt((gamma-1)/(2 gamma)),
 *    lmin = min(v~ - c~, v_l - beta c_l, 0), lmax = max(v~ + c~, v_r + beta c_r, 0);
 *  ideal GLM-MHD (Cargo, Gallice, JCP 136 (1997), the fast speed of their
 *    Roe-type matrix): v, H = (E + p + |B|^2/2)/rho with sqrt(rho) weights, B
 *    with the crossed weights, X = |B_l - B_r|^2 / (2 (sqrt rho_l + sqrt rho_r)^2),
 *    b^2 = |B~|^2 / sqrt(rho_l rho_r), a^2 = (2-gamma) X + (gamma-1)(H~ - |v~|^2/2 - b^2),
 *    c_f~^2 = (a^2 + b^2 + sqrt((a^2 + b^2)^2 - 4 a^2 B~_o^2 / sqrt(rho_l rho_r)))/2,
 *    lmin = min(v_l - c_f,l, v~ - c_f~), lmax = max(v_r + c_f,r, v~ + c_f~). */
static void einfeldt_speeds(const phys_t *P, const double *ul, const double *ur, int o, double *lmin,
                            double *lmax) {
  const double g = P->gamma;
  if (P->eq == ORC_EQ_MHD) {
    double wl[9], wr[9];
    mhd_prim(P, ul, wl);
    mhd_prim(P, ur, wr);
    const double sl = sqrt(wl[0]), sr = sqrt(wr[0]);
    const double ql = sl / (sl + sr), qr = sr / (sl + sr), rho_hat = sl * sr;
    double v[3], B[3], v2 = 0.0, b2 = 0.0, x = 0.0, ml = 0.0, mr = 0.0;
    for (int d = 0; d < 3; ++d) {
      v[d] = ql * wl[1 + d] + qr * wr[1 + d];
      B[d] = qr * wl[5 + d] + ql * wr[5 + d];
      v2 += v[d] * v[d];
      b2 += B[d] * B[d];
      x += (wl[5 + d] - wr[5 + d]) * (wl[5 + d] - wr[5 + d]);
      ml += wl[5 + d] * wl[5 + d];
      mr += wr[5 + d] * wr[5 + d];
    }
    x = 0.5 * x / ((sl + sr) * (sl + sr));
    b2 /= rho_hat;
    const double hl = (ul[4] + wl[4] + 0.5 * ml) / wl[0], hr = (ur[4] + wr[4] + 0.5 * mr) / wr[0];
    const double h = ql * hl + qr * hr;
    const double a2 = (2.0 - g) * x + (g - 1.0) * (h - 0.5 * v2 - b2);
    const double sum = a2 + b2;
    const double cf = sqrt(0.5 * (sum + sqrt(sum * sum - 4.0 * a2 * B[o] * B[o] / rho_hat)));
    const double cl = mhd_fast_speed(P, wl, o), cr = mhd_fast_speed(P, wr, o);
    *lmin = fmin(wl[1 + o] - cl, v[o] - cf);
    *lmax = fmax(wr[1 + o] + cr, v[o] + cf);
    return;
  }
  double rl, rr, vl[3], vr[3], pl, pr;
  cons2prim(P, ul, &rl, vl, &pl);
  cons2prim(P, ur, &rr, vr, &pr);
  const int dim = P->dim;
  const double sl = sqrt(rl), sr = sqrt(rr);
  const double hl = (ul[dim + 1] + pl) / rl, hr = (ur[dim + 1] + pr) / rr;
  double v2 = 0.0, vo = 0.0;
  for (int d = 0; d < dim; ++d) {
    const double vd = (sl * vl[d] + sr * vr[d]) / (sl + sr);
    v2 += vd * vd;
    if (d == o) vo = vd;
  }
  const double h = (sl * hl + sr * hr) / (sl + sr);
  const double c = sqrt((g - 1.0) * (h - 0.5 * v2));
  const double beta = sqrt(0.5 * (g - 1.0) / g);
  const double cl = sqrt(g * pl / rl), cr = sqrt(g * pr / rr);
  *lmin = fmin(fmin(vo - c, vl[o] - beta * cl), 0.0);
  *lmax = fmax(fmax(vo + c, vr[o] + beta * cr), 0.0);
}

/* flux_hlle: the HLL flux of flux_hll with Einfeldt's signal speeds. */
static void flux_hlle(const phys_t *P, const double *ul, const double *ur, int o, double *f) {
  double lmin, lmax, fl[NVMAX], fr[NVMAX];
  einfeldt_speeds(P, ul, ur, o, &lmin, &lmax);
  flux_phys(P, ul, o, fl);
  flux_phys(P, ur, o, fr);
  for (int v = 0; v < P->nv; ++v) {
    if (lmin >= 0) f[v] = fl[v];
    else if (lmax <= 0) f[v] = fr[v];
    else f[v] = (lmax * fl[v] - lmin * fr[v] + lmin * lmax * (ur[v] - ul[v])) / (lmax - lmin);
  }
}

static void two_point_flux(const phys_t *P, int kind, const double *ul, const double *ur, int o, double *f) {
  switch (kind) {
    case ORC_FLUX_HLLE: flux_hlle(P, ul, ur, o, f); break;
    case ORC_FLUX_SHIMA_ETAL: flux_shima(P, ul, ur, o, f); break;
    case ORC_FLUX_HLL: flux_hll(P, ul, ur, o, f); break;
    case ORC_FLUX_RANOCHA: flux_ranocha(P, ul, ur, o, f); break;
    case ORC_FLUX_HINDENLANG_GASSNER: mhd_flux_hindenlang_gassner(P, ul, ur, o, f); break;
    case ORC_FLUX_CENTRAL: flux_central(P, ul, ur, o, f); break;
    case ORC_FLUX_LLF_NAIVE: flux_llf(P, ul, ur, o, 1, f); break;
    default: flux_llf(P, ul, ur, o, 0, f); break;
  }
}

/* f += 0.5 Phi(u_own, u_other): the nonconservative part of a surface or FV
 * subcell flux seen from the element (node) holding u_own
 * (src/solvers/dg_2d_kernel.jl:958-1035) */
static void add_half_noncons(const phys_t *P, const double *uown, const double *uother, int o, double *f) {
  if (P->noncons != ORC_NONCONS_POWELL) return;
  double nc[NVMAX];
  mhd_noncons_powell(P, uown, uother, o, nc);
  for (int v = 0; v < P->nv; ++v) f[v] += 0.5 * nc[v];
}

/* ------------------------------------------------------------------------ */
/* Handle                                                                   */
/* (pointwise fluxes for the tests: oracle_two_point_flux etc. below)       */
/* ------------------------------------------------------------------------ */

struct oracle_handle {
  oracle_desc d;
  phys_t P;
  int N, NN, NF, NV, DIM, nchild;
  double nodes[NMAX], w[NMAX], invw[NMAX];
  double dsplit[NMAX * NMAX], dhat[NMAX * NMAX], ivdm[NMAX * NMAX];
  double fup[NMAX * NMAX], flo[NMAX * NMAX], rup[NMAX * NMAX], rlo[NMAX * NMAX];
  /* scratch for oracle_rhs */
  double *interfaces_u, *sfv, *alpha, *mortar_u[4], *boundaries_u;
};

int oracle_set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
  return omp_get_max_threads();
#else
  (void)nthreads;
  return 1;
#endif
}

static int64_t ipow(int64_t b, int e) { int64_t r = 1; while (e-- > 0) r *= b; return r; }

oracle_handle *oracle_create(const oracle_desc *desc) {
  if (!desc || desc->ndims < 1 || desc->ndims > 3 || desc->polydeg < 1 || desc->polydeg + 1 > NMAX) return NULL;
  oracle_handle *h = (oracle_handle *)calloc(1, sizeof(oracle_handle));
  h->d = *desc;
  h->DIM = desc->ndims;
  h->N = desc->polydeg + 1;
  h->NN = (int)ipow(h->N, h->DIM);
  h->NF = (int)ipow(h->N, h->DIM - 1);
  h->NV = desc->nvars;
  h->nchild = (int)ipow(2, h->DIM - 1);
  h->P.dim = h->DIM; h->P.nv = h->NV; h->P.eq = desc->equation; h->P.gamma = desc->gamma;
  h->P.c_h = desc->glm_speed; h->P.noncons = desc->nonconservative_flux;
  for (int d = 0; d < 3; ++d) h->P.a[d] = desc->advection_velocity[d];
  oracle_basis(desc->polydeg, h->nodes, h->w, NULL, h->dsplit, h->dhat, h->ivdm, h->fup, h->flo, h->rup, h->rlo);
  for (int i = 0; i < h->N; ++i) h->invw[i] = 1.0 / h->w[i];
  h->interfaces_u = (double *)calloc((size_t)(2 * h->NV * h->NF * (desc->ninterfaces > 0 ? desc->ninterfaces : 1)), sizeof(double));
  h->sfv = (double *)calloc((size_t)(h->NV * h->NF * 2 * h->DIM * desc->nelements), sizeof(double));
  h->alpha = (double *)calloc((size_t)desc->nelements, sizeof(double));
  h->boundaries_u = (double *)calloc((size_t)(2 * h->NV * h->NF * (desc->nboundaries > 0 ? desc->nboundaries : 1)), sizeof(double));
  for (int c = 0; c < h->nchild; ++c)
    h->mortar_u[c] = (double *)calloc((size_t)(2 * h->NV * h->NF * (desc->nmortars > 0 ? desc->nmortars : 1)), sizeof(double));
  return h;
}

void oracle_destroy(oracle_handle *h) {
  if (!h) return;
  free(h->interfaces_u); free(h->sfv); free(h->alpha); free(h->boundaries_u);
  for (int c = 0; c < 4; ++c) free(h->mortar_u[c]);
  free(h);
}

int64_t oracle_size(oracle_handle *h, int which) {
  switch (which) {
    case 0: return (int64_t)h->NV * h->NN * h->d.nelements;        /* u */
    case 1: return (int64_t)2 * h->NV * h->NF * h->d.ninterfaces;  /* interfaces_u */
    case 2: return (int64_t)h->NV * h->NF * 2 * h->DIM * h->d.nelements; /* surface_flux_values */
    case 3: return (int64_t)2 * h->NV * h->NF * h->d.nmortars;     /* one mortar u array */
    case 4: return h->nchild;
    case 5: return (int64_t)2 * h->NV * h->NF * h->d.nboundaries;  /* boundaries_u */
    default: return -1;
  }
}

/* node index of the point at position `a` along orientation o, with face
 * coordinates taken from face-node index f (remaining dimensions in order). */
static inline int node_of(int DIM, int N, int o, int a, int f) {
  int n = 0, stride = 1, ff = f;
  for (int d = 0; d < DIM; ++d) {
    int c;
    if (d == o) c = a;
    else { c = ff % N; ff /= N; }
    n += c * stride;
    stride *= N;
  }
  return n;
}

static inline int coord_of(int N, int n, int d) {
  for (int k = 0; k < d; ++k) n /= N;
  return n % N;
}

static inline int with_coord(int N, int n, int d, int c) {
  int s = 1;
  for (int k = 0; k < d; ++k) s *= N;
  return n - coord_of(N, n, d) * s + c * s;
}

/* ------------------------------------------------------------------------ */
/* Stages                                                                   */
/* ------------------------------------------------------------------------ */

void oracle_volume_integral(oracle_handle *h, double *du, const double *u, const double *alpha) {
  const int N = h->N, NN = h->NN, NV = h->NV, DIM = h->DIM;
  const int64_t E = h->d.nelements;
  const int kind = h->d.volume_integral;
  const phys_t *P = &h->P;
  /* atol = max(100 eps, eps^0.75) for Float64 (src/solvers/dg_2d.jl:173) */
  const double eps = 2.220446049250313e-16;
  const double atol = fmax(100 * eps, pow(eps, 0.75));
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < E; ++e) {
    const double *ue = u + (int64_t)NV * NN * e;
    double *due = du + (int64_t)NV * NN * e;
    if (kind == ORC_VOL_WEAK) {
      /* flux_weak_form_kernel!: du_i = sum_m sum_d dhat[i_d, m] f_d(u at m on line d) */
      static __thread double fl[3][NMAX * NMAX * NMAX * NVMAX];
      for (int n = 0; n < NN; ++n)
        for (int d = 0; d < DIM; ++d) flux_phys(P, ue + NV * n, d, &fl[d][NV * n]);
      for (int n = 0; n < NN; ++n)
        for (int v = 0; v < NV; ++v) {
          double val = 0;
          for (int m = 0; m < N; ++m)
            for (int d = 0; d < DIM; ++d) {
              int i = coord_of(N, n, d);
              int nm = with_coord(N, n, d, m);
              val += h->dhat[i + N * m] * fl[d][NV * nm + v];
            }
          due[NV * n + v] = val;
        }
      continue;
    }
    int dg_only = 1;
    double a = 0;
    if (kind == ORC_VOL_SHOCK_HG) {
      a = alpha[e];
      dg_only = fabs(a - 0.0) <= atol;
    }
    for (int n = 0; n < NN; ++n) {
      double val[NVMAX] = {0};
      if (!dg_only) {
        /* FV subcell fluxes between neighbouring LGL nodes on each line; the
         * element-boundary ones are zero (volume_flux_integral_dgfv_kernel!):
         * alpha * sum_d inv_w[i_d] * (fstar_d[i_d+1] - fstar_d[i_d]) */
        for (int d = 0; d < DIM; ++d) {
          int i = coord_of(N, n, d);
          double fr[NVMAX] = {0}, fl[NVMAX] = {0};
          if (i + 1 < N) {
            const double *un = ue + NV * with_coord(N, n, d, i + 1);
            two_point_flux(P, h->d.volume_flux_fv, ue + NV * n, un, d, fr);
            add_half_noncons(P, ue + NV * n, un, d, fr);  /* fstar_L (dg_2d_kernel.jl:650-656) */
          }
          if (i > 0) {
            const double *un = ue + NV * with_coord(N, n, d, i - 1);
            two_point_flux(P, h->d.volume_flux_fv, un, ue + NV * n, d, fl);
            add_half_noncons(P, ue + NV * n, un, d, fl);  /* fstar_R */
          }
          for (int v = 0; v < NV; ++v) val[v] += h->invw[i] * (fr[v] - fl[v]);
        }
        for (int v = 0; v < NV; ++v) val[v] = a * val[v];
      }
      /* DG flux differencing with zeroed diagonal, weighted by (1 - alpha) */
      for (int m = 0; m < N; ++m) {
        double f[3][NVMAX];
        int any = 0;
        for (int d = 0; d < DIM; ++d) {
          int i = coord_of(N, n, d);
          if (i == m) { for (int v = 0; v < NV; ++v) f[d][v] = 0; continue; }
          two_point_flux(P, h->d.volume_flux, ue + NV * n, ue + NV * with_coord(N, n, d, m), d, f[d]);
          any = 1;
        }
        if (!any) continue;
        for (int v = 0; v < NV; ++v) {
          double s = 0;
          for (int d = 0; d < DIM; ++d) {
            int i = coord_of(N, n, d);
            double Dm = (i == m) ? 0.0 : h->dsplit[i + N * m];
            s += (dg_only ? Dm : (1 - a) * Dm) * f[d][v];
          }
          val[v] += s;
        }
      }
      /* nonconservative terms: 0.5 sum_d sum_m D_split[i_d, m] Phi_d(u_n, u_m), the
       * full D_split row (dg_2d_kernel.jl:269-292, 729-741), weighted like the DG part */
      if (P->noncons == ORC_NONCONS_POWELL) {
        const double wdg = dg_only ? 1.0 : (1 - a);
        for (int d = 0; d < DIM; ++d) {
          int i = coord_of(N, n, d);
          for (int m = 0; m < N; ++m) {
            double nc[NVMAX];
            mhd_noncons_powell(P, ue + NV * n, ue + NV * with_coord(N, n, d, m), d, nc);
            const double Dm = h->dsplit[i + N * m];
            for (int v = 0; v < NV; ++v) val[v] += wdg * 0.5 * Dm * nc[v];
          }
        }
      }
      for (int v = 0; v < NV; ++v) due[NV * n + v] = val[v];
    }
  }
}

void oracle_prolong2interfaces(oracle_handle *h, const double *u, double *iu) {
  const int N = h->N, NN = h->NN, NF = h->NF, NV = h->NV, DIM = h->DIM;
  const int64_t I = h->d.ninterfaces;
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < I; ++k) {
    int o = (int)h->d.interface_orientations[k] - 1;
    int64_t left = h->d.interface_neighbor_ids[2 * k] - 1, right = h->d.interface_neighbor_ids[2 * k + 1] - 1;
    for (int f = 0; f < NF; ++f)
      for (int v = 0; v < NV; ++v) {
        iu[0 + 2 * (v + NV * (f + (int64_t)NF * k))] = u[v + NV * (node_of(DIM, N, o, N - 1, f) + (int64_t)NN * left)];
        iu[1 + 2 * (v + NV * (f + (int64_t)NF * k))] = u[v + NV * (node_of(DIM, N, o, 0, f) + (int64_t)NN * right)];
      }
  }
}

void oracle_interface_flux(oracle_handle *h, const double *iu, double *sfv) {
  const int NF = h->NF, NV = h->NV, DIM = h->DIM;
  const int64_t I = h->d.ninterfaces;
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < I; ++k) {
    int o = (int)h->d.interface_orientations[k] - 1;
    int64_t left = h->d.interface_neighbor_ids[2 * k] - 1, right = h->d.interface_neighbor_ids[2 * k + 1] - 1;
    for (int f = 0; f < NF; ++f) {
      double ul[NVMAX], ur[NVMAX], fs[NVMAX];
      for (int v = 0; v < NV; ++v) {
        ul[v] = iu[0 + 2 * (v + NV * (f + (int64_t)NF * k))];
        ur[v] = iu[1 + 2 * (v + NV * (f + (int64_t)NF * k))];
      }
      two_point_flux(&h->P, h->d.surface_flux, ul, ur, o, fs);
      /* with nonconservative terms each side adds 0.5 Phi(own, other)
       * (interface_flux_kernel!, dg_2d_kernel.jl:1009-1035) */
      double fl[NVMAX], fr[NVMAX];
      for (int v = 0; v < NV; ++v) fl[v] = fr[v] = fs[v];
      add_half_noncons(&h->P, ul, ur, o, fl);
      add_half_noncons(&h->P, ur, ul, o, fr);
      for (int v = 0; v < NV; ++v) {
        sfv[v + NV * (f + (int64_t)NF * ((2 * o + 1) + 2 * DIM * left))] = fl[v];
        sfv[v + NV * (f + (int64_t)NF * ((2 * o) + 2 * DIM * right))] = fr[v];
      }
    }
  }
}

/* index of the small-face node (a in first tangent dim, b in second) */
void oracle_prolong2mortars(oracle_handle *h, const double *u, double *const *mu) {
  const int N = h->N, NN = h->NN, NF = h->NF, NV = h->NV, DIM = h->DIM, nc = h->nchild;
  const int64_t M = h->d.nmortars;
#pragma omp parallel for schedule(static)
  for (int64_t m = 0; m < M; ++m) {
    int o = (int)h->d.mortar_orientations[m] - 1;
    int ls = (int)h->d.mortar_large_sides[m];
    int64_t large = h->d.mortar_neighbor_ids[nc + (nc + 1) * m] - 1;
    int small_side = (ls == 1) ? 1 : 0;          /* slot holding the small elements' trace */
    int small_a = (ls == 1) ? 0 : N - 1;         /* small elements' face along o */
    int large_a = (ls == 1) ? N - 1 : 0;         /* large element's face along o */
    for (int c = 0; c < nc; ++c) {
      int64_t small = h->d.mortar_neighbor_ids[c + (nc + 1) * m] - 1;
      double *arr = mu[c];
      for (int f = 0; f < NF; ++f)
        for (int v = 0; v < NV; ++v) {
          arr[small_side + 2 * (v + NV * (f + (int64_t)NF * m))] = u[v + NV * (node_of(DIM, N, o, small_a, f) + (int64_t)NN * small)];
          /* large -> small: tensor-product interpolation (forward_lower/upper) */
          double s = 0;
          if (DIM == 2) {
            const double *F = (c == 1) ? h->fup : h->flo;
            for (int jj = 0; jj < N; ++jj)
              s += F[f + N * jj] * u[v + NV * (node_of(DIM, N, o, large_a, jj) + (int64_t)NN * large)];
          } else {
            const double *F1 = (c & 1) ? h->fup : h->flo;   /* first tangent: left/right */
            const double *F2 = (c >> 1) ? h->fup : h->flo;  /* second tangent: lower/upper */
            int fa = f % N, fb = f / N;
            for (int jb = 0; jb < N; ++jb) {
              double t = 0;
              for (int ja = 0; ja < N; ++ja)
                t += F1[fa + N * ja] * u[v + NV * (node_of(DIM, N, o, large_a, ja + N * jb) + (int64_t)NN * large)];
              s += F2[fb + N * jb] * t;
            }
          }
          arr[(1 - small_side) + 2 * (v + NV * (f + (int64_t)NF * m))] = s;
        }
    }
  }
}

void oracle_mortar_flux(oracle_handle *h, double *const *mu, double *sfv) {
  const int N = h->N, NF = h->NF, NV = h->NV, DIM = h->DIM, nc = h->nchild;
  const int64_t M = h->d.nmortars;
  /* each mortar writes distinct faces of its small elements and one face of its
   * large element; a large element can own several mortars, but on different
   * faces, so mortars are independent. */
#pragma omp parallel for schedule(static)
  for (int64_t m = 0; m < M; ++m) {
    int o = (int)h->d.mortar_orientations[m] - 1;
    int ls = (int)h->d.mortar_large_sides[m];
    int64_t large = h->d.mortar_neighbor_ids[nc + (nc + 1) * m] - 1;
    int small_dir = 2 * o + (ls - 1);
    int large_dir = 2 * o + (ls == 1 ? 1 : 0);
    double fstar[4][NMAX * NMAX * NVMAX];
    for (int c = 0; c < nc; ++c) {
      int64_t small = h->d.mortar_neighbor_ids[c + (nc + 1) * m] - 1;
      for (int f = 0; f < NF; ++f) {
        double ul[NVMAX], ur[NVMAX], fs[NVMAX];
        for (int v = 0; v < NV; ++v) {
          ul[v] = mu[c][0 + 2 * (v + NV * (f + (int64_t)NF * m))];
          ur[v] = mu[c][1 + 2 * (v + NV * (f + (int64_t)NF * m))];
        }
        two_point_flux(&h->P, h->d.surface_flux, ul, ur, o, fs);
        /* nonconservative terms (mortar_flux_kernel!, dg_2d_kernel.jl:1290-1344):
         * the small elements get 0.5 Phi(u_large, u_small) ("primary"), the
         * projection to the large element 0.5 Phi(u_small, u_large) ("secondary"),
         * u_large being the large element's trace projected onto the mortar */
        double fp[NVMAX], fsec[NVMAX];
        for (int v = 0; v < NV; ++v) fp[v] = fsec[v] = fs[v];
        const double *u_large = (ls == 1) ? ul : ur, *u_small = (ls == 1) ? ur : ul;
        add_half_noncons(&h->P, u_large, u_small, o, fp);
        add_half_noncons(&h->P, u_small, u_large, o, fsec);
        for (int v = 0; v < NV; ++v) {
          fstar[c][v + NV * f] = fsec[v];
          sfv[v + NV * (f + (int64_t)NF * (small_dir + 2 * DIM * small))] = fp[v];
        }
      }
    }
    /* large face: L2 back-projection reverse_lower/upper (tensor product in 3D) */
    for (int f = 0; f < NF; ++f)
      for (int v = 0; v < NV; ++v) {
        double s = 0;
        if (DIM == 2) {
          for (int c = 0; c < nc; ++c) {
            const double *R = (c == 1) ? h->rup : h->rlo;
            for (int jj = 0; jj < N; ++jj) s += R[f + N * jj] * fstar[c][v + NV * jj];
          }
        } else {
          int fa = f % N, fb = f / N;
          for (int c = 0; c < nc; ++c) {
            const double *R1 = (c & 1) ? h->rup : h->rlo;
            const double *R2 = (c >> 1) ? h->rup : h->rlo;
            for (int jb = 0; jb < N; ++jb) {
              double t = 0;
              for (int ja = 0; ja < N; ++ja) t += R1[fa + N * ja] * fstar[c][v + NV * (ja + N * jb)];
              s += R2[fb + N * jb] * t;
            }
          }
        }
        sfv[v + NV * (f + (int64_t)NF * (large_dir + 2 * DIM * large))] = s;
      }
  }
}

void oracle_surface_integral(oracle_handle *h, double *du, const double *sfv) {
  const int N = h->N, NN = h->NN, NF = h->NF, NV = h->NV, DIM = h->DIM;
  const int64_t E = h->d.nelements;
  const double factor1 = 1.0 / h->w[0], factor2 = 1.0 / h->w[N - 1];  /* lhat(-1)[1], lhat(+1)[N] */
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < E; ++e)
    for (int n = 0; n < NN; ++n) {
      int on_face = 0;
      for (int d = 0; d < DIM; ++d) { int c = coord_of(N, n, d); if (c == 0 || c == N - 1) on_face = 1; }
      if (!on_face) continue;
      for (int v = 0; v < NV; ++v) {
        double neg = 0, pos = 0;
        for (int d = 0; d < DIM; ++d) {
          int c = coord_of(N, n, d);
          /* face-node index of n on a face normal to d */
          int f = 0, stride = 1;
          for (int dd = 0; dd < DIM; ++dd) {
            if (dd == d) continue;
            f += coord_of(N, n, dd) * stride;
            stride *= N;
          }
          if (c == 0) neg += sfv[v + NV * (f + (int64_t)NF * (2 * d + 2 * DIM * e))];
          if (c == N - 1) pos += sfv[v + NV * (f + (int64_t)NF * (2 * d + 1 + 2 * DIM * e))];
        }
        du[v + NV * (n + (int64_t)NN * e)] -= neg * factor1;
        du[v + NV * (n + (int64_t)NN * e)] += pos * factor2;
      }
    }
}

void oracle_jacobian(oracle_handle *h, double *du) {
  const int64_t E = h->d.nelements, per = (int64_t)h->NV * h->NN;
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < E; ++e) {
    double s = -h->d.inverse_jacobian[e];
    for (int64_t i = 0; i < per; ++i) du[i + per * e] *= s;
  }
}

/* Hennemann-Gassner indicator on rho*p with optional neighbour smoothing. */
void oracle_indicator_hg(oracle_handle *h, const double *u, double *alpha) {
  const int N = h->N, NN = h->NN, NV = h->NV, DIM = h->DIM, nc = h->nchild;
  const int64_t E = h->d.nelements;
  const double threshold = 0.5 * pow(10.0, -1.8 * pow((double)N, 0.25));
  const double o_0001 = 0.0001;
  const double parameter_s = log((1 - o_0001) / o_0001);
  const double amax = h->d.alpha_max, amin = h->d.alpha_min;
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < E; ++e) {
    double ind[NMAX * NMAX * NMAX], tmp[NMAX * NMAX * NMAX];
    for (int n = 0; n < NN; ++n) {
      const double *un = u + NV * (n + (int64_t)NN * e);
      double rho, v[3], p;
      cons2prim(&h->P, un, &rho, v, &p);
      ind[n] = h->d.indicator_variable ? p : rho * p;
    }
    /* modal coefficients: inverse Vandermonde applied dimension by dimension */
    for (int d = 0; d < DIM; ++d) {
      for (int n = 0; n < NN; ++n) {
        int i = coord_of(N, n, d);
        double s = 0;
        for (int m = 0; m < N; ++m) s += h->ivdm[i + N * m] * ind[with_coord(N, n, d, m)];
        tmp[n] = s;
      }
      memcpy(ind, tmp, sizeof(double) * NN);
    }
    double total = 0, clip1 = 0, clip2 = 0;
    for (int n = 0; n < NN; ++n) {
      int maxc = 0;
      for (int d = 0; d < DIM; ++d) { int c = coord_of(N, n, d); if (c > maxc) maxc = c; }
      double m2 = ind[n] * ind[n];
      total += m2;
      if (maxc < N - 1) clip1 += m2;
      if (maxc < N - 2) clip2 += m2;
    }
    double f1 = (total != 0) ? (total - clip1) / total : 0.0;
    double f2 = (clip1 != 0) ? (clip1 - clip2) / clip1 : 0.0;
    double energy = fmax(f1, f2);
    double a = 1.0 / (1.0 + exp(-parameter_s / threshold * (energy - threshold)));
    if (a < amin) a = 0.0;
    if (a > 1 - amin) a = 1.0;
    alpha[e] = fmin(amax, a);
  }
  if (h->d.alpha_smooth) {
    double *tmp = (double *)malloc(sizeof(double) * (size_t)E);
    memcpy(tmp, alpha, sizeof(double) * (size_t)E);
    for (int64_t k = 0; k < h->d.ninterfaces; ++k) {
      int64_t l = h->d.interface_neighbor_ids[2 * k] - 1, r = h->d.interface_neighbor_ids[2 * k + 1] - 1;
      alpha[l] = fmax(fmax(tmp[l], 0.5 * tmp[r]), alpha[l]);
      alpha[r] = fmax(fmax(tmp[r], 0.5 * tmp[l]), alpha[r]);
    }
    for (int64_t m = 0; m < h->d.nmortars; ++m) {
      int64_t large = h->d.mortar_neighbor_ids[nc + (nc + 1) * m] - 1;
      for (int c = 0; c < nc; ++c) {
        int64_t s = h->d.mortar_neighbor_ids[c + (nc + 1) * m] - 1;
        alpha[s] = fmax(fmax(tmp[s], 0.5 * tmp[large]), alpha[s]);
        alpha[large] = fmax(fmax(tmp[large], 0.5 * tmp[s]), alpha[large]);
      }
    }
    free(tmp);
  }
}

/* ------------------------------------------------------------------------ */
/* Boundary states, boundary fluxes and source terms                        */
/* ------------------------------------------------------------------------ */

/* The built-in initial conditions, also the Dirichlet boundary functions:
 * constant state; the convergence test (advection: c + A sin(omega sum_d
 * (x_d - a_d t)); Euler: rho = rho v_d = c + A sin(omega (sum_d x_d - t)),
 * E = rho^2 -- a manufactured solution of the Euler equations with the
 * source term of oracle_sources); the weak blast wave. */
/* Ideal GLM-MHD states: the circularly polarised Alfven waves of the MHD
 * convergence tests (1D/2D after Derigs et al., JCP 317 (2016): rho = 1,
 * p = 0.1, amplitude 0.1, unit background field along the propagation
 * direction -- the x axis in 1D, the diagonal alpha = pi/4 in 2D -- speed 1;
 * 3D after Altmann's thesis (2012): direction (1, 0, 2)/sqrt 5 on [-1, 1]^3,
 * amplitude 0.2, p = 1), and the weak blast wave in the uniform field
 * B = (1, 1, 1); psi = 0 where the system carries it. */
static void eval_ic_mhd(const oracle_handle *h, int kind, const double *x, double t, double *u) {
  const int DIM = h->DIM, NV = h->NV;
  double rho = 1.0, v[3] = {0.0, 0.0, 0.0}, p = 1.0, B[3] = {1.0, 1.0, 1.0};
  if (kind == ORC_IC_CONVERGENCE_TEST) {
    if (DIM == 1) {
      const double ph = 2.0 * ORC_PI * (x[0] + t);
      v[1] = 0.1 * sin(ph);
      v[2] = 0.1 * cos(ph);
      p = 0.1;
      B[0] = 1.0; B[1] = v[1]; B[2] = v[2];
    } else if (DIM == 2) {
      const double ca = cos(0.25 * ORC_PI), sa = sin(0.25 * ORC_PI);
      const double ph = 2.0 * ORC_PI * (x[0] * ca + x[1] * sa + t);
      const double b_perp = 0.1 * sin(ph);
      v[0] = -b_perp * sa; v[1] = b_perp * ca; v[2] = 0.1 * cos(ph);
      p = 0.1;
      B[0] = ca + v[0]; B[1] = sa + v[1]; B[2] = v[2];
    } else {
      const double r = 2.0, amp = 0.2, k = 2.0 * ORC_PI;
      const double nx = 1.0 / sqrt(r * r + 1.0), nz = r / sqrt(r * r + 1.0);
      const double ph = k / nz * (nx * (x[0] - 0.5 * r) + nz * (x[2] - 0.5 * r)) - k / nz * t;
      v[0] = -amp * nz * cos(ph); v[1] = amp * sin(ph); v[2] = amp * nx * cos(ph);
      B[0] = nx - v[0]; B[1] = -v[1]; B[2] = nz - v[2];
    }
  } else { /* weak blast wave: the Euler states below in B = (1, 1, 1) */
    double r2 = 0.0;
    for (int d = 0; d < DIM; ++d) r2 += x[d] * x[d];
    const double r = sqrt(r2);
    if (r <= 0.5) {
      rho = 1.1691; p = 1.245;
      if (DIM == 1) {
        v[0] = x[0] > 0.0 ? 0.1882 : (x[0] < 0.0 ? -0.1882 : 0.0);
      } else if (DIM == 2) {
        const double phi = atan2(x[1], x[0]);
        v[0] = 0.1882 * cos(phi); v[1] = 0.1882 * sin(phi);
      } else {
        const double phi = atan2(x[1], x[0]);
        double c = r > 0.0 ? x[2] / r : 1.0;
        c = c > 1.0 ? 1.0 : (c < -1.0 ? -1.0 : c);
        const double theta = r > 0.0 ? acos(c) : 0.0;
        v[0] = 0.1882 * cos(phi) * sin(theta); v[1] = 0.1882 * sin(phi) * sin(theta); v[2] = 0.1882 * cos(theta);
      }
    }
  }
  double kin = 0.0, mag = 0.0;
  u[0] = rho;
  for (int d = 0; d < 3; ++d) {
    u[1 + d] = rho * v[d];
    u[5 + d] = B[d];
    kin += v[d] * v[d];
    mag += B[d] * B[d];
  }
  u[4] = p / (h->P.gamma - 1.0) + 0.5 * rho * kin + 0.5 * mag;
  if (NV == 9) u[8] = 0.0;
}

void oracle_eval_ic(oracle_handle *h, int kind, const double *params, const double *x, double t, double *u) {
  const int DIM = h->DIM, NV = h->NV;
  if (kind == ORC_IC_CONSTANT) {
    for (int v = 0; v < NV; ++v) u[v] = params[v];
    return;
  }
  if (h->P.eq == ORC_EQ_MHD) {
    eval_ic_mhd(h, kind, x, t, u);
    return;
  }
  if (kind == ORC_IC_CONVERGENCE_TEST) {
    const double c = params[0], A = params[1], L = params[2];
    const double omega = 2.0 * ORC_PI / L;
    double s = 0.0;
    if (h->P.eq == ORC_EQ_ADVECTION) {
      for (int d = 0; d < DIM; ++d) s += x[d] - h->P.a[d] * t;
      u[0] = c + A * sin(omega * s);
      return;
    }
    for (int d = 0; d < DIM; ++d) s += x[d];
    const double ini = c + A * sin(omega * (s - t));
    u[0] = ini;
    for (int d = 0; d < DIM; ++d) u[1 + d] = ini;
    u[DIM + 1] = ini * ini;
    return;
  }
  if (kind == ORC_IC_EOC_EULER_GRAVITY) {
    /* Euler-gravity convergence test (Schlottke-Lakemper et al., JCP 442 (2021)):
     * rho = 2 + 0.1 sin(pi (sum x - t)), v_d = 1, and the pressure of
     * hydrostatic balance grad p = -rho grad phi with lap phi = 4 pi G rho,
     * G = 1: p = 2 rho^2 / (DIM pi) */
    double sx = 0.0;
    for (int d = 0; d < DIM; ++d) sx += x[d];
    const double rho = 2.0 + 0.1 * sin(ORC_PI * (sx - t));
    const double p = 2.0 * rho * rho / (DIM * ORC_PI);
    u[0] = rho;
    for (int d = 0; d < DIM; ++d) u[1 + d] = rho;
    u[DIM + 1] = p / (h->P.gamma - 1.0) + 0.5 * rho * DIM;
    return;
  }
  /* weak blast wave: r <= 0.5: rho 1.1691, radial velocity 0.1882, p 1.245; else 1, 0, 1.
   * The radial direction from the polar angles phi = atan2(y, x) (and
   * theta = acos(z / r) in 3D), so that the centre itself moves along phi = 0
   * (theta = 0 in 3D), as the angle-based definition gives there. */
  double r2 = 0.0, v[3] = {0.0, 0.0, 0.0};
  for (int d = 0; d < DIM; ++d) r2 += x[d] * x[d];
  const double r = sqrt(r2);
  const int inside = r <= 0.5;
  const double rho = inside ? 1.1691 : 1.0, p = inside ? 1.245 : 1.0;
  if (inside) {
    if (DIM == 1) {
      v[0] = x[0] > 0.0 ? 0.1882 : (x[0] < 0.0 ? -0.1882 : 0.0);
    } else if (DIM == 2) {
      const double phi = atan2(x[1], x[0]);
      v[0] = 0.1882 * cos(phi);
      v[1] = 0.1882 * sin(phi);
    } else {
      const double phi = atan2(x[1], x[0]);
      double c = r > 0.0 ? x[2] / r : 1.0;
      c = c > 1.0 ? 1.0 : (c < -1.0 ? -1.0 : c);
      const double theta = r > 0.0 ? acos(c) : 0.0;
      v[0] = 0.1882 * cos(phi) * sin(theta);
      v[1] = 0.1882 * sin(phi) * sin(theta);
      v[2] = 0.1882 * cos(theta);
    }
  }
  double kin = 0.0;
  u[0] = rho;
  for (int d = 0; d < DIM; ++d) {
    u[1 + d] = rho * v[d];
    kin += v[d] * v[d];
  }
  u[DIM + 1] = p / (h->P.gamma - 1.0) + 0.5 * rho * kin;
}

static const double *node_x(const oracle_handle *h, int64_t e, int n) {
  return h->d.node_coordinates + (size_t)h->DIM * ((size_t)n + (size_t)h->NN * (size_t)e);
}

/* boundaries_u[2, nv, N^(d-1), nboundaries]: the element's trace on its side
 * of the boundary, zero on the other (prolong_boundaries_kernel!). */
void oracle_prolong2boundaries(oracle_handle *h, const double *u, double *bu) {
  const int N = h->N, NN = h->NN, NF = h->NF, NV = h->NV, DIM = h->DIM;
  const int64_t B = h->d.nboundaries;
#pragma omp parallel for schedule(static)
  for (int64_t b = 0; b < B; ++b) {
    const int64_t e = h->d.boundary_neighbor_ids[b] - 1;
    const int side = (int)h->d.boundary_neighbor_sides[b], o = (int)h->d.boundary_orientations[b] - 1;
    for (int f = 0; f < NF; ++f)
      for (int v = 0; v < NV; ++v) {
        const double in = u[v + NV * (node_of(DIM, N, o, side == 1 ? N - 1 : 0, f) + (int64_t)NN * e)];
        bu[0 + 2 * (v + NV * (f + (int64_t)NF * b))] = side == 1 ? in : 0.0;
        bu[1 + 2 * (v + NV * (f + (int64_t)NF * b))] = side == 2 ? in : 0.0;
      }
  }
}

/* Dirichlet boundaries: the numerical flux between the inner trace and the
 * boundary function's state at the face node, the inner state on the left
 * for a boundary on the element's upper face (directions 2, 4, 6)
 * (boundary_flux_kernel!, dg_2d_kernel.jl:1067-1110). The reference's
 * boundary condition evaluates the nonconservative part inside Trixi.jl,
 * outside the repository; the element's side of an interface is taken:
 * 0.5 Phi(u_inner, u_boundary). */
void oracle_boundary_flux(oracle_handle *h, const double *bu, double t, double *sfv) {
  const int N = h->N, NF = h->NF, NV = h->NV, DIM = h->DIM;
  const int64_t B = h->d.nboundaries;
#pragma omp parallel for schedule(static)
  for (int64_t b = 0; b < B; ++b) {
    const int64_t e = h->d.boundary_neighbor_ids[b] - 1;
    const int side = (int)h->d.boundary_neighbor_sides[b], o = (int)h->d.boundary_orientations[b] - 1;
    const int dir = 2 * o + (side == 1 ? 1 : 0);
    for (int f = 0; f < NF; ++f) {
      double ui[NVMAX], ub[NVMAX], fs[NVMAX];
      for (int v = 0; v < NV; ++v) ui[v] = bu[(side - 1) + 2 * (v + NV * (f + (int64_t)NF * b))];
      const double *x = node_x(h, e, node_of(DIM, N, o, side == 1 ? N - 1 : 0, f));
      oracle_eval_ic(h, h->d.boundary_function, h->d.boundary_params, x, t, ub);
      if (side == 1)
        two_point_flux(&h->P, h->d.surface_flux, ui, ub, o, fs);
      else
        two_point_flux(&h->P, h->d.surface_flux, ub, ui, o, fs);
      /* nonconservative terms as on the element's side of an interface:
       * 0.5 Phi(u_inner, u_boundary) */
      add_half_noncons(&h->P, ui, ub, o, fs);
      for (int v = 0; v < NV; ++v) sfv[v + NV * (f + (int64_t)NF * (dir + 2 * DIM * e))] = fs[v];
    }
  }
}

/* Source term of the Euler convergence test: S = du/dt + div F(u) of the
 * manufactured solution rho = rho v_d = c + A sin(omega (sum x - t)),
 * E = rho^2 (derived symbolically; rho_x = omega A cos(omega (sum x - t))):
 *   1D: (0, rho_x (g-1)(4 rho - 1)/2, same)
 *   2D: (rho_x, rho_x (2 g rho - g - 2 rho + 2) [x2], 2 rho_x (2 g rho - g - rho + 1))
 *   3D: (2 rho_x, rho_x (4 g rho - 3 g - 4 rho + 7)/2 [x3], rho_x (12 g rho - 9 g - 4 rho + 9)/2)
 * added to du after the Jacobian, as calc_sources! does. */
static void source_convergence(int DIM, double g, const double *prm, const double *x, double t, double *s) {
  const double c = prm[0], A = prm[1], L = prm[2], omega = 2.0 * ORC_PI / L;
  double sx = 0.0;
  for (int d = 0; d < DIM; ++d) sx += x[d];
  const double rho = c + A * sin(omega * (sx - t)), rx = omega * A * cos(omega * (sx - t));
  if (DIM == 1) {
    s[0] = 0.0;
    s[1] = s[2] = 0.5 * rx * (g - 1.0) * (4.0 * rho - 1.0);
  } else if (DIM == 2) {
    s[0] = rx;
    s[1] = s[2] = rx * (2.0 * g * rho - g - 2.0 * rho + 2.0);
    s[3] = 2.0 * rx * (2.0 * g * rho - g - rho + 1.0);
  } else {
    s[0] = 2.0 * rx;
    s[1] = s[2] = s[3] = 0.5 * rx * (4.0 * g * rho - 3.0 * g - 4.0 * rho + 7.0);
    s[4] = 0.5 * rx * (12.0 * g * rho - 9.0 * g - 4.0 * rho + 9.0);
  }
}

/* Source of the Euler-gravity convergence test without gravity
 * (source_terms_eoc_test_euler of test/tree_dgsem_3d/euler_convergence.jl:24):
 * S_q = d U_q/dt + sum_k d F_k,q / dx_k on the manufactured solution of
 * ORC_IC_EOC_EULER_GRAVITY, by the chain rule in the phase
 * xi = pi (sum x - t): d/dt = -r', d/dx_k = +r' with r' = pi A cos(xi) times
 * the derivative in rho; U = (rho, rho [DIM], E), F_k = (rho, rho + delta_ik p,
 * E + p) as v = 1; E(rho) = p/(g-1) + DIM rho/2, p(rho) = K rho^2, K = 2/(DIM pi). */
static void source_eoc_euler(int DIM, double g, const double *x, double t, double *s) {
  const double A = 0.1, K = 2.0 / (DIM * ORC_PI);
  double sx = 0.0;
  for (int d = 0; d < DIM; ++d) sx += x[d];
  const double rho = 2.0 + A * sin(ORC_PI * (sx - t));
  const double rp = ORC_PI * A * cos(ORC_PI * (sx - t));
  const double dp = 2.0 * K * rho, dE = dp / (g - 1.0) + 0.5 * DIM;
  s[0] = -rp;
  for (int k = 0; k < DIM; ++k) s[0] += rp;
  for (int i = 0; i < DIM; ++i) {
    s[1 + i] = -rp;
    for (int k = 0; k < DIM; ++k) s[1 + i] += rp * (1.0 + (k == i ? dp : 0.0));
  }
  s[DIM + 1] = -dE * rp;
  for (int k = 0; k < DIM; ++k) s[DIM + 1] += (dE + dp) * rp;
}

void oracle_sources(oracle_handle *h, double *du, double t) {
  if (h->d.source_terms == ORC_SRC_NONE || h->P.eq != ORC_EQ_EULER) return;
  if (h->d.source_terms == ORC_SRC_EOC_EULER) {
    const int NN = h->NN, NV = h->NV;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < h->d.nelements; ++e)
      for (int n = 0; n < NN; ++n) {
        double s[NVMAX];
        source_eoc_euler(h->DIM, h->P.gamma, node_x(h, e, n), t, s);
        for (int v = 0; v < NV; ++v) du[v + NV * (n + (int64_t)NN * e)] += s[v];
      }
    return;
  }
  const int NN = h->NN, NV = h->NV;
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < h->d.nelements; ++e)
    for (int n = 0; n < NN; ++n) {
      double s[NVMAX];
      source_convergence(h->DIM, h->P.gamma, h->d.source_params, node_x(h, e, n), t, s);
      for (int v = 0; v < NV; ++v) du[v + NV * (n + (int64_t)NN * e)] += s[v];
    }
}

void oracle_rhs(oracle_handle *h, double *du, const double *u, double t) {
  if (h->d.volume_integral == ORC_VOL_SHOCK_HG) oracle_indicator_hg(h, u, h->alpha);
  oracle_volume_integral(h, du, u, h->alpha);
  oracle_prolong2interfaces(h, u, h->interfaces_u);
  oracle_interface_flux(h, h->interfaces_u, h->sfv);
  if (h->d.nboundaries > 0) {  /* periodic meshes have none (src/solvers/dg_2d.jl:419-450) */
    oracle_prolong2boundaries(h, u, h->boundaries_u);
    oracle_boundary_flux(h, h->boundaries_u, t, h->sfv);
  }
  if (h->d.nmortars > 0) {
    oracle_prolong2mortars(h, u, h->mortar_u);
    oracle_mortar_flux(h, h->mortar_u, h->sfv);
  }
  oracle_surface_integral(h, du, h->sfv);
  oracle_jacobian(h, du);
  oracle_sources(h, du, t);
}

/* CarpenterKennedy2N54 (Carpenter & Kennedy 1994, five-stage fourth-order,
 * 2N storage):  k <- A_s k + dt L(u, t + c_s dt);  u <- u + B_s k. */
static const double CK_A[5] = {0.0, -567301805773.0 / 1357537059087.0, -2404267990393.0 / 2016746695238.0,
                               -3550918686646.0 / 2091501179385.0, -1275806237668.0 / 842570457699.0};
static const double CK_B[5] = {1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
                               1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
                               2277821191437.0 / 14882151754819.0};
static const double CK_C[5] = {0.0, 1432997174477.0 / 9575080441755.0, 2526269341429.0 / 6820363962896.0,
                               2006345519317.0 / 3224310063776.0, 2802321613138.0 / 2924317926251.0};

void oracle_rk_ck2n54(oracle_handle *h, double *u, double *k, double t, double dt, int nsteps) {
  int64_t n = (int64_t)h->NV * h->NN * h->d.nelements;
  double *du = (double *)malloc(sizeof(double) * (size_t)n);
  for (int step = 0; step < nsteps; ++step) {
    for (int s = 0; s < 5; ++s) {
      oracle_rhs(h, du, u, t + CK_C[s] * dt);
      double a = CK_A[s], b = CK_B[s];
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; ++i) {
        k[i] = a * k[i] + dt * du[i];
        u[i] = u[i] + b * k[i];
      }
    }
    t += dt;
  }
  free(du);
}

/* Pointwise fluxes of the handle's equations (for the flux pins of the tests). */
void oracle_physical_flux(oracle_handle *h, const double *u, int o, double *f) { flux_phys(&h->P, u, o, f); }
void oracle_two_point_flux(oracle_handle *h, int kind, const double *ul, const double *ur, int o, double *f) {
  two_point_flux(&h->P, kind, ul, ur, o, f);
}
void oracle_noncons_flux(oracle_handle *h, const double *ul, const double *ur, int o, double *f) {
  for (int v = 0; v < h->NV; ++v) f[v] = 0.0;
  if (h->P.noncons == ORC_NONCONS_POWELL) mhd_noncons_powell(&h->P, ul, ur, o, f);
}
