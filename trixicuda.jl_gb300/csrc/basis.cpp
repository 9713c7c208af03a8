// basis.cpp -- Lobatto-Legendre basis and L2 mortar operators (host, FP64
// results computed in long double).
//
// Replaces LobattoLegendreBasisGPU / MortarL2GPU
// (src/solvers/basis_lobatto_legendre.jl:60-100, 155-173), whose arithmetic
// comes from Trixi.jl.  Restated from Kopriva (2009): LGL nodes as the roots
// of (1 - x^2) L'_p(x), weights 2/(p(p+1) L_p(x_j)^2), barycentric Lagrange
// interpolation, derivative matrix with the negative-sum diagonal; the split
// operator D_split = 2D - M^{-1}B (Gassner, Winters, Kopriva 2016); the weak
// operator D_hat = -M^{-1} D^T M; orthonormal Legendre Vandermonde for the
// indicator; mortar forward interpolation and exact L2 back projection
// (Kopriva 1996).
#include "basis.h"

#include <cmath>
#include <vector>

namespace trixi {

namespace {
using real_t = long double;
const real_t kPi = 3.141592653589793238462643383279502884L;

struct LegendreValue {
  real_t p, dp;
};

LegendreValue legendre_value(int n, real_t x) {
  real_t p0 = 1, p1 = x, d0 = 0, d1 = 1;
  if (n == 0) return {1, 0};
  for (int k = 2; k <= n; ++k) {
    real_t p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
    real_t d2 = d0 + (2 * k - 1) * p1;
    p0 = p1;
    p1 = p2;
    d0 = d1;
    d1 = d2;
  }
  return {p1, d1};
}

real_t orthonormal_legendre(int n, real_t x) { return legendre_value(n, x).p * std::sqrt(n + real_t(0.5)); }

std::vector<real_t> lobatto_nodes(int n) {
  const int p = n - 1;
  std::vector<real_t> x(n);
  x.front() = -1;
  x.back() = 1;
  for (int j = 1; j < p; ++j) {
    real_t z = -std::cos(kPi * j / p);
    for (int it = 0; it < 200; ++it) {
      LegendreValue lv = legendre_value(p, z);
      // Newton on L'_p, with L''_p from the Legendre ODE
      real_t d2 = (2 * z * lv.dp - p * (p + 1) * lv.p) / (1 - z * z);
      real_t step = lv.dp / d2;
      z -= step;
      if (std::fabs(step) <= 1e-32L) break;
    }
    x[j] = z;
  }
  for (int j = 0; j < n / 2; ++j) {
    real_t s = (x[n - 1 - j] - x[j]) / 2;
    x[j] = -s;
    x[n - 1 - j] = s;
  }
  if (n % 2) x[n / 2] = 0;
  return x;
}

std::vector<real_t> lobatto_weights(const std::vector<real_t> &x) {
  const int n = (int)x.size(), p = n - 1;
  std::vector<real_t> w(n);
  for (int j = 0; j < n; ++j) {
    real_t lp = legendre_value(p, x[j]).p;
    w[j] = 2 / (p * (p + 1) * lp * lp);
  }
  return w;
}

void gauss_rule(int n, std::vector<real_t> &x, std::vector<real_t> &w) {
  x.resize(n);
  w.resize(n);
  for (int j = 0; j < n; ++j) {
    real_t z = -std::cos(kPi * (j + real_t(0.75)) / (n + real_t(0.5)));
    for (int it = 0; it < 200; ++it) {
      LegendreValue lv = legendre_value(n, z);
      real_t step = lv.p / lv.dp;
      z -= step;
      if (std::fabs(step) <= 1e-32L) break;
    }
    real_t dp = legendre_value(n, z).dp;
    x[j] = z;
    w[j] = 2 / ((1 - z * z) * dp * dp);
  }
}

std::vector<real_t> bary(const std::vector<real_t> &x) {
  const int n = (int)x.size();
  std::vector<real_t> lam(n, 1);
  for (int j = 0; j < n; ++j)
    for (int k = 0; k < n; ++k)
      if (k != j) lam[j] /= (x[j] - x[k]);
  return lam;
}

std::vector<real_t> lagrange(const std::vector<real_t> &x, const std::vector<real_t> &lam, real_t xi) {
  const int n = (int)x.size();
  std::vector<real_t> l(n, 0);
  for (int j = 0; j < n; ++j)
    if (xi == x[j]) {
      l[j] = 1;
      return l;
    }
  real_t den = 0;
  for (int j = 0; j < n; ++j) {
    l[j] = lam[j] / (xi - x[j]);
    den += l[j];
  }
  for (auto &v : l) v /= den;
  return l;
}

bool gauss_jordan_inverse(int n, std::vector<real_t> a, std::vector<real_t> &inv) {
  // a, inv: column-major n x n
  inv.assign((size_t)n * n, 0);
  for (int i = 0; i < n; ++i) inv[i + (size_t)n * i] = 1;
  for (int c = 0; c < n; ++c) {
    int piv = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(a[r + (size_t)n * c]) > std::fabs(a[piv + (size_t)n * c])) piv = r;
    if (a[piv + (size_t)n * c] == 0) return false;
    for (int j = 0; j < n; ++j) {
      std::swap(a[c + (size_t)n * j], a[piv + (size_t)n * j]);
      std::swap(inv[c + (size_t)n * j], inv[piv + (size_t)n * j]);
    }
    const real_t d = a[c + (size_t)n * c];
    for (int j = 0; j < n; ++j) {
      a[c + (size_t)n * j] /= d;
      inv[c + (size_t)n * j] /= d;
    }
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      const real_t f = a[r + (size_t)n * c];
      if (f == 0) continue;
      for (int j = 0; j < n; ++j) {
        a[r + (size_t)n * j] -= f * a[c + (size_t)n * j];
        inv[r + (size_t)n * j] -= f * inv[c + (size_t)n * j];
      }
    }
  }
  return true;
}
}  // namespace

bool compute_basis(int polydeg, Basis &b) {
  const int n = polydeg + 1;
  if (n < 2 || n > 16) return false;
  b.n = n;
  const auto x = lobatto_nodes(n);
  const auto w = lobatto_weights(x);
  const auto lam = bary(x);
  const size_t nn = (size_t)n * n;
  std::vector<real_t> D(nn);
  for (int i = 0; i < n; ++i) {
    real_t diag = 0;
    for (int j = 0; j < n; ++j) {
      if (j == i) continue;
      D[i + (size_t)n * j] = lam[j] / lam[i] / (x[i] - x[j]);
      diag -= D[i + (size_t)n * j];
    }
    D[i + (size_t)n * i] = diag;
  }
  b.nodes.resize(n);
  b.weights.resize(n);
  b.dmat.resize(nn);
  b.dsplit.resize(nn);
  b.dhat.resize(nn);
  for (int i = 0; i < n; ++i) {
    b.nodes[i] = (double)x[i];
    b.weights[i] = (double)w[i];
  }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      const size_t ij = i + (size_t)n * j;
      b.dmat[ij] = (double)D[ij];
      real_t s = 2 * D[ij];
      if (i == j && i == 0) s += 1 / w[0];
      if (i == j && i == n - 1) s -= 1 / w[n - 1];
      b.dsplit[ij] = (double)s;
      b.dhat[ij] = (double)(-D[j + (size_t)n * i] * w[j] / w[i]);
    }
  std::vector<real_t> V(nn), Vi;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) V[i + (size_t)n * j] = orthonormal_legendre(j, x[i]);
  if (!gauss_jordan_inverse(n, V, Vi)) return false;
  b.ivdm.resize(nn);
  for (size_t i = 0; i < nn; ++i) b.ivdm[i] = (double)Vi[i];
  // forward: F_upper[j, i] = l_i((x_j + 1)/2), F_lower[j, i] = l_i((x_j - 1)/2)
  b.fwd_up.resize(nn);
  b.fwd_lo.resize(nn);
  for (int j = 0; j < n; ++j) {
    const auto lu = lagrange(x, lam, (x[j] + 1) / 2);
    const auto ll = lagrange(x, lam, (x[j] - 1) / 2);
    for (int i = 0; i < n; ++i) {
      b.fwd_up[j + (size_t)n * i] = (double)lu[i];
      b.fwd_lo[j + (size_t)n * i] = (double)ll[i];
    }
  }
  // reverse: exact L2 projection of a small-face polynomial (nodal values on
  // the small face's LGL nodes) onto P_{n-1} of the large face, expanded in
  // orthonormal Legendre polynomials and evaluated at the LGL nodes.
  std::vector<real_t> gx, gw;
  gauss_rule(n + 1, gx, gw);
  b.rev_up.resize(nn);
  b.rev_lo.resize(nn);
  for (int half = 0; half < 2; ++half) {
    const real_t shift = half ? 1 : -1;
    std::vector<double> &R = half ? b.rev_up : b.rev_lo;
    for (int j = 0; j < n; ++j) {
      std::vector<real_t> coef(n, 0);
      for (size_t q = 0; q < gx.size(); ++q) {
        const real_t lj = lagrange(x, lam, gx[q])[j];
        const real_t xi = (gx[q] + shift) / 2;  // point of the large face
        for (int m = 0; m < n; ++m) coef[m] += gw[q] * orthonormal_legendre(m, xi) * lj / 2;
      }
      for (int k = 0; k < n; ++k) {
        real_t val = 0;
        for (int m = 0; m < n; ++m) val += orthonormal_legendre(m, x[k]) * coef[m];
        R[k + (size_t)n * j] = (double)val;
      }
    }
  }
  return true;
}

bool lgl_weights_fixed(int polydeg, double *w_out) {
  const int n = polydeg + 1;
  if (n < 2 || n > 16) return false;
  const int p = polydeg;
  real_t x[16];
  x[0] = -1;
  x[n - 1] = 1;
  for (int j = 1; j < p; ++j) {
    real_t z = -std::cos(kPi * j / p);
    for (int it = 0; it < 200; ++it) {
      const LegendreValue lv = legendre_value(p, z);
      const real_t step = lv.dp / ((2 * z * lv.dp - p * (p + 1) * lv.p) / (1 - z * z));
      z -= step;
      if (std::fabs(step) <= 1e-32L) break;
    }
    x[j] = z;
  }
  for (int j = 0; j < n; ++j) {
    const real_t lp = legendre_value(p, x[j]).p;
    w_out[j] = (double)(2 / (p * (p + 1) * lp * lp));
  }
  return true;
}

bool analysis_operators(int polydeg, int na, std::vector<double> &vdm, std::vector<double> &wa,
                        std::vector<double> &xa) {
  const int n = polydeg + 1;
  if (n < 2 || na < 2 || na > 16) return false;
  const auto x = lobatto_nodes(n);
  const auto lam = bary(x);
  const auto xq = lobatto_nodes(na);
  const auto wq = lobatto_weights(xq);
  vdm.assign((size_t)na * n, 0.0);
  wa.resize(na);
  xa.resize(na);
  for (int i = 0; i < na; ++i) {
    const auto l = lagrange(x, lam, xq[i]);
    for (int j = 0; j < n; ++j) vdm[(size_t)i * n + j] = (double)l[j];  // row-major [analysis node][node]
    wa[i] = (double)wq[i];
    xa[i] = (double)xq[i];
  }
  return true;
}

}  // namespace trixi
