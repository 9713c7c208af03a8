// basis.h -- host Lobatto-Legendre basis and mortar operators.
#pragma once
#include <vector>

namespace trixi {

// All matrices n x n, column-major (M[i,j] at i + n*j), the layout of the
// reference's Julia matrices.
struct Basis {
  int n = 0;
  std::vector<double> nodes, weights;
  std::vector<double> dmat, dsplit, dhat, ivdm;
  std::vector<double> fwd_up, fwd_lo, rev_up, rev_lo;
};

bool compute_basis(int polydeg, Basis &b);

// LGL quadrature weights into w_out[polydeg+1] using stack storage only.
bool lgl_weights_fixed(int polydeg, double *w_out);

// Interpolation from the polydeg LGL nodes to `na` LGL analysis nodes
// (row-major [na][polydeg+1]), with the analysis weights and nodes -- the
// SolutionAnalyzer of the reference (src/solvers/basis_lobatto_legendre.jl:120-137).
bool analysis_operators(int polydeg, int na, std::vector<double> &vdm, std::vector<double> &wa,
                        std::vector<double> &xa);

}  // namespace trixi
