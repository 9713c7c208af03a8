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

}  // namespace trixi
