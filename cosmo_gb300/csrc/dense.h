// Small dense FP64 linear algebra for the Davidson projected problem
// (at most a few dozen rows): symmetric eigensolver and Cholesky.
#pragma once
#include <vector>

namespace cg {

// Eigen-decomposition of the symmetric n x n matrix a (row-major, n*n).
// On return w holds the eigenvalues in ascending order and z (row-major, n*n)
// the eigenvectors as columns: z[i*n + k] is component i of eigenvector k.
// Householder tridiagonalisation followed by the implicit QL iteration, the
// method of tav::EigenSystemT (include/tav/EigenSystem.cxx:49-69).
void sym_eig(int n, const std::vector<double>& a, std::vector<double>& w, std::vector<double>& z);

// In-place Cholesky of the SPD n x n matrix a (row-major, lower factor in the
// lower triangle).  Returns the index of the first non-positive pivot, or -1.
int cholesky(int n, std::vector<double>& a);

}  // namespace cg
