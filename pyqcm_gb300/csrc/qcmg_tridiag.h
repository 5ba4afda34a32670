// Lowest eigenpair of a symmetric tridiagonal matrix (host, FP64).
//
// Replaces the reference's per-iteration LAPACK dstev call
// (src_ed/Hamiltonian/Lanczos.cpp:25-52), which computes the full
// eigensystem, by what the Lanczos loop uses: the lowest eigenvalue
// (Sturm-sequence bisection, O(n) per probe) and its eigenvector (inverse
// iteration on the positive-definite shifted matrix T - (lambda - delta) I
// with an LDL^T factorization, O(n) per solve).
#pragma once

#include <vector>

namespace qcmg {

// alpha[0..n-1] diagonal, beta[0..n-2] off-diagonal.  Returns lambda_min and
// fills z (normalized, z[0] >= 0 convention not imposed).
double tridiag_lowest(const std::vector<double>& alpha, const std::vector<double>& beta,
                      std::vector<double>& z);

}  // namespace qcmg
