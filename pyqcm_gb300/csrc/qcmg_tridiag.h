// Lowest eigenpair of a symmetric tridiagonal matrix (host, FP64).
//
// Replaces the reference's per-iteration LAPACK dstev call
// (src_ed/Hamiltonian/Lanczos.cpp:25-52), which computes the full
// eigensystem, by what the Lanczos loop uses: the lowest eigenvalue
// (Sturm-sequence bisection, O(n) per probe) and its eigenvector (inverse
// iteration on the positive-definite shifted matrix T - (lambda - delta) I
// with an LDL^T factorization, O(n) per solve).
#pragma once

#include <cmath>
#include <vector>

namespace qcmg {

// alpha[0..n-1] diagonal, beta[0..n-2] off-diagonal.  Returns lambda_min and
// fills z (normalized, z[0] >= 0 convention not imposed).
double tridiag_lowest(const std::vector<double>& alpha, const std::vector<double>& beta,
                      std::vector<double>& z);

// Lowest eigenvalue of the leading n x n block of a symmetric band matrix
// (half bandwidth b: t(r, c) = 0 for |r - c| > b), read from the lower
// triangle of column-major t with leading dimension ld.  Bisection on
// positive definiteness of t - sigma I, tested by a banded Cholesky
// factorization (O(n b^2) per probe, no pivoting needed for a definiteness
// test), so the result is accurate to the factorization's backward error,
// a few units of eps * ||t||.  This is the convergence probe of band Lanczos
// (src_ed/Hamiltonian/Lanczos.hpp:338-362 compares the lowest eigenvalue of
// the projected matrix every p steps); a dense eigensolver per probe costs
// O(n^3) for the one number it needs.  A hint (near, width > 0: the
// lowest eigenvalue is expected just below near, within about width; the
// previous probe's value and change) narrows the starting bracket, which
// then widens geometrically until it holds the eigenvalue, so a wrong hint
// costs probes, not accuracy.
double band_lowest(const std::vector<double>& t, int ld, int n, int b, double near = NAN,
                   double width = 0.0);

// band_lowest on packed band storage: element (r, c), r >= c, r - c <= b, at
// ab[(r - c) + (b + 1) c] (the lower band of LAPACK's band layout), for
// matrices too large to hold densely.
double band_lowest_packed(const std::vector<double>& ab, int n, int b, double near = NAN,
                          double width = 0.0);

// All eigenvalues (ascending) of the same band matrix, and the leading p
// rows of its eigenvectors: W[k * n + c] is component k of eigenvector c.
// Band Lanczos needs no more to form its Q-matrix (Q = P U(0:p, :),
// src_ed/Hamiltonian/Hamiltonian_base.hpp:249), so the full eigenvector
// matrix is never built: a Givens reduction to tridiagonal form (O(n^2 b))
// and implicit QL iterations, with every rotation applied to p rows only.
// False if the QL iteration does not converge.
bool band_eigen_leading(const std::vector<double>& t, int ld, int n, int b, int p,
                        std::vector<double>& evals, std::vector<double>& W);

}  // namespace qcmg
