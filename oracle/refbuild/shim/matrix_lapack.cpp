// LAPACK-backed definitions of the dense matrix routines that the reference
// declares in src_util/matrix.hpp:740-773 and implements with Eigen in
// src_util/matrix.cpp.  Eigen is not installed here, so the oracle build links
// these instead; the LAPACK comes from SciPy's bundled OpenBLAS (LP64, symbols
// prefixed "scipy_").  Rounding differs from Eigen at the 1e-15 level only.
#include <cmath>
#include <complex>
#include <stdexcept>
#include <vector>

#include "matrix.hpp"

using std::vector;
typedef std::complex<double> cplx;

extern "C" {
void scipy_dgetrf_(int*, int*, double*, int*, int*, int*);
void scipy_dgetri_(int*, double*, int*, int*, double*, int*, int*);
void scipy_zgetrf_(int*, int*, cplx*, int*, int*, int*);
void scipy_zgetri_(int*, cplx*, int*, int*, cplx*, int*, int*);
void scipy_dsyev_(char*, char*, int*, double*, int*, double*, double*, int*, int*);
void scipy_zheev_(char*, char*, int*, cplx*, int*, double*, cplx*, int*, double*, int*);
void scipy_dpotrf_(char*, int*, double*, int*, int*);
void scipy_dtrtri_(char*, char*, int*, double*, int*, int*);
}

static void lapack_check(int info, const char* what) {
  if (info != 0)
    throw std::runtime_error(std::string("oracle LAPACK failure in ") + what +
                             " info=" + std::to_string(info));
}

template <> void matrix<double>::inverse() {
  if (r != c) throw std::runtime_error("inverse of a non-square matrix");
  if (r == 0) return;
  int n = (int)r, info = 0, lwork = 64 * n;
  vector<int> piv(n);
  vector<double> work(lwork);
  scipy_dgetrf_(&n, &n, v.data(), &n, piv.data(), &info);
  lapack_check(info, "dgetrf");
  scipy_dgetri_(&n, v.data(), &n, piv.data(), work.data(), &lwork, &info);
  lapack_check(info, "dgetri");
}

template <> void matrix<Complex>::inverse() {
  if (r != c) throw std::runtime_error("inverse of a non-square matrix");
  if (r == 0) return;
  int n = (int)r, info = 0, lwork = 64 * n;
  vector<int> piv(n);
  vector<cplx> work(lwork);
  scipy_zgetrf_(&n, &n, v.data(), &n, piv.data(), &info);
  lapack_check(info, "zgetrf");
  scipy_zgetri_(&n, v.data(), &n, piv.data(), work.data(), &lwork, &info);
  lapack_check(info, "zgetri");
}

template <> Complex matrix<Complex>::determinant() {
  if (r == 0) return Complex(0);
  int n = (int)r, info = 0;
  vector<cplx> a(v);
  vector<int> piv(n);
  scipy_zgetrf_(&n, &n, a.data(), &n, piv.data(), &info);
  if (info > 0) return Complex(0);  // exactly singular
  lapack_check(info, "zgetrf");
  cplx det(1.0, 0.0);
  for (int i = 0; i < n; i++) {
    det *= a[i + (size_t)n * i];
    if (piv[i] != i + 1) det = -det;
  }
  return det;
}

template <> bool matrix<Complex>::is_real(double accuracy) {
  for (auto& x : v)
    if (std::fabs(x.imag()) > accuracy) return false;
  return true;
}

template <> void matrix<double>::eigensystem(vector<double>& d, matrix<double>& U) const {
  int n = (int)r, info = 0, lwork = -1;
  U.v = v;
  d.resize(n);
  if (n == 0) return;
  char jobz = 'V', uplo = 'L';
  double wq;
  scipy_dsyev_(&jobz, &uplo, &n, U.v.data(), &n, d.data(), &wq, &lwork, &info);
  lwork = (int)wq;
  vector<double> work(lwork);
  scipy_dsyev_(&jobz, &uplo, &n, U.v.data(), &n, d.data(), work.data(), &lwork, &info);
  lapack_check(info, "dsyev");
}

template <> void matrix<double>::eigenvalues(vector<double>& d) {
  int n = (int)r, info = 0, lwork = -1;
  vector<double> a(v);
  d.resize(n);
  if (n == 0) return;
  char jobz = 'N', uplo = 'L';
  double wq;
  scipy_dsyev_(&jobz, &uplo, &n, a.data(), &n, d.data(), &wq, &lwork, &info);
  lwork = (int)wq;
  vector<double> work(lwork);
  scipy_dsyev_(&jobz, &uplo, &n, a.data(), &n, d.data(), work.data(), &lwork, &info);
  lapack_check(info, "dsyev");
}

template <> void matrix<Complex>::eigensystem(vector<double>& d, matrix<Complex>& U) const {
  int n = (int)r, info = 0, lwork = -1;
  U.v = v;
  d.resize(n);
  if (n == 0) return;
  char jobz = 'V', uplo = 'L';
  cplx wq;
  vector<double> rwork(3 * n);
  scipy_zheev_(&jobz, &uplo, &n, U.v.data(), &n, d.data(), &wq, &lwork, rwork.data(), &info);
  lwork = (int)wq.real();
  vector<cplx> work(lwork);
  scipy_zheev_(&jobz, &uplo, &n, U.v.data(), &n, d.data(), work.data(), &lwork, rwork.data(), &info);
  lapack_check(info, "zheev");
}

template <> void matrix<Complex>::eigenvalues(vector<double>& d) {
  int n = (int)r, info = 0, lwork = -1;
  vector<cplx> a(v);
  d.resize(n);
  if (n == 0) return;
  char jobz = 'N', uplo = 'L';
  cplx wq;
  vector<double> rwork(3 * n);
  scipy_zheev_(&jobz, &uplo, &n, a.data(), &n, d.data(), &wq, &lwork, rwork.data(), &info);
  lwork = (int)wq.real();
  vector<cplx> work(lwork);
  scipy_zheev_(&jobz, &uplo, &n, a.data(), &n, d.data(), work.data(), &lwork, rwork.data(), &info);
  lapack_check(info, "zheev");
}

template <> double matrix<double>::norm2() {
  double s = 0.0;
  for (auto x : v) s += x * x;
  return s;
}
template <> double matrix<Complex>::norm2() {
  double s = 0.0;
  for (auto x : v) s += std::norm(x);
  return s;
}
template <> double matrix<double>::norm() { return std::sqrt(norm2()); }
template <> double matrix<Complex>::norm() { return std::sqrt(norm2()); }

template <> bool matrix<double>::is_orthogonal(double accuracy) {
  if (r != c) return false;
  for (size_t i = 0; i < r; i++)
    for (size_t j = 0; j < r; j++) {
      double s = 0.0;
      for (size_t k = 0; k < r; k++) s += v[k + r * i] * v[k + r * j];
      if (std::fabs(s - (i == j ? 1.0 : 0.0)) > accuracy) return false;
    }
  return true;
}

template <> bool matrix<double>::cholesky(matrix<double>& A) {
  int n = (int)A.r, info = 0;
  set_size(A.r);
  v = A.v;
  char uplo = 'L';
  if (n == 0) return true;
  scipy_dpotrf_(&uplo, &n, v.data(), &n, &info);
  if (info != 0) return false;
  for (int j = 0; j < n; j++)
    for (int i = 0; i < j; i++) v[i + (size_t)n * j] = 0.0;  // keep L only
  return true;
}

template <> bool matrix<double>::triangular_inverse() {
  int n = (int)r, info = 0;
  char uplo = 'L', diag = 'N';
  if (n == 0) return true;
  scipy_dtrtri_(&uplo, &diag, &n, v.data(), &n, &info);
  for (int j = 0; j < n; j++)
    for (int i = 0; i < j; i++) v[i + (size_t)n * j] = 0.0;
  return info == 0;
}

matrix<Complex> to_complex_matrix(const matrix<double>& x) {
  matrix<Complex> out(x.r, x.c);
  for (size_t i = 0; i < x.v.size(); i++) out.v[i] = Complex(x.v[i], 0.0);
  return out;
}

// Packing used by the reference's hybridization-fit helpers: per row i, the
// diagonal (real) followed by (re, im) of each element left of the diagonal.
matrix<Complex> hermitian_matrix_from_real_vector(size_t d, const vector<double>& x) {
  matrix<Complex> M(d);
  size_t pos = 0;
  for (size_t i = 0; i < d; i++) {
    M(i, i) = Complex(x[pos], 0.0);
    pos++;
    for (size_t j = 0; j < i; j++, pos += 2) {
      M(i, j) = Complex(x[pos], x[pos + 1]);
      M(j, i) = std::conj(M(i, j));
    }
  }
  return M;
}

void hermitian_matrix_to_real_vector(const matrix<Complex>& M, double* x) {
  size_t pos = 0;
  for (size_t i = 0; i < M.r; i++) {
    x[pos++] = M(i, i).real();
    for (size_t j = 0; j < i; j++) {
      x[pos++] = M(i, j).real();
      x[pos++] = M(i, j).imag();
    }
  }
}
