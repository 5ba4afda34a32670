/* Unprefixed CBLAS / LAPACK entry points that the reference's sources call
 * (src_util/vector_num.cpp:37-106, src_ed/Hamiltonian/Lanczos.cpp:46),
 * forwarded to SciPy's bundled OpenBLAS, which exports them with a "scipy_"
 * prefix and 32-bit integers.  The reference's f2c headers declare LAPACK
 * integers as `long`, so dstev_ narrows them here. */
#include <stddef.h>

void scipy_cblas_daxpy(int, double, const double*, int, double*, int);
double scipy_cblas_ddot(int, const double*, int, const double*, int);
double scipy_cblas_dnrm2(int, const double*, int);
void scipy_cblas_dscal(int, double, double*, int);
void scipy_cblas_zaxpy(int, const void*, const void*, int, void*, int);
void scipy_cblas_zdotc_sub(int, const void*, int, const void*, int, void*);
double scipy_cblas_dznrm2(int, const void*, int);
void scipy_cblas_zscal(int, const void*, void*, int);
void scipy_dstev_(char*, int*, double*, double*, double*, int*, double*, int*);

void cblas_daxpy(const int n, const double a, const double* x, const int ix, double* y,
                 const int iy) {
  scipy_cblas_daxpy(n, a, x, ix, y, iy);
}
double cblas_ddot(const int n, const double* x, const int ix, const double* y, const int iy) {
  return scipy_cblas_ddot(n, x, ix, y, iy);
}
double cblas_dnrm2(const int n, const double* x, const int ix) {
  return scipy_cblas_dnrm2(n, x, ix);
}
void cblas_dscal(const int n, const double a, double* x, const int ix) {
  scipy_cblas_dscal(n, a, x, ix);
}
void cblas_zaxpy(const int n, const void* a, const void* x, const int ix, void* y, const int iy) {
  scipy_cblas_zaxpy(n, a, x, ix, y, iy);
}
void cblas_zdotc_sub(const int n, const void* x, const int ix, const void* y, const int iy,
                     void* out) {
  scipy_cblas_zdotc_sub(n, x, ix, y, iy, out);
}
double cblas_dznrm2(const int n, const void* x, const int ix) {
  return scipy_cblas_dznrm2(n, x, ix);
}
void cblas_zscal(const int n, const void* a, void* x, const int ix) {
  scipy_cblas_zscal(n, a, x, ix);
}

int dstev_(char* jobz, long* n, double* d, double* e, double* z, long* ldz, double* work,
           long* info) {
  int n32 = (int)*n, ldz32 = (int)*ldz, info32 = 0;
  scipy_dstev_(jobz, &n32, d, e, z, &ldz32, work, &info32);
  *info = info32;
  return 0;
}
