#include "qcmg_tridiag.h"

#include <algorithm>
#include <cfloat>
#include <cmath>

namespace qcmg {

// Number of eigenvalues of T strictly below x (Sylvester inertia of the
// LDL^T pivots of T - x I).
static int sturm_below(const std::vector<double>& a, const std::vector<double>& b, double x) {
  const size_t n = a.size();
  int count = 0;
  double d = 1.0;
  for (size_t i = 0; i < n; ++i) {
    double off = (i > 0) ? b[i - 1] * b[i - 1] / d : 0.0;
    d = a[i] - x - off;
    if (d == 0.0) d = -DBL_MIN * 1e10;  // perturb an exact zero pivot
    if (d < 0.0) ++count;
  }
  return count;
}

double tridiag_lowest(const std::vector<double>& a, const std::vector<double>& b,
                      std::vector<double>& z) {
  const size_t n = a.size();
  z.assign(n, 0.0);
  if (n == 0) return 0.0;
  if (n == 1) {
    z[0] = 1.0;
    return a[0];
  }
  // Gershgorin interval.
  double lo = INFINITY, hi = -INFINITY, scale = 0.0;
  for (size_t i = 0; i < n; ++i) {
    double r = (i > 0 ? std::fabs(b[i - 1]) : 0.0) + (i + 1 < n ? std::fabs(b[i]) : 0.0);
    lo = std::min(lo, a[i] - r);
    hi = std::max(hi, a[i] + r);
    scale = std::max(scale, std::fabs(a[i]) + r);
  }
  // Bisection to full precision: invariant count(lo) == 0, count(hi) >= 1.
  for (int it = 0; it < 2000; ++it) {
    double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) break;
    if (sturm_below(a, b, mid) >= 1)
      hi = mid;
    else
      lo = mid;
  }
  const double lam = 0.5 * (lo + hi);
  // Inverse iteration on T - (lam - delta) I, positive definite.
  const double delta = std::max(scale, 1.0) * 64.0 * DBL_EPSILON;
  const double shift = lo - delta;
  std::vector<double> d(n), l(n > 1 ? n - 1 : 1);
  d[0] = a[0] - shift;
  for (size_t i = 0; i + 1 < n; ++i) {
    l[i] = b[i] / d[i];
    d[i + 1] = a[i + 1] - shift - l[i] * b[i];
    if (!(d[i + 1] > 0.0)) d[i + 1] = DBL_MIN * 1e10;
  }
  for (size_t i = 0; i < n; ++i) z[i] = 1.0 / std::sqrt((double)n) * ((i % 2) ? 0.9 : 1.1);
  for (int it = 0; it < 4; ++it) {
    // Solve L D L^T w = z in place.
    for (size_t i = 1; i < n; ++i) z[i] -= l[i - 1] * z[i - 1];
    for (size_t i = 0; i < n; ++i) z[i] /= d[i];
    for (size_t i = n - 1; i-- > 0;) z[i] -= l[i] * z[i + 1];
    double nrm = 0.0;
    for (double v : z) nrm += v * v;
    nrm = std::sqrt(nrm);
    for (double& v : z) v /= nrm;
  }
  // Sign convention of LAPACK's QL-based solvers is arbitrary; make the
  // largest component positive so results are reproducible.
  size_t imax = 0;
  for (size_t i = 1; i < n; ++i)
    if (std::fabs(z[i]) > std::fabs(z[imax])) imax = i;
  if (z[imax] < 0)
    for (double& v : z) v = -v;
  return lam;
}

// True when A - sigma I is positive definite; A is the leading n x n block
// of the band matrix, L (n x (b+1), row i holds L(i, i-b..i)) is scratch.
static bool band_posdef(const std::vector<double>& t, int ld, int n, int b, double sigma,
                        std::vector<double>& L) {
  const int w = b + 1;
  auto Lr = [&](int i, int k) -> double& { return L[(size_t)i * w + (k - i + b)]; };
  for (int i = 0; i < n; ++i) {
    const int k0 = std::max(0, i - b);
    for (int k = k0; k <= i; ++k) {
      double s = t[(size_t)i + (size_t)ld * k] - (k == i ? sigma : 0.0);
      for (int m = std::max(k0, k - b); m < k; ++m) s -= Lr(i, m) * Lr(k, m);
      if (k < i) {
        Lr(i, k) = s / Lr(k, k);
      } else {
        if (!(s > 0.0)) return false;
        Lr(i, i) = std::sqrt(s);
      }
    }
  }
  return true;
}

double band_lowest(const std::vector<double>& t, int ld, int n, int b) {
  if (n <= 0) return 0.0;
  b = std::max(0, std::min(b, n - 1));
  auto A = [&](int r, int c) { return r >= c ? t[(size_t)r + (size_t)ld * c] : t[(size_t)c + (size_t)ld * r]; };
  // lambda_min <= min_i A(i,i); Gershgorin gives the lower end.
  double lo = INFINITY, hi = INFINITY, scale = 0.0;
  for (int i = 0; i < n; ++i) {
    double r = 0.0;
    for (int k = std::max(0, i - b); k <= std::min(n - 1, i + b); ++k)
      if (k != i) r += std::fabs(A(i, k));
    lo = std::min(lo, A(i, i) - r);
    hi = std::min(hi, A(i, i));
    scale = std::max(scale, std::fabs(A(i, i)) + r);
  }
  lo -= 4.0 * DBL_EPSILON * std::max(scale, 1.0);
  std::vector<double> L((size_t)n * (b + 1));
  // invariant: A - lo I definite, A - hi I not
  for (int it = 0; it < 2000; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) break;
    if (band_posdef(t, ld, n, b, mid, L))
      lo = mid;
    else
      hi = mid;
  }
  return 0.5 * (lo + hi);
}

}  // namespace qcmg
