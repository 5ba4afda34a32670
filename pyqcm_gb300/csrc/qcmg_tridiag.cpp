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

// The band solvers read the matrix through low(r, c), the element (r, c)
// for r >= c within the band: the leading block of a dense column-major
// array, or packed band storage.

// True when A - sigma I is positive definite; A is the leading n x n block
// of the band matrix, L (n x (b+1), row i holds L(i, i-b..i)) is scratch.
template <class Low>
static bool band_posdef(const Low& low, int n, int b, double sigma, std::vector<double>& L) {
  const int w = b + 1;
  auto Lr = [&](int i, int k) -> double& { return L[(size_t)i * w + (k - i + b)]; };
  for (int i = 0; i < n; ++i) {
    const int k0 = std::max(0, i - b);
    for (int k = k0; k <= i; ++k) {
      double s = low(i, k) - (k == i ? sigma : 0.0);
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

// Inverse iteration with the Cholesky factor L of A - sigma I (sigma below
// the lowest eigenvalue), then the Rayleigh quotient of the iterate: the
// lowest eigenvalue when the iteration has converged.  O(n b) per step.
template <class Low>
static bool band_refine(const Low& low, int n, int b, const std::vector<double>& L, double* lam) {
  const int w = b + 1;
  auto Lr = [&](int i, int k) { return L[(size_t)i * w + (k - i + b)]; };
  auto A = [&](int r, int c) { return r >= c ? low(r, c) : low(c, r); };
  std::vector<double> x(n), y(n);
  for (int i = 0; i < n; ++i) x[i] = 1.0 + 0.25 * std::sin(0.7 * i + 0.3);
  for (int it = 0; it < 8; ++it) {
    for (int i = 0; i < n; ++i) {  // L y = x
      double v = x[i];
      for (int k = std::max(0, i - b); k < i; ++k) v -= Lr(i, k) * y[k];
      y[i] = v / Lr(i, i);
    }
    for (int i = n - 1; i >= 0; --i) {  // L^T x = y
      double v = y[i];
      for (int m = i + 1; m <= std::min(n - 1, i + b); ++m) v -= Lr(m, i) * x[m];
      x[i] = v / Lr(i, i);
    }
    double nrm = 0.0;
    for (double v : x) nrm += v * v;
    nrm = std::sqrt(nrm);
    if (!(nrm > 0.0) || !std::isfinite(nrm)) return false;
    for (double& v : x) v /= nrm;
  }
  double q = 0.0;
  for (int i = 0; i < n; ++i) {
    double ax = 0.0;
    for (int k = std::max(0, i - b); k <= std::min(n - 1, i + b); ++k) ax += A(i, k) * x[k];
    q += x[i] * ax;
  }
  *lam = q;
  return std::isfinite(q);
}

template <class Low>
static double band_lowest_impl(const Low& low, int n, int b, double near, double width) {
  if (n <= 0) return 0.0;
  b = std::max(0, std::min(b, n - 1));
  auto A = [&](int r, int c) { return r >= c ? low(r, c) : low(c, r); };
  // lambda_min <= min_i A(i,i); Gershgorin gives the lower end.
  double glo = INFINITY, hi = INFINITY, scale = 0.0;
  for (int i = 0; i < n; ++i) {
    double r = 0.0;
    for (int k = std::max(0, i - b); k <= std::min(n - 1, i + b); ++k)
      if (k != i) r += std::fabs(A(i, k));
    glo = std::min(glo, A(i, i) - r);
    hi = std::min(hi, A(i, i));
    scale = std::max(scale, std::fabs(A(i, i)) + r);
  }
  glo -= 4.0 * DBL_EPSILON * std::max(scale, 1.0);
  std::vector<double> L((size_t)n * (b + 1));
  double lo = glo;
  if (std::isfinite(near) && std::isfinite(width) && width > 0.0) {
    // start from a bracket below the hint and widen it until A - lo I is
    // definite (the Gershgorin end always is)
    const double top = near + 64.0 * DBL_EPSILON * std::max(scale, 1.0);
    if (top < hi && !band_posdef(low, n, b, top, L)) hi = top;
    for (double w = width;; w *= 8.0) {
      const double cand = hi - w;
      if (cand <= glo) break;
      if (band_posdef(low, n, b, cand, L)) {
        lo = cand;
        break;
      }
      hi = cand;
    }
  }
  // invariant: A - lo I definite, A - hi I not.  Bisect to a bracket of
  // 1e-4 of the matrix scale, then refine by inverse iteration with the
  // definite shift lo and a Rayleigh quotient; the refined value is taken
  // only if two definiteness probes confirm it to eta (else bisection runs
  // on to full precision), so it is as reliable as bisection.
  const double refine_at = 1e-4 * std::max(scale, 1.0);
  const double eta = 16.0 * DBL_EPSILON * std::max(scale, 1.0);
  bool tried = false;
  for (int it = 0; it < 2000; ++it) {
    if (!tried && hi - lo <= refine_at) {
      tried = true;
      double lam;
      if (band_posdef(low, n, b, lo, L) && band_refine(low, n, b, L, &lam) &&
          lam - eta > lo && lam + eta < hi) {
        if (band_posdef(low, n, b, lam - eta, L) && !band_posdef(low, n, b, lam + eta, L))
          return lam;
      }
    }
    const double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) break;
    if (band_posdef(low, n, b, mid, L))
      lo = mid;
    else
      hi = mid;
  }
  return 0.5 * (lo + hi);
}

double band_lowest(const std::vector<double>& t, int ld, int n, int b, double near,
                   double width) {
  auto low = [&](int r, int c) { return t[(size_t)r + (size_t)ld * c]; };
  return band_lowest_impl(low, n, b, near, width);
}

double band_lowest_packed(const std::vector<double>& ab, int n, int b, double near,
                          double width) {
  const size_t w = (size_t)b + 1;
  auto low = [&](int r, int c) { return ab[(size_t)(r - c) + w * c]; };
  return band_lowest_impl(low, n, b, near, width);
}

namespace {

// c, s with c a + s b = hypot(a, b) and -s a + c b = 0.
inline void givens(double a, double b, double* c, double* s) {
  const double h = std::hypot(a, b);
  if (h == 0.0) {
    *c = 1.0;
    *s = 0.0;
  } else {
    *c = a / h;
    *s = b / h;
  }
}

}  // namespace

bool band_eigen_leading(const std::vector<double>& t, int ld, int n, int b, int p,
                        std::vector<double>& evals, std::vector<double>& W) {
  evals.assign(std::max(n, 0), 0.0);
  W.assign((size_t)std::max(p, 0) * std::max(n, 0), 0.0);
  if (n <= 0 || p <= 0) return true;
  b = std::max(0, std::min(b, n - 1));
  // Dense symmetric copy (row-major); the band reduction only touches a
  // window of width O(b) around each rotation, so the work is O(n^2 b).
  std::vector<double> A((size_t)n * n, 0.0);
  for (int c = 0; c < n; ++c)
    for (int r = c; r <= std::min(n - 1, c + b); ++r) {
      const double v = t[(size_t)r + (size_t)ld * c];
      A[(size_t)r * n + c] = v;
      A[(size_t)c * n + r] = v;
    }
  // Z: the leading p rows of the accumulated orthogonal transform, p x n.
  std::vector<double> Z((size_t)p * n, 0.0);
  for (int k = 0; k < std::min(p, n); ++k) Z[(size_t)k * n + k] = 1.0;
  // A <- G A G^T, G the rotation [c s; -s c] on rows/columns (r, r+1);
  // Z <- Z G^T keeps A_original = Z_full A Z_full^T.
  auto rotate = [&](int r, double c, double s) {
    const int lo = std::max(0, r - b - 2), hi = std::min(n, r + b + 4);
    double* a0 = &A[(size_t)r * n];
    double* a1 = &A[(size_t)(r + 1) * n];
    for (int j = lo; j < hi; ++j) {
      const double x = a0[j], y = a1[j];
      a0[j] = c * x + s * y;
      a1[j] = -s * x + c * y;
    }
    for (int j = lo; j < hi; ++j) {
      double* row = &A[(size_t)j * n];
      const double x = row[r], y = row[r + 1];
      row[r] = c * x + s * y;
      row[r + 1] = -s * x + c * y;
    }
    for (int k = 0; k < p; ++k) {
      double* z = &Z[(size_t)k * n];
      const double x = z[r], y = z[r + 1];
      z[r] = c * x + s * y;
      z[r + 1] = -s * x + c * y;
    }
  };
  // Band to tridiagonal (Schwarz's Givens scheme): clear column k below the
  // subdiagonal from the bottom of the band up; each rotation in the plane
  // (i-1, i) leaves one element at (i+b, i-1) outside the band, which is
  // chased down the matrix b rows at a time.
  for (int k = 0; k + 2 < n; ++k) {
    for (int i = std::min(k + b, n - 1); i >= k + 2; --i) {
      if (A[(size_t)i * n + k] == 0.0) continue;
      double c, s;
      givens(A[(size_t)(i - 1) * n + k], A[(size_t)i * n + k], &c, &s);
      rotate(i - 1, c, s);
      A[(size_t)i * n + k] = A[(size_t)k * n + i] = 0.0;
      for (int j = i + b; j < n; j += b) {
        const int col = j - b - 1;
        if (A[(size_t)j * n + col] == 0.0) break;
        givens(A[(size_t)(j - 1) * n + col], A[(size_t)j * n + col], &c, &s);
        rotate(j - 1, c, s);
        A[(size_t)j * n + col] = A[(size_t)col * n + j] = 0.0;
      }
    }
  }
  std::vector<double> d(n), e(n, 0.0);
  for (int i = 0; i < n; ++i) d[i] = A[(size_t)i * n + i];
  for (int i = 0; i + 1 < n; ++i) e[i] = A[(size_t)(i + 1) * n + i];
  // Tridiagonal eigenproblem by the implicit QL method with Wilkinson-type
  // shifts (Bowdler, Martin, Reinsch and Wilkinson, 1968), each plane
  // rotation also applied to the columns of Z.
  for (int l = 0; l < n; ++l) {
    for (int iter = 0;; ++iter) {
      int m = l;
      for (; m + 1 < n; ++m) {
        const double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
        if (std::fabs(e[m]) <= DBL_EPSILON * dd) break;
      }
      if (m == l) break;
      if (iter == 100) return false;
      double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
      double r = std::hypot(g, 1.0);
      g = d[m] - d[l] + e[l] / (g + std::copysign(r, g));
      double s = 1.0, c = 1.0, shift = 0.0;
      bool split = false;
      for (int i = m - 1; i >= l; --i) {
        const double f = s * e[i], bb = c * e[i];
        r = std::hypot(f, g);
        e[i + 1] = r;
        if (r == 0.0) {  // the subdiagonal underflowed: the matrix splits here
          d[i + 1] -= shift;
          e[m] = 0.0;
          split = true;
          break;
        }
        s = f / r;
        c = g / r;
        g = d[i + 1] - shift;
        r = (d[i] - g) * s + 2.0 * c * bb;
        shift = s * r;
        d[i + 1] = g + shift;
        g = c * r - bb;
        for (int k = 0; k < p; ++k) {
          double* z = &Z[(size_t)k * n];
          const double zf = z[i + 1];
          z[i + 1] = s * z[i] + c * zf;
          z[i] = c * z[i] - s * zf;
        }
      }
      if (split) continue;
      d[l] -= shift;
      e[l] = g;
      e[m] = 0.0;
    }
  }
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return d[a] < d[c]; });
  for (int i = 0; i < n; ++i) {
    evals[i] = d[order[i]];
    for (int k = 0; k < p; ++k) W[(size_t)k * n + i] = Z[(size_t)k * n + order[i]];
  }
  return true;
}

}  // namespace qcmg
