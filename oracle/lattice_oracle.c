/* CPU oracle for the k x omega lattice integrals of CPT / VCA / CDMFT.  TEST
 * INFRASTRUCTURE ONLY: tests and the CPU-baseline legs of bench.py call it
 * as the checker; the product never links or calls it.
 *
 * Every quantity goes through the L x L complex matrix of one point (K, z)
 *   M(K, z) = Base(z) - sum_e v_e exp(2 pi i K.R_{n_e}) |r_e><c_e|,
 *   Base(z) = G(z)^-1 + Gamma(z) - (t - t_c)_0,
 * where G is the cluster Green function, Gamma the bath hybridization and
 * the sum the inter-cluster hopping in the reduced (superlattice-dual)
 * basis, as pyqcm's lattice_model_instance builds V(K) = t(K) - t_c - Gamma
 * (src_qcm/CPT.cpp:22-64).  Then, per point, after an LU factorization with
 * partial pivoting:
 *   SEF   log|det(V G - 1)| = log|det M| + log|det G|
 *         (src_qcm/lattice_model_instance.cpp:624-643), integrated as
 *         sum_w wt_w (1/N_K) sum_K over the K grid (:503-584);
 *   CPT   g(K, z) = (1/L) sum_ab (M^-1)_ab exp(2 pi i K.(x_b - x_a))
 *         (CPT.cpp:76-86, src_qcm/lattice_model.cpp:724-740);
 *   CDMFT (1/N_K) sum_K M^-1 on the midpoint grid (CPT.cpp:283-345).
 * Complex numbers are interleaved (re, im) doubles; matrices row-major.
 * Sums over K are taken row by row (fixed x index) and the rows added in
 * order, so the results do not depend on the thread count.
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;

typedef struct {
  int L, nR, nel;
  const double* R;  /* nR x 3 */
  const int *er, *ec, *en;
  const cplx* ev;
} Hops;

static void grid_K(int i, int j, int l, int gx, int gy, int gz, double off, double* K) {
  K[0] = (i + off) / gx;
  K[1] = gy > 1 ? (j + off) / gy : 0.0;
  K[2] = gz > 1 ? (l + off) / gz : 0.0;
}

/* M = B - sum_e v_e exp(2 pi i K.R_{n_e}) at (r_e, c_e); ph: nR scratch */
static void point_matrix(const Hops* h, const cplx* B, const double* K, cplx* ph, cplx* M) {
  const int L = h->L;
  memcpy(M, B, sizeof(cplx) * (size_t)L * L);
  for (int n = 0; n < h->nR; ++n) {
    const double* Rn = h->R + 3 * n;
    ph[n] = cexp(I * 2.0 * M_PI * (K[0] * Rn[0] + K[1] * Rn[1] + K[2] * Rn[2]));
  }
  for (int e = 0; e < h->nel; ++e) M[h->er[e] * L + h->ec[e]] -= h->ev[e] * ph[h->en[e]];
}

/* In-place LU with row interchanges (largest |pivot|^2, first one on ties);
 * returns log|det M|. */
static double lu(int L, cplx* M, int* perm) {
  double logabs = 0.0;
  for (int i = 0; i < L; ++i) perm[i] = i;
  for (int p = 0; p < L; ++p) {
    int best = p;
    double bv = creal(M[p * L + p]) * creal(M[p * L + p]) + cimag(M[p * L + p]) * cimag(M[p * L + p]);
    for (int r = p + 1; r < L; ++r) {
      cplx m = M[r * L + p];
      double a = creal(m) * creal(m) + cimag(m) * cimag(m);
      if (a > bv) {
        bv = a;
        best = r;
      }
    }
    if (best != p) {
      for (int c = 0; c < L; ++c) {
        cplx t = M[p * L + c];
        M[p * L + c] = M[best * L + c];
        M[best * L + c] = t;
      }
      int t = perm[p];
      perm[p] = perm[best];
      perm[best] = t;
    }
    logabs += 0.5 * log(bv);
    const cplx ip = 1.0 / M[p * L + p];
    for (int r = p + 1; r < L; ++r) {
      const cplx f = M[r * L + p] * ip;
      M[r * L + p] = f;
      for (int c = p + 1; c < L; ++c) M[r * L + c] -= f * M[p * L + c];
    }
  }
  return logabs;
}

/* y = M^-1 b from the LU (b in original row order) */
static void lu_solve(int L, const cplx* M, const int* perm, const cplx* b, cplx* y) {
  for (int i = 0; i < L; ++i) y[i] = b[perm[i]];
  for (int i = 0; i < L; ++i)
    for (int j = 0; j < i; ++j) y[i] -= M[i * L + j] * y[j];
  for (int i = L - 1; i >= 0; --i) {
    for (int j = i + 1; j < L; ++j) y[i] -= M[i * L + j] * y[j];
    y[i] /= M[i * L + i];
  }
}

static Hops hops(int L, int nR, const double* R, int nel, const int* er, const int* ec,
                 const int* en, const double* ev) {
  Hops h = {L, nR, nel, R, er, ec, en, (const cplx*)ev};
  return h;
}

/* sum_w wt_w (1/N_K) sum_K (log|det M(K, i w)| + ldg_w) on the gx x gy x gz
 * grid K = (i/gx, j/gy, l/gz).  base: nw x L x L; ldg: log|det G| per w. */
double lo_sef_grid(int L, int nw, const double* base, const double* ldg, const double* wt, int nR,
                   const double* R, int nel, const int* er, const int* ec, const int* en,
                   const double* ev, int gx, int gy, int gz, int nthreads) {
  Hops h = hops(L, nR, R, nel, er, ec, en, ev);
  const int rows = gy * gz;
  double* rs = (double*)malloc(sizeof(double) * (size_t)rows);
  double total = 0.0;
  if (nthreads < 1) nthreads = 1;
  for (int w = 0; w < nw; ++w) {
    const cplx* B = (const cplx*)base + (size_t)w * L * L;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads)
#endif
    {
      cplx* M = (cplx*)malloc(sizeof(cplx) * (size_t)L * L);
      cplx* ph = (cplx*)malloc(sizeof(cplx) * (size_t)(nR ? nR : 1));
      int* perm = (int*)malloc(sizeof(int) * (size_t)L);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
      for (int row = 0; row < rows; ++row) {
        const int j = row % gy, l = row / gy;
        double s = 0.0;
        for (int i = 0; i < gx; ++i) {
          double K[3];
          grid_K(i, j, l, gx, gy, gz, 0.0, K);
          point_matrix(&h, B, K, ph, M);
          s += lu(L, M, perm) + ldg[w];
        }
        rs[row] = s;
      }
      free(M);
      free(ph);
      free(perm);
    }
    double sk = 0.0;
    for (int row = 0; row < rows; ++row) sk += rs[row];
    total += wt[w] * (sk / ((double)gx * rows));
  }
  free(rs);
  return total;
}

/* g(K, z) for nz frequencies x nk explicit K (nk x 3, reduced basis);
 * gpos: L x 3 orbital positions; g: nz x nk complex. */
void lo_cpt(int L, int nz, const double* base, int nR, const double* R, int nel, const int* er,
            const int* ec, const int* en, const double* ev, int nk, const double* Kl,
            const double* gpos, double* g, int nthreads) {
  Hops h = hops(L, nR, R, nel, er, ec, en, ev);
  if (nthreads < 1) nthreads = 1;
  const long npts = (long)nz * nk;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads)
#endif
  {
    cplx* M = (cplx*)malloc(sizeof(cplx) * (size_t)L * L);
    cplx* ph = (cplx*)malloc(sizeof(cplx) * (size_t)(nR ? nR : 1));
    cplx* u = (cplx*)malloc(sizeof(cplx) * (size_t)L);
    cplx* y = (cplx*)malloc(sizeof(cplx) * (size_t)L);
    int* perm = (int*)malloc(sizeof(int) * (size_t)L);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
    for (long pt = 0; pt < npts; ++pt) {
      const int w = (int)(pt / nk), ik = (int)(pt % nk);
      const double* K = Kl + 3 * ik;
      point_matrix(&h, (const cplx*)base + (size_t)w * L * L, K, ph, M);
      lu(L, M, perm);
      for (int b = 0; b < L; ++b) {
        const double* x = gpos + 3 * b;
        u[b] = cexp(I * 2.0 * M_PI * (K[0] * x[0] + K[1] * x[1] + K[2] * x[2]));
      }
      lu_solve(L, M, perm, u, y);
      cplx s = 0.0;
      for (int a = 0; a < L; ++a) s += conj(u[a]) * y[a];
      s /= L;
      g[2 * pt] = creal(s);
      g[2 * pt + 1] = cimag(s);
    }
    free(M);
    free(ph);
    free(u);
    free(y);
    free(perm);
  }
}

/* (1/N_K) sum_K M(K, z_w)^-1 on the grid K = ((i+off)/gx, ...), per
 * frequency; out: nw x L x L complex. */
void lo_kmean(int L, int nw, const double* base, int nR, const double* R, int nel, const int* er,
              const int* ec, const int* en, const double* ev, int gx, int gy, int gz, double off,
              double* out, int nthreads) {
  Hops h = hops(L, nR, R, nel, er, ec, en, ev);
  const int rows = gy * gz, LL = L * L;
  cplx* rs = (cplx*)malloc(sizeof(cplx) * (size_t)rows * LL);
  if (nthreads < 1) nthreads = 1;
  for (int w = 0; w < nw; ++w) {
    const cplx* B = (const cplx*)base + (size_t)w * LL;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads)
#endif
    {
      cplx* M = (cplx*)malloc(sizeof(cplx) * (size_t)LL);
      cplx* ph = (cplx*)malloc(sizeof(cplx) * (size_t)(nR ? nR : 1));
      cplx* e = (cplx*)malloc(sizeof(cplx) * (size_t)L);
      cplx* y = (cplx*)malloc(sizeof(cplx) * (size_t)L);
      int* perm = (int*)malloc(sizeof(int) * (size_t)L);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
      for (int row = 0; row < rows; ++row) {
        const int j = row % gy, l = row / gy;
        cplx* acc = rs + (size_t)row * LL;
        for (int q = 0; q < LL; ++q) acc[q] = 0.0;
        for (int i = 0; i < gx; ++i) {
          double K[3];
          grid_K(i, j, l, gx, gy, gz, off, K);
          point_matrix(&h, B, K, ph, M);
          lu(L, M, perm);
          for (int c = 0; c < L; ++c) {
            for (int r = 0; r < L; ++r) e[r] = r == c ? 1.0 : 0.0;
            lu_solve(L, M, perm, e, y);
            for (int r = 0; r < L; ++r) acc[r * L + c] += y[r];
          }
        }
      }
      free(M);
      free(ph);
      free(e);
      free(y);
      free(perm);
    }
    cplx* o = (cplx*)out + (size_t)w * LL;
    for (int q = 0; q < LL; ++q) o[q] = 0.0;
    for (int row = 0; row < rows; ++row)
      for (int q = 0; q < LL; ++q) o[q] += rs[(size_t)row * LL + q];
    for (int q = 0; q < LL; ++q) o[q] /= (double)gx * rows;
  }
  free(rs);
}
