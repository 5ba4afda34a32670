/* CPU oracle for the factorized exact-diagonalization path.  TEST
 * INFRASTRUCTURE ONLY: tests, the smoke check and the CPU-baseline leg of
 * bench.py call it as the checker; the product never links or calls it.
 *
 * It restates, in plain C, the integer and FP64 arithmetic of pyqcm's
 * factorized Hamiltonian format:
 *   - half basis: increasing L-bit integers with popcount N
 *       (src_ed/ED_basis.cpp:115-125), rank by binary search (:130-135);
 *   - factorized index I = i_up + dim_up * i_dn (src_ed/ED_basis.cpp:142-165);
 *   - hop r <- c with fermion sign = parity of the occupied orbitals strictly
 *       between (src_ed/binary_state.hpp:42-49, binary_state.cpp:23-28), one
 *       half-operator per spin (src_ed/Operators/HS_half_operator.hpp:21-45);
 *   - y += H x with H = T_dn (x) 1 + 1 (x) T_up + diag
 *       (src_ed/Operators/HS_factorized_operator.hpp:57-84,
 *        src_ed/Operators/HS_interaction_operator.hpp:32-70);
 *   - c / c^dagger on a factorized state with the parity sign, down orbitals
 *       also counting every up electron (src_ed/ED_basis.cpp:79-110,
 *       src_ed/model.cpp:155-180).
 * Parity is pinned by golden vectors produced by the reference's own code
 * (tests/golden).  The half-operator here stores both triangles of the
 * symmetric hopping matrix as CSR rows, which is the same operator the
 * reference stores as a lower triangle applied in both directions.
 */
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int popc32(uint32_t x) {
  int n = 0;
  while (x) {
    x &= x - 1;
    n++;
  }
  return n;
}

/* Increasing list of L-bit integers with popcount N; returns the count. */
size_t qo_halfbasis(int L, int N, uint32_t* out) {
  size_t n = 0;
  uint32_t top = (L >= 32) ? 0xffffffffu : ((1u << L) - 1u);
  for (uint64_t b = 0; b <= top; ++b)
    if (popc32((uint32_t)b) == N) {
      if (out) out[n] = (uint32_t)b;
      n++;
    }
  return n;
}

/* Rank by binary search in the sorted list; returns dim when absent. */
uint32_t qo_rank(const uint32_t* bin, uint32_t dim, uint32_t b) {
  uint32_t lo = 0, hi = dim;
  while (lo < hi) {
    uint32_t mid = lo + (hi - lo) / 2;
    if (bin[mid] < b)
      lo = mid + 1;
    else
      hi = mid;
  }
  return (lo < dim && bin[lo] == b) ? lo : dim;
}

/* Sign of moving the electron at bit c to bit r in state b (r != c). */
static int hop_sign(uint32_t b, int r, int c) {
  int lo = r < c ? r : c, hi = r < c ? c : r;
  uint32_t between = ((hi >= 32 ? 0u : (1u << hi)) - 1u) & ~((2u << lo) - 1u);
  return (popc32(b & between) & 1) ? -1 : 1;
}

/* Half-operator of one spin, as CSR rows indexed by the input state I:
 * entries (J, s*v) for every allowed hop I -> J produced by an element
 * (r, c, v) meaning v c^dagger_r c_c, and diag[I] += v for r == c with bit r
 * set.  Elements must be given for both (r,c) and (c,r), as the reference's
 * one_body_operator stores them (src_ed/Operators/one_body_operator.hpp:62-71).
 * Passing rowptr == NULL counts the entries only.  Returns nnz. */
size_t qo_halfop_build(int L, int N, int nel, const int* er, const int* ec, const double* ev,
                       uint32_t* rowptr, uint32_t* col, double* val, double* diag) {
  size_t dim = qo_halfbasis(L, N, NULL);
  uint32_t* bin = (uint32_t*)malloc(sizeof(uint32_t) * (dim ? dim : 1));
  qo_halfbasis(L, N, bin);
  size_t nnz = 0;
  for (size_t I = 0; I < dim; ++I) {
    uint32_t b = bin[I];
    if (rowptr) rowptr[I] = (uint32_t)nnz;
    if (diag) diag[I] = 0.0;
    for (int k = 0; k < nel; ++k) {
      int r = er[k], c = ec[k];
      if (r == c) {
        if (diag && ((b >> r) & 1u)) diag[I] += ev[k];
        continue;
      }
      if (!((b >> c) & 1u) || ((b >> r) & 1u)) continue;
      if (ev[k] == 0.0) continue;
      uint32_t bp = b ^ (1u << c) ^ (1u << r);
      uint32_t J = qo_rank(bin, (uint32_t)dim, bp);
      if (rowptr) {
        col[nnz] = J;
        val[nnz] = hop_sign(b, r, c) * ev[k];
      }
      nnz++;
    }
  }
  if (rowptr) rowptr[dim] = (uint32_t)nnz;
  free(bin);
  return nnz;
}

/* Density-density diagonal: sum over pairs (r, c, v) of v * n_r * n_c, with
 * spin-orbital r < L an up orbital (bit r of the up state) and r >= L a down
 * orbital (bit r-L of the down state).  Split as e_up(up) + e_dn(dn) +
 * cross(up, dn): pairs_side sums the pairs whose two orbitals are both of
 * one spin (side 0 up, 1 down); cross_tables fills, for one down state, byte
 * tables tab[g][byte] = sum of the cross pairs' v over the up orbitals set
 * in byte g of an up state, so cross(up, dn) is ceil(L/8) lookups. */
static double pairs_side(uint32_t b, int side, int L, int np, const int* pr, const int* pc,
                         const double* pv) {
  double e = 0.0;
  for (int k = 0; k < np; ++k) {
    int r = pr[k], c = pc[k];
    if ((r >= L) != side || (c >= L) != side) continue;
    if (side) r -= L, c -= L;
    if (((b >> r) & 1u) && ((b >> c) & 1u)) e += pv[k];
  }
  return e;
}

static void cross_tables(uint32_t dn, int L, int np, const int* pr, const int* pc,
                         const double* pv, double tab[4][256]) {
  double w[32] = {0.0};
  for (int k = 0; k < np; ++k) {
    int r = pr[k], c = pc[k];
    if (r < L && c >= L && ((dn >> (c - L)) & 1u)) w[r] += pv[k];
    if (c < L && r >= L && ((dn >> (r - L)) & 1u)) w[c] += pv[k];
  }
  for (int g = 0; g * 8 < L; ++g)
    for (int byte = 0; byte < 256; ++byte) {
      double e = 0.0;
      for (int j = 0; j < 8 && g * 8 + j < L; ++j)
        if ((byte >> j) & 1) e += w[g * 8 + j];
      tab[g][byte] = e;
    }
}

/* y += H x for the factorized sector (dim_up x dim_dn), x and y stored with
 * the up index fastest.  Pulls every output slab (fixed down index) from its
 * down-spin neighbours (slab axpys), then adds the in-slab up-spin gathers and
 * the diagonal -- the arithmetic of HS_factorized_operator::multiply_add in
 * per-output order.  nthreads > 1 splits the slabs over OpenMP threads. */
void qo_matvec(int L, uint32_t du, uint32_t dd, const uint32_t* bin_up, const uint32_t* bin_dn,
               const uint32_t* rp_up, const uint32_t* col_up, const double* val_up,
               const double* diag_up, const uint32_t* rp_dn, const uint32_t* col_dn,
               const double* val_dn, const double* diag_dn, int np, const int* pr, const int* pc,
               const double* pv, const double* x, double* y, int nthreads) {
  /* up-state diagonal: one-body part plus the up-up pairs */
  double* dup = (double*)malloc(sizeof(double) * (du ? du : 1));
  for (uint32_t i = 0; i < du; ++i) dup[i] = diag_up[i] + pairs_side(bin_up[i], 0, L, np, pr, pc, pv);
  const int ng = (L + 7) / 8;
#ifdef _OPENMP
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
#endif
  for (long a = 0; a < (long)dd; ++a) {
    double tab[4][256];
    double* ya = y + (size_t)a * du;
    const double* xa = x + (size_t)a * du;
    for (uint32_t k = rp_dn[a]; k < rp_dn[a + 1]; ++k) {
      const double t = val_dn[k];
      const double* xb = x + (size_t)col_dn[k] * du;
      for (uint32_t i = 0; i < du; ++i) ya[i] += t * xb[i];
    }
    const double dda = diag_dn[a] + pairs_side(bin_dn[a], 1, L, np, pr, pc, pv);
    cross_tables(bin_dn[a], L, np, pr, pc, pv, tab);
    for (uint32_t i = 0; i < du; ++i) {
      double acc = 0.0;
      for (uint32_t k = rp_up[i]; k < rp_up[i + 1]; ++k) acc += val_up[k] * xa[col_up[k]];
      const uint32_t u = bin_up[i];
      double cross = 0.0;
      for (int g = 0; g < ng; ++g) cross += tab[g][(u >> (8 * g)) & 0xffu];
      double d = dup[i] + dda + cross;
      ya[i] += acc + d * xa[i];
    }
  }
  free(dup);
}

/* Apply c_a (pm = -1) or c^dagger_a (pm = +1) to x in sector (nup, ndn),
 * adding z * result into y of the target sector.  Orbital a < L is an up
 * orbital, a >= L a down orbital; the sign is the parity of the occupied
 * orbitals below a, counting all up electrons first for a down orbital. */
void qo_apply_c(int L, int a, int pm, int nup, int ndn, const double* x, double* y, double z) {
  int spin = a >= L;
  int orb = spin ? a - L : a;
  int nup2 = nup + (spin ? 0 : pm), ndn2 = ndn + (spin ? pm : 0);
  size_t du = qo_halfbasis(L, nup, NULL), dd = qo_halfbasis(L, ndn, NULL);
  size_t du2 = qo_halfbasis(L, nup2, NULL), dd2 = qo_halfbasis(L, ndn2, NULL);
  uint32_t* bu = (uint32_t*)malloc(4 * (du + 1));
  uint32_t* bd = (uint32_t*)malloc(4 * (dd + 1));
  uint32_t* bu2 = (uint32_t*)malloc(4 * (du2 + 1));
  uint32_t* bd2 = (uint32_t*)malloc(4 * (dd2 + 1));
  qo_halfbasis(L, nup, bu);
  qo_halfbasis(L, ndn, bd);
  qo_halfbasis(L, nup2, bu2);
  qo_halfbasis(L, ndn2, bd2);
  uint32_t m = 1u << orb;
  for (size_t id = 0; id < dd; ++id)
    for (size_t iu = 0; iu < du; ++iu) {
      uint32_t u = bu[iu], d = bd[id];
      int par;
      size_t t;
      if (!spin) {
        if (pm < 0 ? !(u & m) : (u & m)) continue;
        par = popc32(u & (m - 1u));
        uint32_t j = qo_rank(bu2, (uint32_t)du2, u ^ m);
        t = j + du2 * id;
      } else {
        if (pm < 0 ? !(d & m) : (d & m)) continue;
        par = popc32(d & (m - 1u)) + popc32(u);
        uint32_t j = qo_rank(bd2, (uint32_t)dd2, d ^ m);
        t = iu + du2 * (size_t)j;
      }
      y[t] += z * ((par & 1) ? -1.0 : 1.0) * x[iu + du * id];
    }
  free(bu);
  free(bd);
  free(bu2);
  free(bd2);
}

/* Vector kernels of the band Lanczos on a list of vectors, split over
 * OpenMP threads.  Dot products are summed over 256 fixed chunks combined in
 * order, so the results do not depend on the thread count. */
#define QO_CHUNKS 256

/* out[k] = <V[k], w>, k < m */
void qo_multidot(int m, const double* const* V, const double* w, size_t n, double* out,
                 int nthreads) {
  double* part = (double*)malloc(sizeof(double) * (size_t)(m ? m : 1) * QO_CHUNKS);
  if (nthreads < 1) nthreads = 1;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
  for (int c = 0; c < QO_CHUNKS; ++c) {
    const size_t i0 = n * (size_t)c / QO_CHUNKS, i1 = n * (size_t)(c + 1) / QO_CHUNKS;
    for (int k = 0; k < m; ++k) {
      double s = 0.0;
      for (size_t i = i0; i < i1; ++i) s += V[k][i] * w[i];
      part[(size_t)k * QO_CHUNKS + c] = s;
    }
  }
  for (int k = 0; k < m; ++k) {
    double s = 0.0;
    for (int c = 0; c < QO_CHUNKS; ++c) s += part[(size_t)k * QO_CHUNKS + c];
    out[k] = s;
  }
  free(part);
}

/* V[k] -= coef[k] w, k < m */
void qo_sub_rank1(int m, double* const* V, const double* coef, const double* w, size_t n,
                  int nthreads) {
  if (nthreads < 1) nthreads = 1;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
  for (int c = 0; c < QO_CHUNKS; ++c) {
    const size_t i0 = n * (size_t)c / QO_CHUNKS, i1 = n * (size_t)(c + 1) / QO_CHUNKS;
    for (int k = 0; k < m; ++k) {
      const double a = coef[k];
      double* v = V[k];
      for (size_t i = i0; i < i1; ++i) v[i] -= a * w[i];
    }
  }
}

/* w -= sum_k coef[k] V[k], the terms subtracted in the order k = 0 .. m-1 */
void qo_sub_combination(int m, const double* const* V, const double* coef, double* w, size_t n,
                        int nthreads) {
  if (nthreads < 1) nthreads = 1;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
  for (int c = 0; c < QO_CHUNKS; ++c) {
    const size_t i0 = n * (size_t)c / QO_CHUNKS, i1 = n * (size_t)(c + 1) / QO_CHUNKS;
    for (size_t i = i0; i < i1; ++i) {
      double s = w[i];
      for (int k = 0; k < m; ++k) s -= coef[k] * V[k][i];
      w[i] = s;
    }
  }
}
