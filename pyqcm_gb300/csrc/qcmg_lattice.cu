// k x omega lattice integrals over the Lehmann cluster Green function
// (CPT / VCA / CDMFT), batched on the GPU in FP64.
//
// Inputs (one spin block): the cluster Green function G(z) from its
// Q-matrix (e, v), the bath hybridization Gamma(z) = tcb diag(1/(z-eb)) tcb^+,
// and the lattice hopping in Fourier form
//   t(K) - t_c = Hdiff + sum_e v_e exp(2 pi i K.R_{n_e}) |r_e><c_e|
// with K in the reduced (superlattice-dual) basis, as the reference builds it
// (lattice_model_instance::set_V, src_qcm/CPT.cpp:22-64).  Then
//   V(K,z) = t(K) - t_c - Gamma(z),
// and every per-(K,z) quantity goes through M(K,z) = G(z)^-1 - V(K,z):
//   SEF   log|det(V G - 1)| = log|det M| + log|det G|        (lattice_model_instance.cpp:624-643)
//   CPT   Gcpt = G (1 - V G)^-1 = M^-1                       (CPT.cpp:76-86)
//         g(K) = (1/L) sum_ab Gcpt_ab e^{2 pi i K.(x_b - x_a)} (lattice_model.cpp:724-740)
//   CDMFT PGF(z) = mean_K Gcpt(K, z)                          (CPT.cpp:283-345)
// G^-1 and log|det G| are computed once per frequency; each (K, z) point then
// costs one LU factorization of an L x L complex matrix, done by one thread
// with its matrix in shared memory (interleaved across threads, no bank
// conflicts).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <vector>

#include "qcmg_internal.h"
#include "qcmg_krylov.h"
#include "qcmg_lattice.h"

namespace qcmg {

struct cdbl {
  double x, y;
};
__device__ __forceinline__ cdbl cmul(cdbl a, cdbl b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ __forceinline__ cdbl cfma_sub(cdbl acc, cdbl a, cdbl b) {  // acc - a*b
  return {acc.x - (a.x * b.x - a.y * b.y), acc.y - (a.x * b.y + a.y * b.x)};
}
__device__ __forceinline__ cdbl cinv(cdbl a) {
  double d = a.x * a.x + a.y * a.y;
  return {a.x / d, -a.y / d};
}

// ---------------------------------------------------------------------------
// Per-frequency preparation: Base(z) = G(z)^-1 + Gamma(z) - Hdiff and
// log|det G(z)|, one block per frequency, Gauss-Jordan with partial pivoting
// in shared memory.

__global__ void k_freq_prep(int L, int nw, const double2* __restrict__ G,  // nw x L x L (G[b + a L] = G(b,a))
                            const double2* __restrict__ z, int nb, const double2* __restrict__ tcb,
                            const double* __restrict__ eb, const double2* __restrict__ Hdiff,
                            double2* __restrict__ base, double* __restrict__ logdetG) {
  extern __shared__ double2 sm[];
  double2* A = sm;              // L x 2L augmented [G | I], row-major A[r*2L + c]
  __shared__ int piv;
  __shared__ double ldet;
  const int w = blockIdx.x;
  const int L2 = 2 * L;
  // G(r, c) with numpy orientation: G stored as G[b + a L] = G(b, a)  ->  G(r,c) = Gw[r + c L]
  const double2* Gw = G + (size_t)w * L * L;
  for (int idx = threadIdx.x; idx < L * L2; idx += blockDim.x) {
    int r = idx / L2, c = idx % L2;
    A[idx] = c < L ? Gw[r + c * L] : make_double2(c - L == r ? 1.0 : 0.0, 0.0);
  }
  if (threadIdx.x == 0) ldet = 0.0;
  __syncthreads();
  for (int p = 0; p < L; ++p) {
    if (threadIdx.x == 0) {
      int best = p;
      double bv = -1.0;
      for (int r = p; r < L; ++r) {
        double2 a = A[r * L2 + p];
        double m = a.x * a.x + a.y * a.y;
        if (m > bv) {
          bv = m;
          best = r;
        }
      }
      piv = best;
      ldet += 0.5 * log(bv);
    }
    __syncthreads();
    if (piv != p)
      for (int c = threadIdx.x; c < L2; c += blockDim.x) {
        double2 t = A[p * L2 + c];
        A[p * L2 + c] = A[piv * L2 + c];
        A[piv * L2 + c] = t;
      }
    __syncthreads();
    const double2 pp = A[p * L2 + p];
    const cdbl ip = cinv({pp.x, pp.y});
    __syncthreads();
    for (int c = threadIdx.x; c < L2; c += blockDim.x) {
      cdbl v = cmul({A[p * L2 + c].x, A[p * L2 + c].y}, ip);
      A[p * L2 + c] = make_double2(v.x, v.y);
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < L * L2; idx += blockDim.x) {
      int r = idx / L2, c = idx % L2;
      if (r == p) continue;
      double2 f = A[r * L2 + p];
      double2 a = A[p * L2 + c];
      if (c == p) continue;  // column p is cleared below
      cdbl v = cfma_sub({A[idx].x, A[idx].y}, {f.x, f.y}, {a.x, a.y});
      A[idx] = make_double2(v.x, v.y);
    }
    __syncthreads();
    for (int r = threadIdx.x; r < L; r += blockDim.x)
      if (r != p) A[r * L2 + p] = make_double2(0.0, 0.0);
    __syncthreads();
  }
  // Base = G^-1 + Gamma - Hdiff, row-major base[r*L + c]
  const double2 zw = z[w];
  double2* B = base + (size_t)w * L * L;
  for (int idx = threadIdx.x; idx < L * L; idx += blockDim.x) {
    int r = idx / L, c = idx % L;
    double2 gi = A[r * L2 + L + c];
    double gx = gi.x - Hdiff[idx].x, gy = gi.y - Hdiff[idx].y;
    for (int i = 0; i < nb; ++i) {
      // Gamma(r,c) += tcb(r,i) conj(tcb(c,i)) / (z - eb_i)
      double2 a = tcb[r + (size_t)L * i], b = tcb[c + (size_t)L * i];
      double re = zw.x - eb[i], im = zw.y, den = re * re + im * im;
      double ur = re / den, ui = -im / den;
      double pr = a.x * b.x + a.y * b.y, pi = a.y * b.x - a.x * b.y;  // a conj(b)
      gx += pr * ur - pi * ui;
      gy += pr * ui + pi * ur;
    }
    B[idx] = make_double2(gx, gy);
  }
  if (threadIdx.x == 0) logdetG[w] = ldet;  // the pivots are those of G itself
}

// Sigma(z) = z - base with base = G^-1 + Gamma + t_c (k_freq_prep with the
// constant block -t_c); Gamma(z) alone for the hybridization function.
__global__ void k_sigma_from_base(int L, int nw, const double2* __restrict__ z,
                                  double2* __restrict__ base) {
  const int w = blockIdx.x;
  double2* B = base + (size_t)w * L * L;
  for (int idx = threadIdx.x; idx < L * L; idx += blockDim.x) {
    const int r = idx / L, c = idx % L;
    const double2 b = B[idx];
    B[idx] = make_double2((r == c ? z[w].x : 0.0) - b.x, (r == c ? z[w].y : 0.0) - b.y);
  }
}

__global__ void k_gamma(int L, int nw, const double2* __restrict__ z, int nb,
                        const double2* __restrict__ tcb, const double* __restrict__ eb,
                        double2* __restrict__ out) {
  const int w = blockIdx.x;
  const double2 zw = z[w];
  for (int idx = threadIdx.x; idx < L * L; idx += blockDim.x) {
    const int r = idx / L, c = idx % L;
    double gx = 0.0, gy = 0.0;
    for (int i = 0; i < nb; ++i) {  // the same sum as in k_freq_prep
      double2 a = tcb[r + (size_t)L * i], b = tcb[c + (size_t)L * i];
      double re = zw.x - eb[i], im = zw.y, den = re * re + im * im;
      double ur = re / den, ui = -im / den;
      double pr = a.x * b.x + a.y * b.y, pi = a.y * b.x - a.x * b.y;
      gx += pr * ur - pi * ui;
      gy += pr * ui + pi * ur;
    }
    out[(size_t)w * L * L + idx] = make_double2(gx, gy);
  }
}

void self_energy_batch(int L, int M, const double* e, const double* v, int nb, const double* tcb,
                       const double* eb, const double* tc, int nz, const double* z, double* sigma,
                       double* gamma, cudaStream_t s) {
  QCMG_CHECK_ARG(L > 0 && L <= 32, "Green function dimension must be 1..32");
  DevBuf<double> G, ldg, mtc;
  G.alloc((size_t)2 * L * L * nz);
  if (M > 0)
    green_function_batch(L, M, e, v, nz, z, G.p, s);
  else
    QCMG_CUDA(cudaMemsetAsync(G.p, 0, G.n * 8, s));
  // constant block -t_c
  std::vector<double> h((size_t)2 * L * L);
  QCMG_CUDA(cudaMemcpyAsync(h.data(), tc, h.size() * 8, cudaMemcpyDeviceToHost, s));
  QCMG_CUDA(cudaStreamSynchronize(s));
  for (double& x : h) x = -x;
  mtc.upload(h.data(), h.size(), s);
  ldg.alloc(nz);
  const size_t smem = (size_t)L * 2 * L * sizeof(double2);
  k_freq_prep<<<nz, 128, smem, s>>>(L, nz, (const double2*)G.p, (const double2*)z, nb,
                                    (const double2*)tcb, eb, (const double2*)mtc.p,
                                    (double2*)sigma, ldg.p);
  k_sigma_from_base<<<nz, 128, 0, s>>>(L, nz, (const double2*)z, (double2*)sigma);
  if (gamma)
    k_gamma<<<nz, 128, 0, s>>>(L, nz, (const double2*)z, nb, (const double2*)tcb, eb,
                               (double2*)gamma);
  QCMG_CUDA(cudaGetLastError());
  QCMG_CUDA(cudaStreamSynchronize(s));  // mtc, G go out of scope
}

// ---------------------------------------------------------------------------
// Per-point kernel.  MODE 0: SEF (sum of log|det M| weighted), MODE 1: CPT
// periodized g(K,z), MODE 2: mean of M^-1 (CDMFT projected GF).

struct PointArgs {
  int L;
  int nw;
  const double2* base;  // nw x L x L row-major
  int nel;
  const int* el_r;
  const int* el_c;
  const int* el_n;
  const double2* el_v;
  int nR;
  const double* R;  // nR x 3
  // K points: explicit list or a grid
  int nk;
  const double* K;  // nk x 3 (explicit) or null
  int gx, gy, gz;   // grid sizes (K = (i+off)/gx, ...)
  double off;       // 0 for the SEF grid, 0.5 for the CDMFT midpoint grid
  const double* gpos;  // L x 3 (CPT)
  double2* out;        // MODE 1: nw x nk;  MODE 2: partial sums
  double* vals;        // MODE 0: the per-point values, nw x nk
  int bpf;             // MODE 0: > 0: blocks per frequency (block b works on
                       // frequency b / bpf only, so partials never mix
                       // frequencies); 0: one flat range over all points
  const double* ldg;   // MODE 0: log|det G| per frequency, added point by point
  const int* el_start;  // nR + 1 element ranges per translation
  const double2* tab;   // grid phase tables (gx + gy + gz) x nR, or null: sincos per point
};

__device__ __forceinline__ void point_K(const PointArgs& A, int ik, double* K) {
  if (A.K) {
    K[0] = A.K[3 * ik];
    K[1] = A.K[3 * ik + 1];
    K[2] = A.K[3 * ik + 2];
  } else {
    int i = ik % A.gx, j = (ik / A.gx) % A.gy, l = ik / (A.gx * A.gy);
    K[0] = (i + A.off) / A.gx;
    K[1] = A.gy > 1 ? (j + A.off) / A.gy : 0.0;
    K[2] = A.gz > 1 ? (l + A.off) / A.gz : 0.0;
  }
}

template <int MODE>
__global__ void k_points(PointArgs A) {
  extern __shared__ double smem[];
  const int T = blockDim.x, t = threadIdx.x, L = A.L, LL = L * L;
  double* mr = smem;            // LL x T
  double* mi = smem + LL * T;   // LL x T
#define MR(r, c) mr[((r) * L + (c)) * T + t]
#define MI(r, c) mi[((r) * L + (c)) * T + t]
  const size_t npts = (size_t)A.nk * A.nw;
  // points of this block: a flat range, or (bpf > 0) the K points of one
  // frequency, strided by the frequency's blocks
  const bool per_freq = MODE == 0 && A.bpf > 0;
  const size_t w_blk = per_freq ? blockIdx.x / A.bpf : 0;
  const size_t first = per_freq ? w_blk * A.nk + (blockIdx.x % A.bpf) * (size_t)T + t
                                : blockIdx.x * (size_t)T + t;
  const size_t last = per_freq ? (w_blk + 1) * A.nk : npts;
  const size_t step = per_freq ? (size_t)A.bpf * T : (size_t)gridDim.x * T;
  for (size_t pt = first; pt < last; pt += step) {
    const int w = (int)(pt / A.nk), ik = (int)(pt % A.nk);
    double K[3];
    point_K(A, ik, K);
    const double2* B = A.base + (size_t)w * LL;
    for (int e = 0; e < LL; ++e) {
      double2 b = B[e];
      mr[e * T + t] = b.x;
      mi[e * T + t] = b.y;
    }
    // M = Base - sum_e v_e e^{2 pi i K.R_n(e)} at (r_e, c_e), one phase per
    // translation: on a grid the product of the three axes' table entries,
    // else a sincos
    for (int n = 0; n < A.nR; ++n) {
      const int e0 = A.el_start[n], e1 = A.el_start[n + 1];
      if (e0 == e1) continue;
      double s, c;
      if (A.tab) {
        const int ix = ik % A.gx, iy = (ik / A.gx) % A.gy, iz = ik / (A.gx * A.gy);
        const double2 tx = A.tab[(size_t)ix * A.nR + n];
        const double2 ty = A.tab[(size_t)(A.gx + iy) * A.nR + n];
        const double2 tz = A.tab[(size_t)(A.gx + A.gy + iz) * A.nR + n];
        const double xr = tx.x * ty.x - tx.y * ty.y, xi = tx.x * ty.y + tx.y * ty.x;
        c = xr * tz.x - xi * tz.y;
        s = xr * tz.y + xi * tz.x;
      } else {
        const double* Rn = A.R + 3 * n;
        const double ph = 2.0 * M_PI * (K[0] * Rn[0] + K[1] * Rn[1] + K[2] * Rn[2]);
        sincos(ph, &s, &c);
      }
      for (int e = e0; e < e1; ++e) {
        const double2 v = A.el_v[e];
        const int r = A.el_r[e], cc = A.el_c[e];
        MR(r, cc) -= v.x * c - v.y * s;
        MI(r, cc) -= v.x * s + v.y * c;
      }
    }
    // LU with partial pivoting (row interchanges), in place.
    int perm[32];
    for (int i = 0; i < L; ++i) perm[i] = i;
    double logabs = 0.0;
    for (int p = 0; p < L; ++p) {
      int best = p;
      double bv = MR(p, p) * MR(p, p) + MI(p, p) * MI(p, p);
      for (int r = p + 1; r < L; ++r) {
        double m = MR(r, p) * MR(r, p) + MI(r, p) * MI(r, p);
        if (m > bv) {
          bv = m;
          best = r;
        }
      }
      if (best != p) {
        for (int c = 0; c < L; ++c) {
          double a = MR(p, c), b = MI(p, c);
          MR(p, c) = MR(best, c);
          MI(p, c) = MI(best, c);
          MR(best, c) = a;
          MI(best, c) = b;
        }
        int tp = perm[p];
        perm[p] = perm[best];
        perm[best] = tp;
      }
      logabs += 0.5 * log(bv);
      const cdbl ip = cinv({MR(p, p), MI(p, p)});
      for (int r = p + 1; r < L; ++r) {
        cdbl f = cmul({MR(r, p), MI(r, p)}, ip);
        MR(r, p) = f.x;
        MI(r, p) = f.y;
        for (int c = p + 1; c < L; ++c) {
          cdbl v = cfma_sub({MR(r, c), MI(r, c)}, f, {MR(p, c), MI(p, c)});
          MR(r, c) = v.x;
          MI(r, c) = v.y;
        }
      }
    }
    if (MODE == 0) {
      // log|det(VG - 1)| = log|det M| + log|det G|, formed point by point:
      // at high frequencies both terms are ~L log|z| and their sum is tiny,
      // so summing the large terms over K first would leave the result to
      // the rounding of that sum
      A.vals[pt] = logabs + (A.ldg ? A.ldg[w] : 0.0);
      (void)perm;
    } else if (MODE == 1) {
      // y = M^-1 u, u_b = e^{2 pi i K.x_b};  g = (1/L) u^+ y
      cdbl y[32];
      for (int i = 0; i < L; ++i) {
        const double* x = A.gpos + 3 * perm[i];
        double ph = 2.0 * M_PI * (K[0] * x[0] + K[1] * x[1] + K[2] * x[2]);
        double s, c;
        sincos(ph, &s, &c);
        y[i] = {c, s};  // (P u)_i
      }
      for (int i = 0; i < L; ++i)  // forward: unit lower
        for (int j = 0; j < i; ++j) y[i] = cfma_sub(y[i], {MR(i, j), MI(i, j)}, y[j]);
      for (int i = L - 1; i >= 0; --i) {  // backward: upper
        for (int j = i + 1; j < L; ++j) y[i] = cfma_sub(y[i], {MR(i, j), MI(i, j)}, y[j]);
        y[i] = cmul(y[i], cinv({MR(i, i), MI(i, i)}));
      }
      double gr = 0.0, gi = 0.0;
      for (int b = 0; b < L; ++b) {
        const double* x = A.gpos + 3 * b;
        double ph = 2.0 * M_PI * (K[0] * x[0] + K[1] * x[1] + K[2] * x[2]);
        double s, c;
        sincos(ph, &s, &c);
        // conj(u_b) y_b
        gr += c * y[b].x + s * y[b].y;
        gi += c * y[b].y - s * y[b].x;
      }
      A.out[(size_t)w * A.nk + ik] = make_double2(gr / L, gi / L);
    } else {
      // column j of M^-1: solve M x = e_j (P applied), accumulate into out
      double2* O = A.out + ((size_t)blockIdx.x * A.nw + w) * LL;  // unused layout guard
      (void)O;
      for (int j = 0; j < L; ++j) {
        cdbl y[32];
        for (int i = 0; i < L; ++i) y[i] = {perm[i] == j ? 1.0 : 0.0, 0.0};
        for (int i = 0; i < L; ++i)
          for (int q = 0; q < i; ++q) y[i] = cfma_sub(y[i], {MR(i, q), MI(i, q)}, y[q]);
        for (int i = L - 1; i >= 0; --i) {
          for (int q = i + 1; q < L; ++q) y[i] = cfma_sub(y[i], {MR(i, q), MI(i, q)}, y[q]);
          y[i] = cmul(y[i], cinv({MR(i, i), MI(i, i)}));
        }
        // accumulate column j of the inverse: out[(w*nk + ik) ...] reduced later
        for (int i = 0; i < L; ++i)
          A.out[((size_t)w * A.nk + ik) * LL + i * L + j] = make_double2(y[i].x, y[i].y);
      }
    }
  }
#undef MR
#undef MI
}

// Sum of each row of vals (nrow x ncol), one block of kSumThreads per row:
// thread t adds the elements t, t + kSumThreads, ... in order, then a fixed
// tree adds the threads' sums.  The order depends on neither the point
// kernel's block size nor its grid, so the Potthoff functional is the same
// number whatever block size the tuner picks.
constexpr int kSumThreads = 256;
__global__ void __launch_bounds__(kSumThreads) k_row_sums(const double* __restrict__ vals,
                                                          int ncol, double* __restrict__ sums) {
  __shared__ double sh[kSumThreads];
  const double* row = vals + (size_t)blockIdx.x * ncol;
  double s = 0.0;
  for (int i = threadIdx.x; i < ncol; i += kSumThreads) s += row[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int h = kSumThreads / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) sh[threadIdx.x] += sh[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = sh[0];
}

// ---------------------------------------------------------------------------
// host side

static int point_threads(int L) {
  // one L x L complex matrix per thread in shared memory, up to 224 KB a
  // block (one block per SM at L = 12: 96 points)
  const size_t per = (size_t)2 * L * L * 8;  // bytes per point
  int T = (int)((224 * 1024) / per);
  if (const char* e = std::getenv("QCMG_POINT_THREADS")) {  // tuning override
    const int v = std::atoi(e);
    if (v >= 32 && (size_t)v * per <= 224 * 1024) T = v;
  }
  T = (T / 32) * 32;
  if (T > 256) T = 256;
  if (T < 32) T = 32;
  return T;
}

// Block size of the SEF point kernel, tuned once per matrix dimension L and
// process: each candidate (multiples of 32 whose matrices fit the shared
// memory budget, at most four, largest first) runs the same launch on the
// caller's first frequencies (as many as one launch of that shape takes),
// timed with CUDA events after one untimed run; the least time per
// frequency is kept.  QCMG_POINT_THREADS overrides the choice;
// QCMG_VERBOSE reports it on stderr.
static std::mutex g_tune_mu;
static std::map<int, int> g_tuned_sef;

template <class Launch>
static int tuned_sef_threads(int L, Launch&& launch, cudaStream_t s) {
  if (std::getenv("QCMG_POINT_THREADS")) return point_threads(L);
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tuned_sef.find(L);
    if (it != g_tuned_sef.end()) return it->second;
  }
  const int tmax = point_threads(L);
  std::vector<int> cand;
  for (int T = tmax; T >= 32 && cand.size() < 4; T -= 32) cand.push_back(T);
  cudaEvent_t e0, e1;
  QCMG_CUDA(cudaEventCreate(&e0));
  QCMG_CUDA(cudaEventCreate(&e1));
  int best = tmax;
  float best_ms = 0.0f;
  for (int T : cand) {
    launch(T);  // untimed: first-launch costs
    QCMG_CUDA(cudaEventRecord(e0, s));
    const int nf = launch(T);  // frequencies this launch covered
    QCMG_CUDA(cudaEventRecord(e1, s));
    QCMG_CUDA(cudaEventSynchronize(e1));
    float ms = 0.0f;
    QCMG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    ms /= (float)nf;
    if (T == cand.front() || ms < best_ms) {
      best_ms = ms;
      best = T;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (std::getenv("QCMG_VERBOSE"))
    std::fprintf(stderr,
                 "qcmg: SEF point kernel, L = %d: %d threads per block (%.3f ms per frequency)\n",
                 L, best, best_ms);
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tuned_sef[L] = best;
  return best;
}

void Lattice::prepare(int nw, const double* z, cudaStream_t s) {
  QCMG_CHECK_ARG(L > 0 && L <= 32, "lattice Green function dimension must be 1..32");
  QCMG_CHECK_ARG(M >= 0, "Q-matrix not set");
  DevBuf<double> dz;
  dz.upload(z, (size_t)2 * nw, s);
  DevBuf<double> G;
  G.alloc((size_t)2 * L * L * nw);
  if (M > 0) {
    green_function_batch(L, M, e.p, v.p, nw, dz.p, G.p, s);
  } else {
    QCMG_CUDA(cudaMemsetAsync(G.p, 0, G.n * 8, s));
  }
  base.alloc((size_t)2 * L * L * nw);
  logdetG.alloc(nw);
  size_t smem = (size_t)L * 2 * L * sizeof(double2);
  k_freq_prep<<<nw, 128, smem, s>>>(L, nw, (const double2*)G.p, (const double2*)dz.p, nb,
                                    (const double2*)tcb.p, eb.p, (const double2*)hdiff.p,
                                    (double2*)base.p, logdetG.p);
  QCMG_CUDA(cudaGetLastError());
  QCMG_CUDA(cudaStreamSynchronize(s));
  prepared_nw = nw;
}

static PointArgs point_args(const Lattice& lat, int nw) {
  PointArgs A;
  A.L = lat.L;
  A.nw = nw;
  A.base = (const double2*)lat.base.p;
  A.nel = lat.nel;
  A.el_r = lat.el_r.p;
  A.el_c = lat.el_c.p;
  A.el_n = lat.el_n.p;
  A.el_v = (const double2*)lat.el_v.p;
  A.nR = lat.nR;
  A.R = lat.R.p;
  A.K = nullptr;
  A.gx = A.gy = A.gz = 1;
  A.off = 0.0;
  A.gpos = lat.gpos.p;
  A.out = nullptr;
  A.vals = nullptr;
  A.bpf = 0;
  A.ldg = nullptr;
  A.el_start = lat.el_start.p;
  A.tab = nullptr;
  return A;
}

const double* Lattice::phase_tables(int gx, int gy, int gz, double off, cudaStream_t s) {
  if (tab.p && gx == tab_gx && gy == tab_gy && gz == tab_gz && off == tab_off) return tab.p;
  // K = ((i + off)/gx, gy > 1 ? (j + off)/gy : 0, gz > 1 ? (l + off)/gz : 0), as point_K
  std::vector<double> h((size_t)2 * (gx + gy + gz) * nR);
  auto fill = [&](int base, int g, int axis) {
    for (int i = 0; i < g; ++i) {
      const double k = (axis == 0 || g > 1) ? (i + off) / g : 0.0;
      for (int n = 0; n < nR; ++n) {
        const double ph = 2.0 * M_PI * k * R_host[3 * n + axis];
        const size_t at = ((size_t)(base + i) * nR + n) * 2;
        h[at] = std::cos(ph);
        h[at + 1] = std::sin(ph);
      }
    }
  };
  fill(0, gx, 0);
  fill(gx, gy, 1);
  fill(gx + gy, gz, 2);
  tab.upload(h.data(), h.size(), s);
  QCMG_CUDA(cudaStreamSynchronize(s));
  tab_gx = gx;
  tab_gy = gy;
  tab_gz = gz;
  tab_off = off;
  return tab.p;
}

double Lattice::sef_grid(int nw, const double* w, const double* wt, int nkx, int nky, int nkz,
                         cudaStream_t s) {
  std::vector<double> z(2 * nw);
  for (int i = 0; i < nw; ++i) {
    z[2 * i] = 0.0;
    z[2 * i + 1] = w[i];
  }
  double total = 0.0;
  const int nk = nkx * nky * nkz;
  // frequencies are processed one by one so the per-frequency weight is
  // applied exactly; each launch covers the whole K grid
  prepare(nw, z.data(), s);
  const double2* phases = (const double2*)phase_tables(nkx, nky, nkz, 0.0, s);
  // Several frequencies per launch (enough blocks for many waves on every
  // SM), each block working on the points of one frequency; every point's
  // log|det| is stored, and each frequency's sum is then taken in a fixed
  // order (k_row_sums), so the weights apply to whole per-frequency sums and
  // the result does not depend on the block size.
  auto shape = [&](int T, unsigned& bpf, int& fpl) {
    bpf = (unsigned)std::max<size_t>(1, std::min<size_t>((nk + T - 1) / T, 152 * 4));
    fpl = std::max(1, std::min(nw, (int)((152u * 16u + bpf - 1) / bpf)));
  };
  DevBuf<double> vals, sums;
  auto launch = [&](int T, int i0, int nf, unsigned bpf) {
    const size_t smem = (size_t)2 * L * L * T * 8;
    QCMG_CUDA(cudaFuncSetAttribute(k_points<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)smem));
    if (vals.n < (size_t)nf * nk) vals.alloc((size_t)nf * nk);
    PointArgs A = point_args(*this, nf);
    A.base = (const double2*)base.p + (size_t)i0 * L * L;
    A.nk = nk;
    A.gx = nkx;
    A.gy = nky;
    A.gz = nkz;
    A.off = 0.0;
    A.vals = vals.p;
    A.bpf = (int)bpf;
    A.ldg = logdetG.p + i0;
    A.tab = phases;
    k_points<0><<<bpf * nf, T, smem, s>>>(A);
    QCMG_CUDA(cudaGetLastError());
  };
  const int T = tuned_sef_threads(
      L,
      [&](int Tc) {
        unsigned b;
        int f;
        shape(Tc, b, f);
        const int nf = std::min(f, nw);
        launch(Tc, 0, nf, b);
        return nf;
      },
      s);
  unsigned bpf;
  int fpl;
  shape(T, bpf, fpl);
  if (sums.n < (size_t)fpl) sums.alloc((size_t)fpl);
  std::vector<double> hs((size_t)fpl);
  for (int i0 = 0; i0 < nw; i0 += fpl) {
    const int nf = std::min(fpl, nw - i0);
    launch(T, i0, nf, bpf);
    k_row_sums<<<nf, kSumThreads, 0, s>>>(vals.p, nk, sums.p);
    QCMG_CUDA(cudaGetLastError());
    QCMG_CUDA(cudaMemcpyAsync(hs.data(), sums.p, (size_t)nf * 8, cudaMemcpyDeviceToHost, s));
    QCMG_CUDA(cudaStreamSynchronize(s));
    for (int f = 0; f < nf; ++f) total += wt[i0 + f] * (hs[f] / nk);
  }
  return total;
}

void Lattice::cpt(int nz, const double* z, int nk, const double* K, double* g, cudaStream_t s) {
  prepare(nz, z, s);
  PointArgs A = point_args(*this, nz);
  DevBuf<double> dK, out;
  dK.upload(K, (size_t)3 * nk, s);
  out.alloc((size_t)2 * nz * nk);
  A.nk = nk;
  A.K = dK.p;
  A.out = (double2*)out.p;
  const int T = point_threads(L);
  const size_t smem = (size_t)2 * L * L * T * 8;
  QCMG_CUDA(cudaFuncSetAttribute(k_points<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const size_t npts = (size_t)nz * nk;
  unsigned gr = (unsigned)std::max<size_t>(1, std::min<size_t>((npts + T - 1) / T, 152 * 8));
  k_points<1><<<gr, T, smem, s>>>(A);
  QCMG_CUDA(cudaGetLastError());
  QCMG_CUDA(cudaMemcpyAsync(g, out.p, (size_t)2 * nz * nk * 8, cudaMemcpyDeviceToHost, s));
  QCMG_CUDA(cudaStreamSynchronize(s));
}

// K means of the per-point inverses, per frequency and moment:
//   out[(w nmom + m) LL + e] = (1/nk) sum_K ph[m nk + K] inv[w][K][e]
// (ph null: one moment with phase 1).  One block per (frequency, 32
// consecutive elements e): the lanes take consecutive e (coalesced loads of
// each point's block), the warps interleave over K, and every moment's sums
// stay in registers until a fixed-order reduction over the warps in shared
// memory.
constexpr int kMaxMoments = 16;
constexpr int kMomWarps = 8;

__global__ void __launch_bounds__(32 * kMomWarps)
    k_mean_moments(const double2* __restrict__ inv, int nw, int nk, int LL, int nmom,
                   const double2* __restrict__ ph, double2* __restrict__ out) {
  __shared__ double red[2][kMomWarps][32];
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const int w = blockIdx.x, e = blockIdx.y * 32 + lane;
  const int nm = ph ? nmom : 1;
  double sr[kMaxMoments], si[kMaxMoments];
#pragma unroll
  for (int m = 0; m < kMaxMoments; ++m) sr[m] = si[m] = 0.0;
  if (e < LL) {
    const double2* col = inv + (size_t)w * nk * LL + e;
    for (int k = wp; k < nk; k += kMomWarps) {
      const double2 v = col[(size_t)k * LL];
      if (!ph) {
        sr[0] += v.x;
        si[0] += v.y;
        continue;
      }
#pragma unroll
      for (int m = 0; m < kMaxMoments; ++m) {
        if (m < nm) {
          const double2 p = ph[(size_t)m * nk + k];
          sr[m] += v.x * p.x - v.y * p.y;
          si[m] += v.x * p.y + v.y * p.x;
        }
      }
    }
  }
#pragma unroll
  for (int m = 0; m < kMaxMoments; ++m) {
    if (m < nm) {  // the same for the whole block
      red[0][wp][lane] = sr[m];
      red[1][wp][lane] = si[m];
      __syncthreads();
      if (wp == 0 && e < LL) {
        double a = 0.0, b = 0.0;
        for (int q = 0; q < kMomWarps; ++q) {
          a += red[0][q][lane];
          b += red[1][q][lane];
        }
        out[((size_t)w * nm + m) * LL + e] = make_double2(a / nk, b / nk);
      }
      __syncthreads();
    }
  }
}

void Lattice::projected(int nw, const double* w, int kside, int dimk, double* pgf, cudaStream_t s) {
  std::vector<double> z(2 * nw);
  for (int i = 0; i < nw; ++i) {
    z[2 * i] = 0.0;
    z[2 * i + 1] = w[i];
  }
  const int g = kside;
  kmean(nw, z.data(), dimk >= 1 ? g : 1, dimk >= 2 ? g : 1, dimk >= 3 ? g : 1,
        dimk >= 1 ? 0.5 : 0.0, pgf, s);
}

void Lattice::kmean(int nz, const double* z, int gx, int gy, int gz, double off, double* out_host,
                    cudaStream_t s) {
  kmoments(nz, z, gx, gy, gz, off, 0, nullptr, out_host, s);
}

void Lattice::kmoments(int nz, const double* z, int gx, int gy, int gz, double off, int nmom,
                       const double* Rm, double* out_host, cudaStream_t s) {
  QCMG_CHECK_ARG(nmom >= 0 && nmom <= kMaxMoments, "at most 16 translations per call");
  const int nk = gx * gy * gz, LL = L * L;
  const int T = point_threads(L);
  const size_t smem = (size_t)2 * L * L * T * 8;
  QCMG_CUDA(cudaFuncSetAttribute(k_points<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  // phase of each translation at each grid point, K as point_K lays it out
  DevBuf<double> ph;
  if (nmom > 0) {
    std::vector<double> h((size_t)2 * nmom * nk);
    for (int m = 0; m < nmom; ++m)
      for (int ik = 0; ik < nk; ++ik) {
        const int i = ik % gx, j = (ik / gx) % gy, l = ik / (gx * gy);
        const double K0 = (i + off) / gx, K1 = gy > 1 ? (j + off) / gy : 0.0,
                     K2 = gz > 1 ? (l + off) / gz : 0.0;
        const double a = 2.0 * M_PI * (K0 * Rm[3 * m] + K1 * Rm[3 * m + 1] + K2 * Rm[3 * m + 2]);
        h[2 * ((size_t)m * nk + ik)] = std::cos(a);
        h[2 * ((size_t)m * nk + ik) + 1] = std::sin(a);
      }
    ph.upload(h.data(), h.size(), s);
  }
  const int nm = nmom > 0 ? nmom : 1;
  // frequencies in chunks whose per-point inverses fit in ~512 MB
  const size_t per_z = (size_t)nk * LL * 16;
  const int chunk = (int)std::max<size_t>(1, std::min<size_t>(nz, ((size_t)512 << 20) / per_z));
  DevBuf<double> inv, out;
  inv.alloc((size_t)2 * chunk * nk * LL);
  out.alloc((size_t)2 * chunk * nm * LL);
  for (int z0 = 0; z0 < nz; z0 += chunk) {
    const int nc = std::min(chunk, nz - z0);
    prepare(nc, z + 2 * (size_t)z0, s);
    PointArgs A = point_args(*this, nc);
    A.gx = gx;
    A.gy = gy;
    A.gz = gz;
    A.nk = nk;
    A.off = off;
    A.tab = (const double2*)phase_tables(gx, gy, gz, off, s);
    A.out = (double2*)inv.p;
    const size_t npts = (size_t)nc * nk;
    unsigned gr = (unsigned)std::max<size_t>(1, std::min<size_t>((npts + T - 1) / T, 152 * 8));
    k_points<2><<<gr, T, smem, s>>>(A);
    k_mean_moments<<<dim3(nc, (LL + 31) / 32), 32 * kMomWarps, 0, s>>>(
        (const double2*)inv.p, nc, nk, LL, nm, nmom > 0 ? (const double2*)ph.p : nullptr,
        (double2*)out.p);
    QCMG_CUDA(cudaGetLastError());
    QCMG_CUDA(cudaMemcpyAsync(out_host + (size_t)2 * z0 * nm * LL, out.p,
                              (size_t)2 * nc * nm * LL * 8, cudaMemcpyDeviceToHost, s));
    QCMG_CUDA(cudaStreamSynchronize(s));
  }
}

}  // namespace qcmg
