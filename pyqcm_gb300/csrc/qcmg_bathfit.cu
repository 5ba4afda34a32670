// CDMFT bath fit on the device: least squares of the residuals
//   r_n = sqrt(w_n) (Gamma(i w_n) + G_host(i w_n)),  real and imaginary parts,
//   Gamma(z) = theta (z - E)^-1 theta^T,  E diagonal (bath energies),
// over the bath parameters x, which enter theta (cluster-bath hybridization,
// ns x nb) and E linearly through a list of entries (parameter p adds
// v * x_p to theta[i][j] or to E[j][j]).
//
// Restates the fit of the reference's CDMFT step: the residuals of
// CDMFT_residuals (pyqcm src_qcm/CPT.cpp:556-610) minimized by least squares
// (optimize(method='trf'), pyqcm/cdmft.py:1539-1640).  Here the Jacobian is
// exact (Gamma is linear in theta and in (z - e_b)^-1 per bath orbital) and
// the minimizer is Levenberg-Marquardt with Marquardt's diagonal scaling and
// Nielsen's damping update; it stops on the same three tests as the
// reference's solver: relative cost decrease below ftol on a step whose gain
// ratio exceeds 1/4, step below xtol (xtol + |x|), gradient below gtol.
// With ftol = 0 (convergence on the gradient) exact Gauss-Newton steps
// follow for as long as they lower the gradient.
//
// One CTA per instance runs the whole fit: the normal equations J^T J,
// J^T r and the cost are reduced in shared memory in a fixed order
// (deterministic), J^T J through frequency sums of the bath propagators
// (see fit_normal), and thread 0 solves the damped system by Cholesky.  The
// iteration count is bounded by max_iter; no thread waits on another block.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <memory>
#include <vector>

#include "qcmg.h"
#include "qcmg_internal.h"

namespace qcmg {

constexpr int kFitMaxSites = 8;
constexpr int kFitMaxBath = 16;
constexpr int kFitMaxPar = 32;
constexpr int kFitMaxEnt = 128;
constexpr int kFitMaxChunk = 64;  // frequencies per chunk of residuals
constexpr int kFitThreads = 256;

struct BathFitArgs {
  int ns, nb, nw, npar, nent;
  const double* w;       // nw frequencies
  const double* wt;      // nw weights
  const double* host;    // ninst x nw x ns x ns complex (re, im)
  const int* ent_par;    // nent
  const int* ent_kind;   // 0: theta[i][j], 1: E[j][j]
  const int* ent_i;
  const int* ent_j;
  const double* ent_val;
  const double* theta0;  // ninst x ns x nb
  const double* e0;      // ninst x nb (diagonal of E)
  double* x;             // ninst x npar
  int max_iter;
  int fc;                // frequencies per chunk of residuals
  double xtol, ftol, gtol;
  double* cost;          // ninst: final cost 1/2 sum r^2
  int* iters;            // ninst
  int* status;           // ninst: 1 ftol, 2 xtol, 3 gtol, 0 max_iter, -1 singular
};

struct FitShared {
  double x[kFitMaxPar], xn[kFitMaxPar], dx[kFitMaxPar];
  double theta[kFitMaxSites * kFitMaxBath], e[kFitMaxBath];
  double A[kFitMaxPar * kFitMaxPar], g[kFitMaxPar];
  double M[kFitMaxPar * kFitMaxPar], rhs[kFitMaxPar];
  double red[kFitThreads];
  int ep[kFitMaxEnt], ek[kFitMaxEnt], ei[kFitMaxEnt], ej[kFitMaxEnt];
  double ev[kFitMaxEnt];
  double gent[kFitMaxEnt];  // gradient contribution of each entry
  double gram[kFitMaxBath * kFitMaxBath];
  double cost, accepted, lambda, nu;
  int flag, done, it;
  // behind the struct (dynamic shared memory): the residual chunk
  // R[f][a*ns+c] (fc x ns^2), g_b(w) of the chunk (fc x nb) and the
  // frequency sums T (3 x nb x nb)
  double2* R;
  double2* gb;
  double2* T;
};

__device__ __forceinline__ double2& R_at(FitShared& S, const BathFitArgs& A, int f, int ac) {
  return S.R[(size_t)f * A.ns * A.ns + ac];
}

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// theta and e from parameters xs (whole block; ends with a barrier)
__device__ void fit_blocks(FitShared& S, const BathFitArgs& A, int inst, const double* xs) {
  const int ns = A.ns, nb = A.nb;
  for (int k = threadIdx.x; k < ns * nb; k += blockDim.x) S.theta[k] = A.theta0[(size_t)inst * ns * nb + k];
  for (int k = threadIdx.x; k < nb; k += blockDim.x) S.e[k] = A.e0[(size_t)inst * nb + k];
  __syncthreads();
  if (threadIdx.x == 0) {  // entries may share a target: one thread, fixed order
    for (int q = 0; q < A.nent; ++q) {
      const double v = S.ev[q] * xs[S.ep[q]];
      if (S.ek[q] == 0)
        S.theta[S.ei[q] * nb + S.ej[q]] += v;
      else
        S.e[S.ej[q]] += v;
    }
  }
  __syncthreads();
}

// Residual chunk f0..f0+nf at the current theta/e: R = Gamma + G_host.
__device__ void fit_residual_chunk(FitShared& S, const BathFitArgs& A, int inst, int f0, int nf) {
  const int ns = A.ns, nb = A.nb, n2 = ns * ns;
  for (int k = threadIdx.x; k < nf * n2; k += blockDim.x) {
    const int f = k / n2, ac = k - f * n2, a = ac / ns, c = ac - a * ns;
    const double wv = A.w[f0 + f];
    double2 G = make_double2(0.0, 0.0);
    for (int b = 0; b < nb; ++b) {
      // 1 / (i w - e_b) = (-e_b - i w) / (e_b^2 + w^2)
      const double eb = S.e[b], den = eb * eb + wv * wv;
      const double t = S.theta[a * nb + b] * S.theta[c * nb + b];
      G.x += t * (-eb / den);
      G.y += t * (-wv / den);
    }
    const double2 h = reinterpret_cast<const double2*>(A.host)[((size_t)inst * A.nw + f0 + f) * n2 + ac];
    R_at(S, A, f, ac) = make_double2(G.x + h.x, G.y + h.y);
  }
}

// Block sum of one value per thread, fixed order; every thread gets it.
__device__ double fit_block_sum(FitShared& S, double v) {
  S.red[threadIdx.x] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < (int)blockDim.x; ++k) s += S.red[k];
    S.red[0] = s;
  }
  __syncthreads();
  const double s = S.red[0];
  __syncthreads();
  return s;
}

// Cost 1/2 sum_n w_n |Gamma + G_host|^2 at the current theta/e.
__device__ double fit_cost(FitShared& S, const BathFitArgs& A, int inst) {
  const int n2 = A.ns * A.ns;
  double part = 0.0;
  for (int f0 = 0; f0 < A.nw; f0 += A.fc) {
    const int nf = min(A.fc, A.nw - f0);
    fit_residual_chunk(S, A, inst, f0, nf);
    __syncthreads();
    for (int k = threadIdx.x; k < nf * n2; k += blockDim.x) {
      const int f = k / n2, ac = k - f * n2;
      const double2 r = R_at(S, A, f, ac);
      part += A.wt[f0 + f] * (r.x * r.x + r.y * r.y);
    }
    __syncthreads();
  }
  return 0.5 * fit_block_sum(S, part);
}

// Upper-triangle pair k -> (p, q), q >= p, row-major.
__device__ __forceinline__ void fit_pair(int k, int np, int* p, int* q) {
  int pp = 0, rem = k;
  while (rem >= np - pp) {
    rem -= np - pp;
    ++pp;
  }
  *p = pp;
  *q = pp + rem;
}

__device__ __forceinline__ double2 cconjmul(double2 a, double2 b) {  // a * conj(b)
  return make_double2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}

// The Jacobian blocks are outer products: with g_b(w) = 1/(i w - e_b) and
// theta_b the b-th column of theta (real),
//   d Gamma / d theta[s][b] = g_b (e_s theta_b^T + theta_b e_s^T),
//   d Gamma / d e_b         = g_b^2 theta_b theta_b^T,
// so sum_ac dG_p conj(dG_q) is a product of the scalar functions times real
// dot products of {e_s, theta_b}; summed over frequencies, J^T J needs only
//   T1[b][b'] = sum_w wt g_b conj(g_b'),  T2[b][b'] = sum_w wt g_b conj(g_b'^2),
//   T3[b][b'] = sum_w wt g_b^2 conj(g_b'^2)
// and the Gram matrix of the columns of theta (same values as the dense
// sum over frequencies and matrix elements, summed in another order).
// Dot product of two term vectors: kind 0 = unit vector e_i, 1 = theta_b.
__device__ __forceinline__ double fit_vdot(const FitShared& S, const double* gram, int nb, int k1,
                                           int i1, int k2, int i2) {
  if (k1 == 0 && k2 == 0) return i1 == i2 ? 1.0 : 0.0;
  if (k1 == 0) return S.theta[i1 * nb + i2];
  if (k2 == 0) return S.theta[i2 * nb + i1];
  return gram[i1 * nb + i2];
}

// Terms of entry q: (u kind, u index, w kind, w index) of u w^T; a theta
// entry (s, b) has two terms, an E entry (b, b) one.
__device__ __forceinline__ int fit_terms(const FitShared& S, int q, int (&t)[2][4]) {
  const int b = S.ej[q];
  if (S.ek[q] == 0) {
    const int s = S.ei[q];
    t[0][0] = 0; t[0][1] = s; t[0][2] = 1; t[0][3] = b;
    t[1][0] = 1; t[1][1] = b; t[1][2] = 0; t[1][3] = s;
    return 2;
  }
  t[0][0] = 1; t[0][1] = b; t[0][2] = 1; t[0][3] = b;
  return 1;
}

// J^T J (A), J^T r (g) and the cost at the current theta/e.
__device__ double fit_normal(FitShared& S, const BathFitArgs& A, int inst) {
  const int ns = A.ns, nb = A.nb, n2 = ns * ns, np = A.npar, nbb = nb * nb;
  double2* gb = S.gb;   // nf x nb: g_b(w) of the chunk
  double2* T = S.T;     // 3 x nb x nb
  double* gram = S.gram;
  for (int k = threadIdx.x; k < nbb; k += blockDim.x) {
    const int b = k / nb, c = k - b * nb;
    double sum = 0.0;
    for (int a = 0; a < ns; ++a) sum += S.theta[a * nb + b] * S.theta[a * nb + c];
    gram[k] = sum;
  }
  // per-thread accumulators owned across chunks (fixed assignment):
  // table element k = tid (< nb^2) and gradient entry q = tid (< nent)
  double2 t1 = make_double2(0.0, 0.0), t2 = t1, t3 = t1;
  double gq = 0.0, part = 0.0;
  for (int f0 = 0; f0 < A.nw; f0 += A.fc) {
    const int nf = min(A.fc, A.nw - f0);
    fit_residual_chunk(S, A, inst, f0, nf);
    for (int k = threadIdx.x; k < nf * nb; k += blockDim.x) {
      const int f = k / nb, b = k - f * nb;
      const double wv = A.w[f0 + f], eb = S.e[b], den = eb * eb + wv * wv;
      gb[k] = make_double2(-eb / den, -wv / den);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nf * n2; k += blockDim.x) {
      const int f = k / n2, ac = k - f * n2;
      const double2 r = R_at(S, A, f, ac);
      part += A.wt[f0 + f] * (r.x * r.x + r.y * r.y);
    }
    if ((int)threadIdx.x < nbb) {
      const int b = threadIdx.x / nb, c = threadIdx.x - b * nb;
      for (int f = 0; f < nf; ++f) {
        const double wt = A.wt[f0 + f];
        const double2 u = gb[f * nb + b], v = gb[f * nb + c];
        const double2 u2 = cmul(u, u), v2 = cmul(v, v);
        const double2 a1 = cconjmul(u, v), a2 = cconjmul(u, v2), a3 = cconjmul(u2, v2);
        t1.x += wt * a1.x; t1.y += wt * a1.y;
        t2.x += wt * a2.x; t2.y += wt * a2.y;
        t3.x += wt * a3.x; t3.y += wt * a3.y;
      }
    }
    if ((int)threadIdx.x < A.nent) {
      const int q = threadIdx.x, b = S.ej[q];
      for (int f = 0; f < nf; ++f) {
        // sum_ac u_a w_c conj(R_ac) over the entry's terms, times its g
        double2 sum = make_double2(0.0, 0.0);
        if (S.ek[q] == 0) {
          const int s = S.ei[q];
          for (int c = 0; c < ns; ++c) {
            const double2 r1 = R_at(S, A, f, s * ns + c), r2 = R_at(S, A, f, c * ns + s);
            const double th = S.theta[c * nb + b];
            sum.x += th * (r1.x + r2.x);
            sum.y -= th * (r1.y + r2.y);
          }
        } else {
          for (int a2 = 0; a2 < ns; ++a2)
            for (int c = 0; c < ns; ++c) {
              const double2 r = R_at(S, A, f, a2 * ns + c);
              const double th = S.theta[a2 * nb + b] * S.theta[c * nb + b];
              sum.x += th * r.x;
              sum.y -= th * r.y;
            }
        }
        double2 g = gb[f * nb + b];
        if (S.ek[q] != 0) g = cmul(g, g);
        const double2 z = cmul(g, sum);
        gq += A.wt[f0 + f] * z.x;
      }
    }
    __syncthreads();
  }
  if ((int)threadIdx.x < nbb) {
    T[threadIdx.x] = t1;
    T[nbb + threadIdx.x] = t2;
    T[2 * nbb + threadIdx.x] = t3;
  }
  if ((int)threadIdx.x < A.nent) S.gent[threadIdx.x] = S.ev[threadIdx.x] * gq;
  __syncthreads();
  // gradient: the entries of each parameter in their fixed order
  if ((int)threadIdx.x < np) {
    double sum = 0.0;
    for (int q = 0; q < A.nent; ++q)
      if (S.ep[q] == (int)threadIdx.x) sum += S.gent[q];
    S.g[threadIdx.x] = sum;
  }
  // J^T J from the tables: pair (p, q) over the entries of p and of q
  const int npairs = np * (np + 1) / 2;
  for (int k = threadIdx.x; k < npairs; k += blockDim.x) {
    int p, q;
    fit_pair(k, np, &p, &q);
    double sum = 0.0;
    for (int e1 = 0; e1 < A.nent; ++e1) {
      if (S.ep[e1] != p) continue;
      int ta[2][4];
      const int na = fit_terms(S, e1, ta);
      for (int e2 = 0; e2 < A.nent; ++e2) {
        if (S.ep[e2] != q) continue;
        int tb[2][4];
        const int nbt = fit_terms(S, e2, tb);
        const int b1 = S.ej[e1], b2 = S.ej[e2];
        double2 Tv;
        if (S.ek[e1] == 0 && S.ek[e2] == 0) {
          Tv = T[b1 * nb + b2];
        } else if (S.ek[e1] == 0) {
          Tv = T[nbb + b1 * nb + b2];
        } else if (S.ek[e2] == 0) {
          const double2 c = T[nbb + b2 * nb + b1];  // sum g_b1^2 conj(g_b2) = conj(T2[b2][b1])
          Tv = make_double2(c.x, -c.y);
        } else {
          Tv = T[2 * nbb + b1 * nb + b2];
        }
        double dots = 0.0;
        for (int i = 0; i < na; ++i)
          for (int j = 0; j < nbt; ++j)
            dots += fit_vdot(S, gram, nb, ta[i][0], ta[i][1], tb[j][0], tb[j][1]) *
                    fit_vdot(S, gram, nb, ta[i][2], ta[i][3], tb[j][2], tb[j][3]);
        sum += S.ev[e1] * S.ev[e2] * Tv.x * dots;
      }
    }
    S.A[p * np + q] = sum;
    S.A[q * np + p] = sum;
  }
  __syncthreads();
  return 0.5 * fit_block_sum(S, part);
}

// Solves M dx = rhs (n x n symmetric positive definite) by Cholesky in place
// (thread 0).  False when M is not positive definite.
__device__ bool fit_cholesky_solve(double* M, double* rhs, double* dx, int n) {
  for (int j = 0; j < n; ++j) {
    double d = M[j * n + j];
    for (int k = 0; k < j; ++k) d -= M[j * n + k] * M[j * n + k];
    if (!(d > 0.0)) return false;
    d = sqrt(d);
    M[j * n + j] = d;
    for (int i = j + 1; i < n; ++i) {
      double s = M[i * n + j];
      for (int k = 0; k < j; ++k) s -= M[i * n + k] * M[j * n + k];
      M[i * n + j] = s / d;
    }
  }
  for (int i = 0; i < n; ++i) {
    double s = rhs[i];
    for (int k = 0; k < i; ++k) s -= M[i * n + k] * dx[k];
    dx[i] = s / M[i * n + i];
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = dx[i];
    for (int k = i + 1; k < n; ++k) s -= M[k * n + i] * dx[k];
    dx[i] = s / M[i * n + i];
  }
  return true;
}

__global__ void __launch_bounds__(kFitThreads) k_bath_fit(BathFitArgs A) {
  extern __shared__ __align__(16) unsigned char fit_smem[];
  FitShared& S = *reinterpret_cast<FitShared*>(fit_smem);
  const int inst = blockIdx.x, np = A.npar, tid = threadIdx.x;
  if (tid == 0) {
    const size_t head = (sizeof(FitShared) + 15) & ~(size_t)15;
    S.R = reinterpret_cast<double2*>(fit_smem + head);
    S.gb = S.R + (size_t)A.fc * A.ns * A.ns;
    S.T = S.gb + (size_t)A.fc * A.nb;
  }
  for (int q = tid; q < A.nent; q += blockDim.x) {
    S.ep[q] = A.ent_par[q];
    S.ek[q] = A.ent_kind[q];
    S.ei[q] = A.ent_i[q];
    S.ej[q] = A.ent_j[q];
    S.ev[q] = A.ent_val[q];
  }
  for (int p = tid; p < np; p += blockDim.x) S.x[p] = A.x[(size_t)inst * np + p];
  __syncthreads();
  fit_blocks(S, A, inst, S.x);
  double cost = fit_normal(S, A, inst);
  if (tid == 0) {
    double dmax = 0.0;
    for (int p = 0; p < np; ++p) dmax = fmax(dmax, S.A[p * np + p]);
    S.lambda = 1e-3 * dmax;
    S.nu = 2.0;
    S.cost = cost;
    S.done = 0;
    S.flag = 0;
    S.it = 0;
  }
  __syncthreads();
  for (int it = 0; it < A.max_iter; ++it) {
    if (tid == 0) {
      S.it = it + 1;
      double gmax = 0.0;
      for (int p = 0; p < np; ++p) gmax = fmax(gmax, fabs(S.g[p]));
      if (gmax < A.gtol) {
        S.done = 1;
        S.flag = 3;
      } else {
        // damped normal equations (A + lambda diag A) dx = -g, with a
        // floor on the scaling for parameters the residuals do not see
        bool ok = false;
        for (int tries = 0; tries < 40 && !ok; ++tries) {
          for (int i = 0; i < np * np; ++i) S.M[i] = S.A[i];
          for (int p = 0; p < np; ++p) {
            S.M[p * np + p] += S.lambda * fmax(S.A[p * np + p], 1e-300);
            S.rhs[p] = -S.g[p];
          }
          ok = fit_cholesky_solve(S.M, S.rhs, S.dx, np);
          if (!ok) S.lambda *= 10.0;
        }
        if (!ok) {
          S.done = 1;
          S.flag = -1;
        } else {
          double nx = 0.0, ndx = 0.0;
          for (int p = 0; p < np; ++p) {
            nx += S.x[p] * S.x[p];
            ndx += S.dx[p] * S.dx[p];
            S.xn[p] = S.x[p] + S.dx[p];
          }
          if (sqrt(ndx) < A.xtol * (A.xtol + sqrt(nx))) {
            S.done = 1;
            S.flag = 2;
          }
        }
      }
    }
    __syncthreads();
    if (S.done) break;
    fit_blocks(S, A, inst, S.xn);
    const double cost_new = fit_cost(S, A, inst);
    if (tid == 0) {
      // gain ratio against the damped linear model's predicted decrease
      double pred = 0.0;
      for (int p = 0; p < np; ++p)
        pred += S.dx[p] * (S.lambda * fmax(S.A[p * np + p], 1e-300) * S.dx[p] - S.g[p]);
      pred *= 0.5;
      const double rho = pred > 0.0 ? (S.cost - cost_new) / pred : -1.0;
      if (rho > 0.0) {
        // the cost test counts only well-predicted steps (gain ratio above
        // 1/4), as the reference's solver does: a heavily damped tiny step
        // is not convergence
        S.flag = ((S.cost - cost_new) < A.ftol * S.cost && rho > 0.25) ? 1 : 0;
        for (int p = 0; p < np; ++p) S.x[p] = S.xn[p];
        const double t = 2.0 * rho - 1.0;
        S.lambda *= fmax(1.0 / 3.0, 1.0 - t * t * t);
        S.nu = 2.0;
        S.accepted = 1.0;
      } else {
        S.lambda *= S.nu;
        S.nu *= 2.0;
        S.accepted = 0.0;
      }
    }
    __syncthreads();
    if (S.accepted > 0.5) {
      fit_blocks(S, A, inst, S.x);  // the accepted point
      cost = fit_normal(S, A, inst);
      if (tid == 0) {
        S.cost = cost;
        if (S.flag == 1) S.done = 1;
      }
      __syncthreads();
      if (S.done) break;
    }
  }
  // With ftol = 0 the caller asks for convergence on the gradient: at a
  // large-residual minimum the cost's rounding hides the last decreases the
  // damped steps could verify, so finish with exact Gauss-Newton steps
  // (A dx = -g) for as long as the largest gradient component decreases.
  if (A.ftol == 0.0 && S.done && S.flag != -1 && S.flag != 3) {
    for (int k = 0; k < 64; ++k) {
      if (tid == 0) {
        double gmax = 0.0;
        for (int p = 0; p < np; ++p) gmax = fmax(gmax, fabs(S.g[p]));
        S.lambda = gmax;  // reused: the gradient before the step
        for (int i = 0; i < np * np; ++i) S.M[i] = S.A[i];
        for (int p = 0; p < np; ++p) S.rhs[p] = -S.g[p];
        S.accepted = (gmax >= A.gtol && fit_cholesky_solve(S.M, S.rhs, S.dx, np)) ? 1.0 : 0.0;
        if (S.accepted > 0.5)
          for (int p = 0; p < np; ++p) S.xn[p] = S.x[p] + S.dx[p];
      }
      __syncthreads();
      if (S.accepted < 0.5) break;
      fit_blocks(S, A, inst, S.xn);
      const double cn = fit_normal(S, A, inst);  // A, g at the candidate
      if (tid == 0) {
        double gmax = 0.0;
        for (int p = 0; p < np; ++p) gmax = fmax(gmax, fabs(S.g[p]));
        if (gmax < S.lambda) {
          for (int p = 0; p < np; ++p) S.x[p] = S.xn[p];
          S.cost = cn;
          S.accepted = 1.0;
          if (gmax < A.gtol) S.flag = 3;
        } else {
          S.accepted = 0.0;
        }
      }
      __syncthreads();
      if (S.accepted < 0.5) {
        fit_blocks(S, A, inst, S.x);  // back to the last accepted point
        cost = fit_normal(S, A, inst);
        break;
      }
      if (S.flag == 3) break;
    }
  }
  if (tid == 0) {
    for (int p = 0; p < np; ++p) A.x[(size_t)inst * np + p] = S.x[p];
    A.cost[inst] = S.cost;
    A.iters[inst] = S.it;
    A.status[inst] = S.done ? S.flag : 0;
  }
}

// Buffers and stream of the calling host thread on one device, kept across
// calls: a fit allocates nothing after its first call of a given size, and
// runs on a non-blocking stream of its own, so fits of concurrent CDMFT
// loops (one host thread each) neither synchronize the device through
// cudaFree nor wait for each other's kernels.
struct FitContext {
  cudaStream_t s = nullptr;
  DevBuf<double> w, wt, host, v, th, e, x, cost;
  DevBuf<int> p, k, i, j, it, st;
  ~FitContext() {
    if (s) cudaStreamDestroy(s);
  }
};

static FitContext& fit_context(int device) {
  static thread_local std::map<int, std::unique_ptr<FitContext>> ctx;
  auto& c = ctx[device];
  if (!c) {
    c.reset(new FitContext);
    QCMG_CUDA(cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking));
  }
  return *c;
}

}  // namespace qcmg

using namespace qcmg;

extern "C" int qcmg_bath_fit(int n_inst, int ns, int nb, int nw, const double* w,
                             const double* weights, const double* host, int npar, int nent,
                             const int* ent_par, const int* ent_kind, const int* ent_i,
                             const int* ent_j, const double* ent_val, const double* theta0,
                             const double* e0, double* x, int max_iter, double xtol, double ftol,
                             double gtol, double* cost, int* iters, int* status) {
  try {
    clear_error();
    QCMG_CHECK_ARG(n_inst >= 0, "n_inst must not be negative");
    if (n_inst == 0) return QCMG_OK;
    QCMG_CHECK_ARG(ns >= 1 && ns <= kFitMaxSites, "1 <= n_sites <= 8");
    QCMG_CHECK_ARG(nb >= 1 && nb <= kFitMaxBath, "1 <= n_bath <= 16");
    QCMG_CHECK_ARG(npar >= 1 && npar <= kFitMaxPar, "1 <= n_par <= 32");
    QCMG_CHECK_ARG(nent >= 1 && nent <= kFitMaxEnt, "1 <= n_entries <= 128");
    QCMG_CHECK_ARG(nw >= 1, "at least one frequency");
    QCMG_CHECK_ARG(max_iter >= 0, "max_iter must not be negative");
    QCMG_CHECK_ARG(w && weights && host && ent_par && ent_kind && ent_i && ent_j && ent_val &&
                       theta0 && e0 && x && cost && iters && status,
                   "NULL argument");
    for (int q = 0; q < nent; ++q) {
      QCMG_CHECK_ARG(ent_par[q] >= 0 && ent_par[q] < npar, "entry parameter out of range");
      QCMG_CHECK_ARG(ent_kind[q] == 0 || ent_kind[q] == 1, "entry kind must be 0 (theta) or 1 (E)");
      QCMG_CHECK_ARG(ent_j[q] >= 0 && ent_j[q] < nb, "entry bath index out of range");
      QCMG_CHECK_ARG(ent_kind[q] == 1 || (ent_i[q] >= 0 && ent_i[q] < ns),
                     "entry site index out of range");
      QCMG_CHECK_ARG(ent_kind[q] == 0 || ent_i[q] == ent_j[q],
                     "bath-energy entries must be diagonal (the device fit takes a diagonal E)");
    }
    const size_t n2 = (size_t)ns * ns;
    int device = 0;
    QCMG_CUDA(cudaGetDevice(&device));
    FitContext& C = fit_context(device);
    cudaStream_t st = C.s;
    C.w.upload(w, nw, st);
    C.wt.upload(weights, nw, st);
    C.host.upload(host, (size_t)n_inst * nw * n2 * 2, st);
    C.p.upload(ent_par, nent, st);
    C.k.upload(ent_kind, nent, st);
    C.i.upload(ent_i, nent, st);
    C.j.upload(ent_j, nent, st);
    C.v.upload(ent_val, nent, st);
    C.th.upload(theta0, (size_t)n_inst * ns * nb, st);
    C.e.upload(e0, (size_t)n_inst * nb, st);
    C.x.upload(x, (size_t)n_inst * npar, st);
    C.cost.alloc(n_inst);
    C.it.alloc(n_inst);
    C.st.alloc(n_inst);
    BathFitArgs a;
    a.ns = ns;
    a.nb = nb;
    a.nw = nw;
    a.npar = npar;
    a.nent = nent;
    a.w = C.w.p;
    a.wt = C.wt.p;
    a.host = C.host.p;
    a.ent_par = C.p.p;
    a.ent_kind = C.k.p;
    a.ent_i = C.i.p;
    a.ent_j = C.j.p;
    a.ent_val = C.v.p;
    a.theta0 = C.th.p;
    a.e0 = C.e.p;
    a.x = C.x.p;
    a.max_iter = max_iter;
    a.xtol = xtol;
    a.ftol = ftol;
    a.gtol = gtol;
    a.cost = C.cost.p;
    a.iters = C.it.p;
    a.status = C.st.p;
    // frequencies per chunk of residuals
    const size_t per_f = (n2 + (size_t)nb) * sizeof(double2);
    a.fc = kFitMaxChunk;
    const size_t smem = ((sizeof(FitShared) + 15) & ~(size_t)15) + (size_t)a.fc * per_f +
                        3 * (size_t)nb * nb * sizeof(double2);
    QCMG_CUDA(cudaFuncSetAttribute(k_bath_fit, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_bath_fit<<<n_inst, kFitThreads, smem, st>>>(a);
    QCMG_CUDA(cudaGetLastError());
    QCMG_CUDA(cudaMemcpyAsync(x, C.x.p, (size_t)n_inst * npar * 8, cudaMemcpyDeviceToHost, st));
    QCMG_CUDA(cudaMemcpyAsync(cost, C.cost.p, (size_t)n_inst * 8, cudaMemcpyDeviceToHost, st));
    QCMG_CUDA(cudaMemcpyAsync(iters, C.it.p, (size_t)n_inst * 4, cudaMemcpyDeviceToHost, st));
    QCMG_CUDA(cudaMemcpyAsync(status, C.st.p, (size_t)n_inst * 4, cudaMemcpyDeviceToHost, st));
    QCMG_CUDA(cudaStreamSynchronize(st));
    return QCMG_OK;
  } catch (const Error& e) {
    set_error(e.what());
    return e.code;
  } catch (const std::exception& e) {
    set_error(e.what());
    return QCMG_ERR_CUDA;
  }
}
