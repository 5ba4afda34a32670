// Krylov solvers on device-resident vectors: Lanczos ground state (with an
// optional fully reorthogonalized variant) and Freund's band Lanczos.
// The host keeps only the scalars (alpha, beta, the projected matrix) and the
// control flow; every length-dim vector stays in HBM.
#include <cusolverDn.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <random>

#include "qcmg_blas.h"
#include "qcmg_fxpath.h"
#include "qcmg_internal.h"
#include "qcmg_krylov.h"
#include "qcmg_tridiag.h"

namespace qcmg {

// ---------------------------------------------------------------------------
// multi-vector kernels used by reorthogonalization and band Lanczos

constexpr int kTile = 2048;  // elements of w staged per block iteration

// Vector lists and coefficients passed to the kernels by value (up to
// kByValue entries): no host-to-device copy of a pointer array per call,
// which on small sectors costs more than the kernel.  Longer lists go
// through device arrays (the same kernels, instantiated on pointers).
constexpr int kByValue = 64;
struct VecList {
  const double* v[kByValue];
  __device__ const double* operator[](int k) const { return v[k]; }
};
struct MutVecList {
  double* v[kByValue];
  __device__ double* operator[](int k) const { return v[k]; }
};
struct CoefList {
  double c[kByValue];
  __device__ double operator[](int k) const { return c[k]; }
};

// part[b*m + k] = sum over block b's tiles of V_k . w
template <class VL>
__global__ void __launch_bounds__(256) k_multidot(VL V, int m, const double* __restrict__ w,
                                                  size_t n, double* __restrict__ part) {
  __shared__ double ws[kTile];
  extern __shared__ double acc[];  // m accumulators
  for (int k = threadIdx.x; k < m; k += blockDim.x) acc[k] = 0.0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  for (size_t base = (size_t)blockIdx.x * kTile; base < n; base += (size_t)gridDim.x * kTile) {
    const size_t len = min((size_t)kTile, n - base);
    __syncthreads();
    for (size_t i = threadIdx.x; i < len; i += blockDim.x) ws[i] = w[base + i];
    __syncthreads();
    for (int k = warp; k < m; k += nwarp) {
      const double* vk = V[k] + base;
      double s = 0.0;
      for (size_t i = lane; i < len; i += 32) s = fma(vk[i], ws[i], s);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) acc[k] += s;  // warp k%nwarp owns acc[k]: no race
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < m; k += blockDim.x) part[(size_t)blockIdx.x * m + k] = acc[k];
}

// The same partials for short lists, accumulated in registers: each thread
// keeps m sums over its elements, so an element costs one load of w and m
// independent loads and FMAs (no dependent chain per vector, no staging
// barrier), and the block then reduces each sum in a fixed order.
template <int MAXM>
__global__ void __launch_bounds__(256) k_multidot_reg(VecList V, int m,
                                                      const double* __restrict__ w, size_t n,
                                                      double* __restrict__ part) {
  double acc[MAXM];
#pragma unroll
  for (int k = 0; k < MAXM; ++k) acc[k] = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const double wi = w[i];
#pragma unroll
    for (int k = 0; k < MAXM; ++k)
      if (k < m) acc[k] = fma(V[k][i], wi, acc[k]);
  }
  __shared__ double red[8][MAXM];  // one row per warp of the 256-thread block
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < MAXM; ++k) {
    double v = acc[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[wp][k] = v;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < m; k += blockDim.x) {
    double t = 0.0;
    for (int q = 0; q < 8; ++q) t += red[q][k];
    part[(size_t)blockIdx.x * m + k] = t;
  }
}

// out[k] = sum_b part[b*m + k], fixed order.
__global__ void k_multidot_final(const double* __restrict__ part, int nb, int m,
                                 double* __restrict__ out) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int b = 0; b < nb; ++b) s += part[(size_t)b * m + k];
    out[k] = s;
  }
}

// w -= sum_k c_k V_k
template <class VL, class CL>
__global__ void __launch_bounds__(256) k_multiaxpy(VL V, int m, CL c, double* __restrict__ w,
                                                   size_t n) {
  extern __shared__ double cs[];
  for (int k = threadIdx.x; k < m; k += blockDim.x) cs[k] = c[k];
  __syncthreads();
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    double s = w[i];
    for (int k = 0; k < m; ++k) s = fma(-cs[k], V[k][i], s);
    w[i] = s;
  }
}

// v <- sc * v, then V_k <- V_k - c_k * v for k < m (the scaled v): one pass
// over v for the whole Gram-Schmidt sweep of a band-Lanczos step.
template <class VL, class CL>
__global__ void __launch_bounds__(256) k_scale_sub(double* __restrict__ v, double sc, VL V, CL c,
                                                   int m, size_t n) {
  extern __shared__ double cs[];
  for (int k = threadIdx.x; k < m; k += blockDim.x) cs[k] = c[k];
  __syncthreads();
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const double x = v[i] * sc;
    v[i] = x;
    for (int k = 0; k < m; ++k) V[k][i] = fma(-cs[k], x, V[k][i]);
  }
}

// Fixed-order block sum; the result is valid in thread 0.
__device__ __forceinline__ double block_sum_fixed(double v) {
  __shared__ double ws[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) ws[w] = v;
  __syncthreads();
  v = (threadIdx.x < (blockDim.x >> 5)) ? ws[threadIdx.x] : 0.0;
  if (w == 0) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  }
  return v;
}

// w -= sum_k c_k V_k (the band recurrence), then one partial of w . u per
// block for the closing Gram-Schmidt step against u = v_j.
template <class VL, class CL>
__global__ void __launch_bounds__(256) k_multiaxpy_dot(VL V, int m, CL c, double* __restrict__ w,
                                                       const double* __restrict__ u, size_t n,
                                                       double* __restrict__ part) {
  extern __shared__ double cs[];
  for (int k = threadIdx.x; k < m; k += blockDim.x) cs[k] = c[k];
  __syncthreads();
  double d = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    double s = w[i];
    for (int k = 0; k < m; ++k) s = fma(-cs[k], V[k][i], s);
    w[i] = s;
    d = fma(s, u[i], d);
  }
  d = block_sum_fixed(d);
  if (threadIdx.x == 0) part[blockIdx.x] = d;
}

// Every block sums the nb partials in the same fixed order (so all agree on
// the dot), then w -= dot * u; block 0 also stores the dot at dot_out.
__global__ void __launch_bounds__(256) k_dot_axpy(const double* __restrict__ part, int nb,
                                                  const double* __restrict__ u,
                                                  double* __restrict__ w, size_t n,
                                                  double* __restrict__ dot_out) {
  __shared__ double total;
  double t = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) t += part[b];
  t = block_sum_fixed(t);
  if (threadIdx.x == 0) {
    total = t;
    if (blockIdx.x == 0) *dot_out = t;
  }
  __syncthreads();
  const double cdot = -total;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    w[i] = fma(cdot, u[i], w[i]);
}

// Block count of a multi-dot over n elements (fixed: deterministic order).
int multidot_blocks(size_t n) {
  return (int)std::max<size_t>(1, std::min<size_t>((n + kTile - 1) / kTile, 2 * 152));
}

// Launches the two kernels of a multi-dot: part (m x nblocks doubles) is
// scratch, every element of it read by the second kernel is first written
// by the first; out (m doubles, device) receives the result.
void multidot_launch(int m, const double* const* V, const double* w, size_t n, double* part,
                     double* out, cudaStream_t s) {
  const int nb = multidot_blocks(n);
  k_multidot<const double* const*><<<nb, 256, m * sizeof(double), s>>>(V, m, w, n, part);
  k_multidot_final<<<(m + 127) / 128, 128, 0, s>>>(part, nb, m, out);
  QCMG_CUDA(cudaGetLastError());
}

struct MultiOps {
  DevBuf<const double*> ptrs;
  DevBuf<double> part, coef;
  std::vector<double> host;
  int nblocks = 0;
  void multidot(const std::vector<const double*>& V, const double* w, size_t n, cudaStream_t s,
                std::vector<double>& out) {
    const int m = (int)V.size();
    out.assign(m, 0.0);
    if (m == 0) return;
    nblocks = multidot_blocks(n);
    if (m <= 32) {
      // register accumulators: 256-thread blocks, two per SM at most
      nblocks = (int)std::max<size_t>(1, std::min<size_t>((n + 255) / 256, 2 * 152));
      part.alloc((size_t)nblocks * m);
      VecList L;
      for (int k = 0; k < m; ++k) L.v[k] = V[k];
      if (m <= 4)
        k_multidot_reg<4><<<nblocks, 256, 0, s>>>(L, m, w, n, part.p);
      else if (m <= 8)
        k_multidot_reg<8><<<nblocks, 256, 0, s>>>(L, m, w, n, part.p);
      else if (m <= 16)
        k_multidot_reg<16><<<nblocks, 256, 0, s>>>(L, m, w, n, part.p);
      else
        k_multidot_reg<32><<<nblocks, 256, 0, s>>>(L, m, w, n, part.p);
    } else if (m <= kByValue) {
      part.alloc((size_t)nblocks * m);
      VecList L;
      for (int k = 0; k < m; ++k) L.v[k] = V[k];
      k_multidot<VecList><<<nblocks, 256, m * sizeof(double), s>>>(L, m, w, n, part.p);
    } else {
      part.alloc((size_t)nblocks * m);
      ptrs.alloc(m);
      QCMG_CUDA(cudaMemcpyAsync(ptrs.p, V.data(), m * sizeof(double*), cudaMemcpyHostToDevice, s));
      k_multidot<const double* const*>
          <<<nblocks, 256, m * sizeof(double), s>>>(ptrs.p, m, w, n, part.p);
    }
    QCMG_CUDA(cudaGetLastError());
    // the partials come back and are summed here in k_multidot_final's order
    // (one launch fewer per call; the sums are bitwise the same)
    host.resize((size_t)nblocks * m);
    QCMG_CUDA(cudaMemcpyAsync(host.data(), part.p, host.size() * sizeof(double),
                              cudaMemcpyDeviceToHost, s));
    QCMG_CUDA(cudaStreamSynchronize(s));
    for (int k = 0; k < m; ++k) {
      double acc = 0.0;
      for (int b = 0; b < nblocks; ++b) acc += host[(size_t)b * m + k];
      out[k] = acc;
    }
  }
  // w -= sum_k c_k V_k, then d = w . u and w -= d u with d left at d_dev:
  // two launches.  False (nothing done) for lists longer than kByValue.
  DevBuf<double> opart;
  bool multiaxpy_orth(const std::vector<const double*>& V, const std::vector<double>& c,
                      double* w, const double* u, size_t n, double* d_dev, cudaStream_t s) {
    const int m = (int)V.size();
    if (m > kByValue || n == 0) return false;
    VecList L;
    CoefList C;
    for (int k = 0; k < m; ++k) {
      L.v[k] = V[k];
      C.c[k] = c[k];
    }
    const unsigned g = elementwise_grid(n);
    opart.alloc(g);
    k_multiaxpy_dot<VecList, CoefList>
        <<<g, 256, std::max(m, 1) * sizeof(double), s>>>(L, m, C, w, u, n, opart.p);
    k_dot_axpy<<<g, 256, 0, s>>>(opart.p, (int)g, u, w, n, d_dev);
    QCMG_CUDA(cudaGetLastError());
    return true;
  }
  static unsigned elementwise_grid(size_t n) {
    return (unsigned)std::max<size_t>(1, std::min<size_t>((n + 255) / 256, 152 * 8));
  }
  void multiaxpy(const std::vector<const double*>& V, const std::vector<double>& c, double* w,
                 size_t n, cudaStream_t s) {
    const int m = (int)V.size();
    if (m == 0 || n == 0) return;
    if (m <= kByValue) {
      VecList L;
      CoefList C;
      for (int k = 0; k < m; ++k) {
        L.v[k] = V[k];
        C.c[k] = c[k];
      }
      k_multiaxpy<VecList, CoefList>
          <<<elementwise_grid(n), 256, m * sizeof(double), s>>>(L, m, C, w, n);
    } else {
      ptrs.alloc(m);
      coef.alloc(m);
      QCMG_CUDA(cudaMemcpyAsync(ptrs.p, V.data(), m * sizeof(double*), cudaMemcpyHostToDevice, s));
      QCMG_CUDA(cudaMemcpyAsync(coef.p, c.data(), m * sizeof(double), cudaMemcpyHostToDevice, s));
      k_multiaxpy<const double* const*, const double*>
          <<<elementwise_grid(n), 256, m * sizeof(double), s>>>(ptrs.p, m, coef.p, w, n);
    }
    QCMG_CUDA(cudaGetLastError());
  }
  // v <- sc v;  V_k <- V_k - c_k v  (k_scale_sub)
  DevBuf<double*> wptrs;
  DevBuf<double> wcoef;
  void scale_sub(double* v, double sc, const std::vector<double*>& V, const std::vector<double>& c,
                 size_t n, cudaStream_t s) {
    const int m = (int)V.size();
    if (n == 0) return;
    const size_t sh = std::max(m, 1) * sizeof(double);
    if (m <= kByValue) {
      MutVecList L;
      CoefList C;
      for (int k = 0; k < m; ++k) {
        L.v[k] = V[k];
        C.c[k] = c[k];
      }
      k_scale_sub<MutVecList, CoefList><<<elementwise_grid(n), 256, sh, s>>>(v, sc, L, C, m, n);
    } else {
      wptrs.alloc(m);
      wcoef.alloc(m);
      QCMG_CUDA(cudaMemcpyAsync(wptrs.p, V.data(), m * sizeof(double*), cudaMemcpyHostToDevice, s));
      QCMG_CUDA(cudaMemcpyAsync(wcoef.p, c.data(), m * sizeof(double), cudaMemcpyHostToDevice, s));
      k_scale_sub<double* const*, const double*>
          <<<elementwise_grid(n), 256, sh, s>>>(v, sc, wptrs.p, wcoef.p, m, n);
    }
    QCMG_CUDA(cudaGetLastError());
  }
};

// ---------------------------------------------------------------------------

void seeded_vector(size_t dim, unsigned seed, double* out) {
  std::normal_distribution<double> dist(0.0, 1.0);
  std::default_random_engine gen(seed);
  double s = 0.0;
  for (size_t i = 0; i < dim; ++i) {
    out[i] = dist(gen);
    s += out[i] * out[i];
  }
  s = 1.0 / std::sqrt(s);
  for (size_t i = 0; i < dim; ++i) out[i] *= s;
}

static void dalloc(double** p, size_t n) { QCMG_CUDA(cudaMalloc(p, std::max<size_t>(n, 1) * 8)); }

struct DevVec {
  double* p = nullptr;
  DevVec() = default;
  explicit DevVec(size_t n) { dalloc(&p, n); }
  DevVec(const DevVec&) = delete;
  DevVec(DevVec&& o) noexcept : p(o.p) { o.p = nullptr; }
  ~DevVec() {
    if (p) cudaFree(p);
  }
};

// CUDA events for the per-solve device-time breakdown.
struct Events {
  cudaEvent_t e[4] = {nullptr, nullptr, nullptr, nullptr};
  Events() {
    for (auto& x : e) QCMG_CUDA(cudaEventCreate(&x));
  }
  ~Events() {
    for (auto& x : e)
      if (x) cudaEventDestroy(x);
  }
  void record(int k, cudaStream_t s) { QCMG_CUDA(cudaEventRecord(e[k], s)); }
  double elapsed(int a, int b) const {  // both recorded and complete
    float ms = 0.0f;
    QCMG_CUDA(cudaEventElapsedTime(&ms, e[a], e[b]));
    return ms;
  }
};

LanczosResult lanczos_ground_state(qcmg_hamiltonian* H, const double* x0_host, unsigned seed,
                                   double tol, int max_iter, int reorth, double* psi_host) {
  const size_t n = H->dim;
  cudaStream_t s = H->stream;
  LanczosResult res;
  QCMG_CHECK_ARG(n > 0, "empty sector");
  // Start vector: the caller's, or the seeded one.  The seeded vector is
  // generated on the host (the reference's sequential std::normal_distribution
  // stream, bit for bit) and kept on the device per handle, so repeated solves
  // of a sector (VCA / CDMFT loops) generate it once.
  DevVec x0_own(x0_host ? n : 1);
  const double* x0_dev = nullptr;
  if (!x0_host) {
    if (!(H->seed_ok && H->seed_key == seed && H->seed_vec.n == n)) {
      H->seed_ok = false;
      std::vector<double> hx0(n);
      seeded_vector(n, seed, hx0.data());
      H->seed_vec.upload(hx0.data(), n, s);
      QCMG_CUDA(cudaStreamSynchronize(s));  // hx0 goes out of scope
      H->seed_key = seed;
      H->seed_ok = true;
    }
    x0_dev = H->seed_vec.p;
  } else {
    QCMG_CUDA(cudaMemcpyAsync(x0_own.p, x0_host, n * 8, cudaMemcpyHostToDevice, s));
    x0_dev = x0_own.p;
  }
  if (reorth <= 0 && H->use_fx && fx_prepare(H)) {
    // fixed-point fast path (one hop magnitude per spin)
    DevVec psi_dev(psi_host ? n : 1);
    LanczosResult fr = fx_lanczos(H, x0_dev, tol, max_iter, psi_host ? psi_dev.p : nullptr);
    if (psi_host) {
      QCMG_CUDA(cudaMemcpyAsync(psi_host, psi_dev.p, n * 8, cudaMemcpyDeviceToHost, s));
      QCMG_CUDA(cudaStreamSynchronize(s));
    }
    return fr;
  }
  DevVec r(n), q(n);
  QCMG_CUDA(cudaMemcpyAsync(r.p, x0_dev, n * 8, cudaMemcpyDeviceToDevice, s));
  QCMG_CUDA(cudaMemsetAsync(q.p, 0, n * 8, s));
  Reducer red;
  std::vector<double> z;
  double* rp = r.p;
  double* qp = q.p;

  if (reorth <= 0) {
    // Three-term recurrence of LanczosEigenvalue (Lanczos.hpp:64-93).
    double ritz = 2.0 * tol;
    while (ritz > tol) {
      if (!res.beta.empty()) scale2(rp, 1.0 / res.beta.back(), qp, -res.beta.back(), n, s);
      matvec(H, rp, qp, true);
      std::swap(rp, qp);
      double a = red.dot(qp, rp, n, s);
      res.alpha.push_back(a);
      double b2 = red.axpy_norm2(rp, qp, a, n, s);
      res.beta.push_back(std::sqrt(b2));
      res.energy = tridiag_lowest(res.alpha, res.beta, z);
      ritz = std::fabs(z.back() * res.beta.back());
      if (!std::isfinite(res.energy) || !std::isfinite(ritz))
        throw Error(QCMG_ERR_NUMERIC, "Lanczos produced a non-finite value");
      if ((int)res.alpha.size() > max_iter)
        throw Error(QCMG_ERR_NOCONV,
                    "Lanczos procedure exceeded " + std::to_string(max_iter) + " iterations");
    }
    res.niter = (int)res.alpha.size();
    if (psi_host) {
      // Eigenvector replay of LanczosEigenvector (Lanczos.hpp:109-131).
      DevVec gs(n);
      QCMG_CUDA(cudaMemcpyAsync(gs.p, x0_dev, n * 8, cudaMemcpyDeviceToDevice, s));
      scale(gs.p, z[0], n, s);
      QCMG_CUDA(cudaMemcpyAsync(r.p, x0_dev, n * 8, cudaMemcpyDeviceToDevice, s));
      QCMG_CUDA(cudaMemsetAsync(q.p, 0, n * 8, s));
      for (size_t j = 1; j < z.size(); ++j) {
        matvec(H, r.p, q.p, true);
        replay_step(r.p, q.p, gs.p, res.alpha[j - 1], res.beta[j - 1], z[j], n, s);
      }
      QCMG_CUDA(cudaMemcpyAsync(psi_host, gs.p, n * 8, cudaMemcpyDeviceToHost, s));
      QCMG_CUDA(cudaStreamSynchronize(s));
    }
    return res;
  }

  // Fully reorthogonalized Lanczos: the basis is kept in HBM and every new
  // residual is projected out of it twice (classical Gram-Schmidt x2).  At
  // most `reorth` vectors are kept: when the cap is reached before the Ritz
  // residual converges, the iteration restarts from the current Ritz vector
  // (explicit restart).  The product is the fixed-point one where it applies
  // (the vectors stay FP64).  Device time of the products and of the
  // reorthogonalization is recorded with events (qcmg_lanczos_last_stats).
  const bool fx = H->use_fx && fx_prepare(H);
  auto product = [&](const double* x, double* y) {
    if (fx)
      fx_matvec_f64(H, x, y, false);
    else
      matvec(H, x, y, false);
  };
  const int keep = std::max(reorth, 2);
  std::vector<DevVec> V;  // pool, reused across restarts
  std::vector<const double*> Vp;
  MultiOps mops;
  std::vector<double> c;
  V.emplace_back(n);
  QCMG_CUDA(cudaMemcpyAsync(V[0].p, x0_dev, n * 8, cudaMemcpyDeviceToDevice, s));
  double* w = r.p;  // residual
  Events ev;
  int total = 0;
  bool converged = false;
  while (!converged) {
    Vp.assign(1, V[0].p);
    res.alpha.clear();
    res.beta.clear();
    for (int j = 0;; ++j) {
      ev.record(0, s);
      product(V[j].p, w);
      ev.record(1, s);
      if (j > 0) axpy(w, V[j - 1].p, -res.beta.back(), n, s);
      double a = red.dot(V[j].p, w, n, s);
      res.alpha.push_back(a);
      axpy(w, V[j].p, -a, n, s);
      ev.record(2, s);
      for (int pass = 0; pass < 2; ++pass) {
        mops.multidot(Vp, w, n, s, c);
        mops.multiaxpy(Vp, c, w, n, s);
      }
      ev.record(3, s);
      double b = std::sqrt(red.dot(w, w, n, s));  // synchronizes the stream
      res.product_ms += ev.elapsed(0, 1);
      res.reorth_ms += ev.elapsed(2, 3);
      res.reorth_bytes += 2.0 * 16.0 * (double)Vp.size() * (double)n;  // 16 B per stored element per pass
      res.beta.push_back(b);
      ++total;
      res.energy = tridiag_lowest(res.alpha, res.beta, z);
      const double ritz = std::fabs(z.back() * b);
      if (!std::isfinite(res.energy) || !std::isfinite(ritz))
        throw Error(QCMG_ERR_NUMERIC, "Lanczos produced a non-finite value");
      if (ritz <= tol || b == 0.0) {
        converged = true;
        break;
      }
      if (total >= max_iter)
        throw Error(QCMG_ERR_NOCONV, "reorthogonalized Lanczos did not converge within " +
                                         std::to_string(max_iter) + " iterations");
      if ((int)Vp.size() >= keep) break;  // cap reached: restart
      if ((int)V.size() <= j + 1) V.emplace_back(n);
      QCMG_CUDA(cudaMemcpyAsync(V[j + 1].p, w, n * 8, cudaMemcpyDeviceToDevice, s));
      scale(V[j + 1].p, 1.0 / b, n, s);
      Vp.push_back(V[j + 1].p);
    }
    if (converged) break;
    // restart from the Ritz vector sum_k z_k V_k, normalized
    QCMG_CUDA(cudaMemsetAsync(w, 0, n * 8, s));
    std::vector<double> mz(z.size());
    for (size_t k = 0; k < z.size(); ++k) mz[k] = -z[k];
    mops.multiaxpy(Vp, mz, w, n, s);
    const double nrm = std::sqrt(red.dot(w, w, n, s));
    if (!(nrm > 0.0)) throw Error(QCMG_ERR_NUMERIC, "Lanczos restart vector vanished");
    QCMG_CUDA(cudaMemcpyAsync(V[0].p, w, n * 8, cudaMemcpyDeviceToDevice, s));
    scale(V[0].p, 1.0 / nrm, n, s);
    ++res.restarts;
  }
  res.niter = total;
  res.vectors = (int)V.size();
  if (psi_host) {
    DevVec gs(n);
    QCMG_CUDA(cudaMemsetAsync(gs.p, 0, n * 8, s));
    std::vector<const double*> Vz(Vp.begin(), Vp.begin() + z.size());
    std::vector<double> mz(z.size());
    for (size_t k = 0; k < z.size(); ++k) mz[k] = -z[k];
    mops.multiaxpy(Vz, mz, gs.p, n, s);
    QCMG_CUDA(cudaMemcpyAsync(psi_host, gs.p, n * 8, cudaMemcpyDeviceToHost, s));
    QCMG_CUDA(cudaStreamSynchronize(s));
  }
  return res;
}

// ---------------------------------------------------------------------------
// Band Lanczos (Freund), as in src_ed/Hamiltonian/Lanczos.hpp:214-395.

struct Cusolver {
  cusolverDnHandle_t h = nullptr;
  DevBuf<double> A, W, work;
  DevBuf<int> info;
  ~Cusolver() {
    if (h) cusolverDnDestroy(h);
  }
  // Eigen-decomposition of the leading j x j block of column-major t (ld).
  void syevd(const std::vector<double>& t, int ld, int j, bool vectors, cudaStream_t s,
             std::vector<double>& evals, std::vector<double>* U) {
    if (!h) {
      if (cusolverDnCreate(&h) != CUSOLVER_STATUS_SUCCESS)
        throw Error(QCMG_ERR_CUDA, "cusolverDnCreate failed");
    }
    cusolverDnSetStream(h, s);
    std::vector<double> a((size_t)j * j);
    for (int c = 0; c < j; ++c)
      for (int r = 0; r < j; ++r) a[r + (size_t)j * c] = t[r + (size_t)ld * c];
    A.upload(a.data(), a.size(), s);
    W.alloc(j);
    info.alloc(1);
    auto jobz = vectors ? CUSOLVER_EIG_MODE_VECTOR : CUSOLVER_EIG_MODE_NOVECTOR;
    int lwork = 0;
    if (cusolverDnDsyevd_bufferSize(h, jobz, CUBLAS_FILL_MODE_LOWER, j, A.p, j, W.p, &lwork) !=
        CUSOLVER_STATUS_SUCCESS)
      throw Error(QCMG_ERR_CUDA, "cusolverDnDsyevd_bufferSize failed");
    work.alloc(std::max(lwork, 1));
    if (cusolverDnDsyevd(h, jobz, CUBLAS_FILL_MODE_LOWER, j, A.p, j, W.p, work.p, lwork,
                         info.p) != CUSOLVER_STATUS_SUCCESS)
      throw Error(QCMG_ERR_CUDA, "cusolverDnDsyevd failed");
    int hinfo = 0;
    evals.resize(j);
    QCMG_CUDA(cudaMemcpyAsync(&hinfo, info.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    QCMG_CUDA(cudaMemcpyAsync(evals.data(), W.p, j * 8, cudaMemcpyDeviceToHost, s));
    if (U) {
      U->resize((size_t)j * j);
      QCMG_CUDA(cudaMemcpyAsync(U->data(), A.p, (size_t)j * j * 8, cudaMemcpyDeviceToHost, s));
    }
    QCMG_CUDA(cudaStreamSynchronize(s));
    if (hinfo != 0) throw Error(QCMG_ERR_NUMERIC, "syevd did not converge");
  }
};

// LanczosGreen (src_ed/Hamiltonian/Lanczos.hpp:156-183): the three-term
// recurrence from a normalized start vector, on device vectors with the
// host keeping a and b; the reference's stopping rule (product of the b's
// or the last b at or below accur, or max_iter steps).
GreenResult lanczos_green(qcmg_hamiltonian* H, const double* psi0, bool on_device, double accur,
                          int max_iter) {
  const size_t n = H->dim;
  cudaStream_t s = H->stream;
  GreenResult out;
  out.b.push_back(1.0);
  if (n == 0) return out;
  DevVec P(n), Q(n);
  QCMG_CUDA(cudaMemcpyAsync(P.p, psi0, n * 8,
                            on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
  QCMG_CUDA(cudaMemsetAsync(Q.p, 0, n * 8, s));
  double* pp = P.p;  // psi
  double* qp = Q.p;  // q
  Reducer red;
  double prod = 1.0;
  while (prod > accur && std::fabs(out.b.back()) > accur && (int)out.a.size() < max_iter) {
    if (!out.a.empty()) {  // psi <- q / beta, q <- -beta psi
      const double beta = out.b.back();
      std::swap(pp, qp);
      scale2(pp, 1.0 / beta, qp, -beta, n, s);
    }
    matvec(H, pp, qp, true);  // q += H psi
    const double z = red.dot(pp, qp, n, s);
    out.a.push_back(z);
    const double zz = std::sqrt(red.axpy_norm2(qp, pp, z, n, s));  // q -= z psi
    if (!std::isfinite(z) || !std::isfinite(zz))
      throw Error(QCMG_ERR_NUMERIC, "continued-fraction Lanczos produced a non-finite value");
    out.b.push_back(zz);
    prod *= std::fabs(zz);
  }
  return out;
}

// Block Lanczos with Hermitian (polar) coupling blocks, the reference's
// default block method for matrix continued fractions (blockLanczosSVD,
// src_ed/Hamiltonian/Lanczos.hpp:603-790), preceded by the QR factor W of the
// start vectors that build_mcf extracts (model_instance.hpp:884-915).  All
// length-dim vectors stay on the device; the host holds the p x p blocks.
BlockResult block_lanczos(qcmg_hamiltonian* H, int p, const double* phi_in, bool on_device,
                          int M0, int max_iter, double acc_defl, double acc_band) {
  const size_t n = H->dim;
  cudaStream_t s = H->stream;
  BlockResult out;
  QCMG_CHECK_ARG(p > 0, "block Lanczos needs at least one start vector");
  if (n == 0) return out;
  Reducer red;
  MultiOps mops;
  std::vector<DevVec> store;
  std::vector<double*> q(p);
  for (int k = 0; k < p; ++k) {
    store.emplace_back(n);
    q[k] = store.back().p;
    QCMG_CUDA(cudaMemcpyAsync(q[k], phi_in + (size_t)k * n, n * 8,
                              on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
  }
  // modified Gram-Schmidt of the start block: phi[l] = sum_{k<=l} q[k] W(k,l);
  // the block stops at the first column whose norm falls below acc_defl
  std::vector<double> W((size_t)p * p, 0.0);
  int pa = p;
  for (int l = 0; l < p; ++l) {
    for (int k = 0; k < l; ++k) {
      const double z = red.dot(q[k], q[l], n, s);
      W[(size_t)k * p + l] = z;
      axpy(q[l], q[k], -z, n, s);
    }
    const double nrm = std::sqrt(red.dot(q[l], q[l], n, s));
    if (nrm < acc_defl) {
      pa = l;
      break;
    }
    W[(size_t)l * p + l] = nrm;
    scale(q[l], 1.0 / nrm, n, s);
  }
  out.pa = pa;
  out.W.assign(W.begin(), W.begin() + (size_t)pa * p);
  if (pa == 0) return out;
  // build_mcf sizes the run on the block that survives: 14 p' ln(dim)
  if (pa < p) M0 = (int)(14 * pa * std::log(1.0 * n));
  // blockLanczosSVD orthonormalizes the (already orthonormal) block once more
  for (int l = 0; l < pa; ++l) {
    for (int k = 0; k < l; ++k) axpy(q[l], q[k], -red.dot(q[k], q[l], n, s), n, s);
    const double nrm = std::sqrt(red.dot(q[l], q[l], n, s));
    if (nrm < acc_defl) throw Error(QCMG_ERR_NUMERIC, "block Lanczos: rank-deficient start block");
    scale(q[l], 1.0 / nrm, n, s);
  }
  if (M0 > max_iter) M0 = max_iter;
  // four blocks of pa vectors: Q_prev, Q_cur, Z, Q_next (rotated by pointer)
  auto block = [&]() {
    std::vector<double*> b(pa);
    for (int k = 0; k < pa; ++k) {
      store.emplace_back(n);
      b[k] = store.back().p;
    }
    return b;
  };
  std::vector<double*> Qc(q.begin(), q.begin() + pa), Qp = block(), Z = block(), Qn = block();
  const int pp = pa * pa;
  std::vector<double> Aj(pp), Bj(pp), G(pp), Binv(pp), D, V, dots, col(pa);
  std::vector<const double*> lst;
  std::vector<double> t;  // block-tridiagonal T, column-major, for the convergence probe
  double ev_old = 1e12, last_change = INFINITY;
  for (int j = 0; j < M0; ++j) {
    for (int k = 0; k < pa; ++k) matvec(H, Qc[k], Z[k], false);  // Z = H Q
    // A(k,l) = <Q_k|Z_l>, k <= l, mirrored
    for (int l = 0; l < pa; ++l) {
      lst.assign(Qc.begin(), Qc.begin() + l + 1);
      mops.multidot(lst, Z[l], n, s, dots);
      for (int k = 0; k <= l; ++k) Aj[(size_t)k * pa + l] = Aj[(size_t)l * pa + k] = dots[k];
    }
    out.A.insert(out.A.end(), Aj.begin(), Aj.end());
    // Z_l -= sum_k A(k,l) Q_k  (- sum_k B_{j-1}(l,k) Qprev_k for j > 0)
    for (int l = 0; l < pa; ++l) {
      lst.assign(Qc.begin(), Qc.end());
      for (int k = 0; k < pa; ++k) col[k] = Aj[(size_t)k * pa + l];
      if (j > 0) {
        lst.insert(lst.end(), Qp.begin(), Qp.end());
        for (int k = 0; k < pa; ++k) col.push_back(out.B[(size_t)(j - 1) * pp + (size_t)l * pa + k]);
      }
      mops.multiaxpy(lst, col, Z[l], n, s);
      col.resize(pa);
    }
    // polar decomposition of Z: Gram G = V D V^T, B_j = V D^1/2 V^T
    for (int l = 0; l < pa; ++l) {
      lst.assign(Z.begin(), Z.begin() + l + 1);
      mops.multidot(lst, Z[l], n, s, dots);
      for (int k = 0; k <= l; ++k) G[(size_t)k * pa + l] = G[(size_t)l * pa + k] = dots[k];
    }
    std::vector<double> gcm((size_t)pa * pa);  // lower triangle, column-major, for the solver
    for (int c = 0; c < pa; ++c)
      for (int r = 0; r < pa; ++r) gcm[(size_t)r + (size_t)pa * c] = G[(size_t)r * pa + c];
    if (!band_eigen_leading(gcm, pa, pa, pa - 1, pa, D, V))  // V[k*pa + m]: component k of vector m
      throw Error(QCMG_ERR_NUMERIC, "block Lanczos: Gram eigensolver did not converge");
    bool singular = false;
    for (int m = 0; m < pa; ++m)
      if (D[m] < acc_defl * acc_defl) {
        singular = true;
        break;
      }
    for (int r = 0; r < pa; ++r)
      for (int c = 0; c < pa; ++c) {
        double b = 0.0, bi = 0.0;
        for (int m = 0; m < pa; ++m) {
          const double vv = V[(size_t)r * pa + m] * V[(size_t)c * pa + m];
          b += vv * std::sqrt(std::max(D[m], 0.0));
          if (!singular) bi += vv / std::sqrt(D[m]);
        }
        Bj[(size_t)r * pa + c] = b;
        Binv[(size_t)r * pa + c] = bi;
      }
    out.B.insert(out.B.end(), Bj.begin(), Bj.end());
    out.M = j + 1;
    if (singular) break;
    // Q_next_l = sum_k Binv(k,l) Z_k  (into zeroed vectors: w -= sum (-c) V)
    for (int l = 0; l < pa; ++l) {
      QCMG_CUDA(cudaMemsetAsync(Qn[l], 0, n * 8, s));
      lst.assign(Z.begin(), Z.end());
      for (int k = 0; k < pa; ++k) col[k] = -Binv[(size_t)k * pa + l];
      mops.multiaxpy(lst, col, Qn[l], n, s);
    }
    std::swap(Qp, Qc);  // Q_prev <- Q_cur
    std::swap(Qc, Qn);  // Q_cur <- Q_next (the old Q_prev becomes scratch)
    // convergence every pa steps: lowest eigenvalue of the block-tridiagonal
    // projection (half bandwidth 2 pa - 1, so the banded probe applies)
    if ((j + 1) >= 2 * pa && (j + 1) % pa == 0) {
      const int sz = (j + 1) * pa, bw = 2 * pa - 1;
      t.assign((size_t)(bw + 1) * sz, 0.0);  // packed lower band: (r, c) at (r - c) + (bw + 1) c
      auto put = [&](int r, int c, double v) {
        if (r >= c) t[(size_t)(r - c) + (size_t)(bw + 1) * c] = v;
      };
      for (int jj = 0; jj <= j; ++jj)
        for (int r = 0; r < pa; ++r)
          for (int c = 0; c < pa; ++c) {
            put(jj * pa + r, jj * pa + c, out.A[(size_t)jj * pp + r * pa + c]);
            if (jj < j) put((jj + 1) * pa + r, jj * pa + c, out.B[(size_t)jj * pp + r * pa + c]);
          }
      const bool warm = ev_old < 1e12;
      const double width = std::isfinite(last_change) && warm
                               ? std::max(4.0 * last_change, 1e-12 * std::max(1.0, std::fabs(ev_old)))
                               : 1e-3 * std::max(1.0, std::fabs(ev_old));
      const double e0 = warm ? band_lowest_packed(t, sz, bw, ev_old, width)
                             : band_lowest_packed(t, sz, bw);
      const double delta = std::fabs(e0 - ev_old);
      if (ev_old < 1e12) last_change = delta;
      ev_old = e0;
      if (delta < acc_band) break;
    }
  }
  return out;
}

BandResult band_lanczos(qcmg_hamiltonian* H, int p, const double* phi_in, bool phi_on_device, int M0,
                        int max_iter,
                        double acc_defl, double acc_band) {
  const size_t n = H->dim;
  cudaStream_t s = H->stream;
  BandResult out;
  QCMG_CHECK_ARG(p > 0, "band Lanczos needs at least one start vector");
  int pc = p;
  if (M0 > max_iter) M0 = max_iter;
  int M0p = (M0 / p + 1) * p;
  M0 = M0p - pc;
  QCMG_CHECK_ARG(M0 > 0, "band Lanczos needs M > 0");
  // Device vectors: the p start vectors (the caller's own when they are on
  // the device: they are only read) plus a pool for v[0..M0p).
  std::vector<DevVec> phi;
  std::vector<const double*> phip;
  for (int k = 0; k < p; ++k) {
    if (phi_on_device) {
      phip.push_back(phi_in + (size_t)k * n);
      continue;
    }
    phi.emplace_back(n);
    QCMG_CUDA(cudaMemcpyAsync(phi[k].p, phi_in + (size_t)k * n, n * 8, cudaMemcpyHostToDevice, s));
    phip.push_back(phi[k].p);
  }
  std::vector<double*> v(M0p, nullptr);
  std::vector<double*> pool;
  std::vector<DevVec> owned;
  auto get = [&]() -> double* {
    if (!pool.empty()) {
      double* r = pool.back();
      pool.pop_back();
      return r;
    }
    owned.emplace_back(n);
    return owned.back().p;
  };
  auto erase = [&](int k) {
    if (v[k]) pool.push_back(v[k]);
    v[k] = nullptr;
  };
  for (int i = 0; i < p; ++i) {
    v[i] = get();
    QCMG_CUDA(cudaMemcpyAsync(v[i], phip[i], n * 8, cudaMemcpyDeviceToDevice, s));
  }
  std::vector<double> t((size_t)M0 * M0, 0.0);  // column-major t(r,c) = t[r + M0*c]
  auto T = [&](int r, int c) -> double& { return t[(size_t)r + (size_t)M0 * c]; };
  std::vector<double> P((size_t)p * M0, 0.0);   // P(k,j) = P[k + p*j]
  std::vector<int> defl(M0, 0);
  std::vector<int> I;
  Reducer red;
  MultiOps mops;
  std::vector<double> tmp;
  Cusolver solver;
  double ev_old = 1e12;
  double last_change = INFINITY;
  int j;
  std::vector<const double*> tg;
  std::vector<double*> gs_vecs;
  std::vector<double> gs_coef;
  std::vector<const double*> rec_vecs;
  std::vector<double> rec_coef;
  // The dots of the closing Gram-Schmidt sweep stay on the device: each
  // lands in a slot of tdev (p + 1 slots per step), its axpy reads it there,
  // and the host copies the slots into t only where t is read next (the
  // convergence probe and the end), so a step waits on the device once.
  const int slots = p + 1;
  DevBuf<double> tdev;
  tdev.alloc((size_t)M0 * slots);
  std::vector<double> thost((size_t)M0 * slots);
  struct Pending {
    int slot, r, c;
  };
  std::vector<Pending> pend;
  auto flush = [&]() {
    if (pend.empty()) return;
    int lo = pend.front().slot, hi = lo;
    for (const Pending& q : pend) {
      lo = std::min(lo, q.slot);
      hi = std::max(hi, q.slot);
    }
    QCMG_CUDA(cudaMemcpyAsync(thost.data() + lo, tdev.p + lo, (size_t)(hi - lo + 1) * 8,
                              cudaMemcpyDeviceToHost, s));
    QCMG_CUDA(cudaStreamSynchronize(s));
    for (const Pending& q : pend) T(q.r, q.c) = T(q.c, q.r) = thost[q.slot];
    pend.clear();
  };
  for (j = 0; j < M0; ++j) {
    // One multi-dot on the unscaled v_j gives its norm, its projections on
    // the p start vectors and its dots with the next pc-1 vectors (each of
    // those vectors is changed only by its own update below, so the dots
    // are independent): one synchronization instead of pc + 1.  The
    // projections P(:, j) are taken for j < p only: the Q-matrix product
    // bounds its inner index by p (Hamiltonian_base.hpp:249), so no later
    // column of P reaches the result, and on GB300 each dot is an FP64 FMA
    // per element.
    const int nproj = j < p ? p : 0;
    tg.clear();
    tg.push_back(v[j]);
    for (int k = 0; k < nproj; ++k) tg.push_back(phip[k]);
    for (int k = j + 1; k < j + pc; ++k) tg.push_back(v[k]);
    mops.multidot(tg, v[j], n, s, tmp);
    double z = std::sqrt(tmp[0]);
    if (z < acc_defl) {
      if (j >= pc) {
        I.push_back(j - pc);
        defl[j - pc] = 1;
      }
      pc--;
      if (pc == 0) break;
      erase(j);
      for (int k = j; k < j + pc; ++k) v[k] = v[k + 1];
      v[j + pc] = nullptr;
      j--;
      continue;
    }
    // v_j /= z; v_k -= <v_j, v_k> v_j for the next pc-1 vectors (one kernel)
    const double iz = 1.0 / z;
    if (j >= pc) T(j, j - pc) = z;
    for (int k = 0; k < nproj; ++k) P[k + (size_t)p * j] = tmp[1 + k] * iz;
    gs_vecs.clear();
    gs_coef.clear();
    for (int k = j + 1; k < j + pc; ++k) {
      const double zz = tmp[1 + nproj + (k - j - 1)] * iz;
      gs_vecs.push_back(v[k]);
      gs_coef.push_back(zz);
      if (k >= pc) T(j, k - pc) = zz;
    }
    mops.scale_sub(v[j], iz, gs_vecs, gs_coef, n, s);
    v[j + pc] = get();
    matvec(H, v[j], v[j + pc], false);
    int k0 = 0;
    if (j > pc) {
      k0 = j - pc;
      if (defl[k0 - 1] == 0) erase(k0 - 1);
    }
    // v_{j+pc} -= sum_k T(k, j) v_k over the band (one kernel)
    rec_vecs.clear();
    rec_coef.clear();
    for (int k = k0; k < j; ++k) {
      T(k, j) = T(j, k);
      rec_vecs.push_back(v[k]);
      rec_coef.push_back(T(k, j));
    }
    // with no deflated vectors the recurrence and the closing step against
    // v_j are one fused pair of launches
    if (!(I.empty() &&
          mops.multiaxpy_orth(rec_vecs, rec_coef, v[j + pc], v[j], n, tdev.p + j * slots, s))) {
      mops.multiaxpy(rec_vecs, rec_coef, v[j + pc], n, s);
      for (size_t q = 0; q < I.size(); ++q) {
        const int slot = j * slots + 1 + (int)q;
        red.dot_dev(v[I[q]], v[j + pc], n, tdev.p + slot, s);
        axpy_neg_dev(v[j + pc], v[I[q]], tdev.p + slot, n, s);
        pend.push_back({slot, I[q], j});  // t(idx, j) = t(j, idx)
      }
      red.dot_dev(v[j], v[j + pc], n, tdev.p + j * slots, s);
      axpy_neg_dev(v[j + pc], v[j], tdev.p + j * slots, n, s);
    }
    pend.push_back({j * slots, j, j});
    if (j >= 4 * p && j % p == 0) {
      flush();
      // Until a vector deflates inside the band, t is a band matrix of half
      // bandwidth p, and its lowest eigenvalue comes from banded-Cholesky
      // bisection on the host; a deflated vector adds entries outside the
      // band, and then the device eigensolver takes the whole block.
      double e0;
      if (I.empty()) {
        // the previous probe's value bounds this one from above (the
        // earlier block is a leading principal submatrix) and its last
        // change sizes the starting bracket
        const bool warm = ev_old < 1e12;
        const double width =
            std::isfinite(last_change) && warm
                ? std::max(4.0 * last_change, 1e-12 * std::max(1.0, std::fabs(ev_old)))
                : 1e-3 * std::max(1.0, std::fabs(ev_old));
        e0 = warm ? band_lowest(t, M0, j, p, ev_old, width) : band_lowest(t, M0, j, p);
      } else {
        std::vector<double> ev;
        solver.syevd(t, M0, j, false, s, ev, nullptr);
        e0 = ev[0];
      }
      double test = std::fabs(e0 - ev_old);
      if (ev_old < 1e12) last_change = test;
      ev_old = e0;
      if (test < acc_band) break;
    }
  }
  flush();
  out.M = j;
  if (j == 0) return out;
  // Q = P(:, 0:k) U(0:k, :), k = min(p, M) (Hamiltonian_base.hpp:249 with
  // matrix::product's bound on the inner index): all eigenvalues of t but
  // only the leading k rows of its eigenvectors.  Without in-band
  // deflation t is a band matrix and the host band solver gives exactly
  // that; otherwise the device eigensolver takes the whole block.
  const int M = j, kk = std::min(p, M);
  std::vector<double> U;  // U(k, c) = U[k * ustride_k + c * ustride_c]
  size_t ustride_k = 1, ustride_c = (size_t)M;
  if (!(I.empty() && band_eigen_leading(t, M0, M, p, kk, out.evals, U))) {
    solver.syevd(t, M0, j, true, s, out.evals, &U);
  } else {
    ustride_k = (size_t)M;
    ustride_c = 1;
  }
  out.Q.assign((size_t)p * M, 0.0);
  for (int a = 0; a < p; ++a)
    for (int c = 0; c < M; ++c) {
      double acc = 0.0;
      for (int k = 0; k < kk; ++k) acc += P[a + (size_t)p * k] * U[k * ustride_k + c * ustride_c];
      out.Q[(size_t)a * M + c] = acc;
    }
  return out;
}

}  // namespace qcmg
