// Half-basis indexing and half-operator construction on the GPU.
//
// A half basis is the increasing list of L-bit integers with N set bits
// (pyqcm src_ed/ED_basis.cpp:115-125).  For a fixed popcount, increasing
// integer order is colexicographic order of the occupied-orbital sets, so
// the rank of a state b with occupied orbitals c_1 < ... < c_N is
//     rank(b) = sum_k C(c_k, k)        (combinatorial number system)
// and a rank is unranked greedily from the top.  This replaces the
// reference's materialized list plus binary search
// (src_ed/ED_basis.cpp:130-135) with exact integer arithmetic: no table
// larger than the 33 x 33 binomials is needed on the device.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "qcmg_internal.h"

namespace qcmg {

__constant__ uint32_t c_binom[kMaxOrbitals + 1][kMaxOrbitals + 1];

uint64_t binomial(int n, int k) {
  if (k < 0 || n < 0 || k > n) return 0;
  uint64_t r = 1;
  for (int i = 1; i <= k; ++i) r = r * (uint64_t)(n - k + i) / (uint64_t)i;
  return r;
}

void ensure_device_tables(int device) {
  static std::mutex m;
  static std::vector<int> done;
  std::lock_guard<std::mutex> lock(m);
  if (std::find(done.begin(), done.end(), device) != done.end()) return;
  uint32_t h[kMaxOrbitals + 1][kMaxOrbitals + 1];
  for (int n = 0; n <= kMaxOrbitals; ++n)
    for (int k = 0; k <= kMaxOrbitals; ++k) h[n][k] = (uint32_t)binomial(n, k);
  QCMG_CUDA(cudaMemcpyToSymbol(c_binom, h, sizeof(h)));
  done.push_back(device);
}

__device__ __forceinline__ uint32_t dev_rank(uint32_t b) {
  uint32_t r = 0;
  int k = 1;
  while (b) {
    int c = __ffs(b) - 1;
    r += c_binom[c][k];
    ++k;
    b &= b - 1;
  }
  return r;
}

__device__ __forceinline__ uint32_t dev_unrank(uint32_t r, int L, int N) {
  uint32_t b = 0;
  int c = L - 1;
  for (int k = N; k >= 1; --k) {
    while (c_binom[c][k] > r) --c;
    b |= 1u << c;
    r -= c_binom[c][k];
    --c;
  }
  return b;
}

__global__ void k_halfbasis(int L, int N, uint32_t dim, uint32_t* out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < dim; i += gridDim.x * blockDim.x)
    out[i] = dev_unrank(i, L, N);
}

__global__ void k_rank(int L, const uint32_t* __restrict__ st, size_t n, uint32_t dim,
                       uint32_t* __restrict__ ranks) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    uint32_t b = st[i];
    bool ok = (L >= 32) || (b >> L) == 0;
    uint32_t r = ok ? dev_rank(b) : dim;
    ranks[i] = (r < dim) ? r : dim;
  }
}

static unsigned grid_for(size_t n, unsigned block) {
  size_t g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (g > 65535u * 8) g = 65535u * 8;
  return (unsigned)g;
}

void launch_halfbasis(int L, int N, uint32_t dim, uint32_t* out, cudaStream_t s) {
  if (!dim) return;
  k_halfbasis<<<grid_for(dim, 256), 256, 0, s>>>(L, N, dim, out);
  QCMG_CUDA(cudaGetLastError());
}

void launch_rank(int L, const uint32_t* states, size_t n, uint32_t dim, uint32_t* ranks,
                 cudaStream_t s) {
  if (!n) return;
  k_rank<<<grid_for(n, 256), 256, 0, s>>>(L, states, n, dim, ranks);
  QCMG_CUDA(cudaGetLastError());
}

// Fermion sign of moving the electron at bit c to bit r: parity of the
// occupied orbitals strictly between (binary_state::interphase,
// src_ed/binary_state.hpp:42-49).
__device__ __forceinline__ int hop_parity(uint32_t b, int r, int c) {
  int lo = min(r, c), hi = max(r, c);
  uint32_t between = (hi >= 32 ? 0xffffffffu : ((1u << hi) - 1u)) & ~((2u << lo) - 1u);
  return __popc(b & between) & 1;
}

// Pass 1: entries per row (hops allowed from each state).
__global__ void k_halfop_count(uint32_t dim, const uint32_t* __restrict__ bin,
                               const HopElement* __restrict__ el, int nel,
                               uint32_t* __restrict__ cnt) {
  for (uint32_t I = blockIdx.x * blockDim.x + threadIdx.x; I < dim; I += gridDim.x * blockDim.x) {
    uint32_t b = bin[I], n = 0;
    for (int k = 0; k < nel; ++k) {
      int r = el[k].r, c = el[k].c;
      if (r == c || el[k].v == 0.0) continue;
      if (((b >> c) & 1u) && !((b >> r) & 1u)) ++n;
    }
    cnt[I] = n;
  }
}

// Pass 2: fill (J, sign * v) in element order and the diagonal.
__global__ void k_halfop_fill(uint32_t dim, const uint32_t* __restrict__ bin,
                              const HopElement* __restrict__ el, int nel,
                              const uint32_t* __restrict__ rowptr, uint32_t* __restrict__ col,
                              double* __restrict__ val, double* __restrict__ diag) {
  for (uint32_t I = blockIdx.x * blockDim.x + threadIdx.x; I < dim; I += gridDim.x * blockDim.x) {
    uint32_t b = bin[I];
    uint32_t pos = rowptr[I];
    double d = 0.0;
    for (int k = 0; k < nel; ++k) {
      int r = el[k].r, c = el[k].c;
      double v = el[k].v;
      if (r == c) {
        if ((b >> r) & 1u) d += v;
        continue;
      }
      if (v == 0.0) continue;
      if (((b >> c) & 1u) && !((b >> r) & 1u)) {
        uint32_t bp = b ^ (1u << c) ^ (1u << r);
        col[pos] = dev_rank(bp);
        val[pos] = hop_parity(b, r, c) ? -v : v;
        ++pos;
      }
    }
    diag[I] = d;
  }
}

void build_halfop(HalfOp& op, int L, int N, const std::vector<HopElement>& el, cudaStream_t s) {
  op.L = L;
  op.N = N;
  uint64_t dim64 = binomial(L, N);
  QCMG_CHECK_ARG(dim64 < (1ull << 31), "half basis too large");
  op.dim = (uint32_t)dim64;
  op.bin.alloc(op.dim);
  launch_halfbasis(L, N, op.dim, op.bin.p, s);
  for (auto& e : el) {
    QCMG_CHECK_ARG(e.r >= 0 && e.r < L && e.c >= 0 && e.c < L, "hop element orbital out of range");
  }
  DevBuf<HopElement> d_el;
  d_el.upload(el.data(), el.size(), s);
  DevBuf<uint32_t> cnt;
  cnt.alloc(op.dim);
  op.rowptr.alloc(op.dim + 1);
  op.diag.alloc(op.dim);
  if (op.dim) {
    k_halfop_count<<<grid_for(op.dim, 256), 256, 0, s>>>(op.dim, op.bin.p, d_el.p, (int)el.size(),
                                                          cnt.p);
    QCMG_CUDA(cudaGetLastError());
  }
  std::vector<uint32_t> h_cnt(op.dim), h_rp(op.dim + 1);
  if (op.dim)
    QCMG_CUDA(cudaMemcpyAsync(h_cnt.data(), cnt.p, op.dim * 4, cudaMemcpyDeviceToHost, s));
  QCMG_CUDA(cudaStreamSynchronize(s));
  size_t nnz = 0;
  for (uint32_t i = 0; i < op.dim; ++i) {
    h_rp[i] = (uint32_t)nnz;
    nnz += h_cnt[i];
  }
  h_rp[op.dim] = (uint32_t)nnz;
  QCMG_CHECK_ARG(nnz < (1ull << 32), "half operator too large");
  op.nnz = nnz;
  QCMG_CUDA(cudaMemcpyAsync(op.rowptr.p, h_rp.data(), (op.dim + 1) * 4, cudaMemcpyHostToDevice, s));
  op.col.alloc(nnz);
  op.val.alloc(nnz);
  if (op.dim) {
    k_halfop_fill<<<grid_for(op.dim, 256), 256, 0, s>>>(op.dim, op.bin.p, d_el.p, (int)el.size(),
                                                         op.rowptr.p, op.col.p, op.val.p,
                                                         op.diag.p);
    QCMG_CUDA(cudaGetLastError());
  }
  // Row bounds for the fixed-point headroom: |T|_inf and |diag|_max.
  std::vector<double> h_val(nnz), h_diag(op.dim);
  if (nnz) QCMG_CUDA(cudaMemcpyAsync(h_val.data(), op.val.p, nnz * 8, cudaMemcpyDeviceToHost, s));
  if (op.dim)
    QCMG_CUDA(cudaMemcpyAsync(h_diag.data(), op.diag.p, op.dim * 8, cudaMemcpyDeviceToHost, s));
  QCMG_CUDA(cudaStreamSynchronize(s));
  op.max_row_abs = 0.0;
  op.max_diag_abs = 0.0;
  for (uint32_t i = 0; i < op.dim; ++i) {
    double a = 0.0;
    for (uint32_t k = h_rp[i]; k < h_rp[i + 1]; ++k) a += std::fabs(h_val[k]);
    op.max_row_abs = std::max(op.max_row_abs, a);
    op.max_diag_abs = std::max(op.max_diag_abs, std::fabs(h_diag[i]));
  }
}

// ---------------------------------------------------------------------------
// c / c^dagger on a factorized state (model::create_or_destroy, factorized
// branch, src_ed/model.cpp:160-180; sign from Destroy, src_ed/ED_basis.cpp:79-110).
// One thread per SOURCE state for destruction and per TARGET state for
// creation, so every output element is written by exactly one thread.

__global__ void k_apply_c(int L, int orb, int spin, int pm, int nup, int ndn, uint32_t du,
                          uint32_t dd, uint32_t du2, uint32_t dd2, const double* __restrict__ x,
                          double* __restrict__ y, double z, int accumulate) {
  // Iterate over the TARGET sector: y[t] = z * sign * x[s], where s is the
  // state obtained by removing (creation) or adding (destruction) the electron.
  size_t n2 = (size_t)du2 * dd2;
  uint32_t m = 1u << orb;
  int nup2 = nup + (spin ? 0 : pm), ndn2 = ndn + (spin ? pm : 0);
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n2;
       t += (size_t)gridDim.x * blockDim.x) {
    uint32_t iu2 = (uint32_t)(t % du2), id2 = (uint32_t)(t / du2);
    uint32_t u2 = dev_unrank(iu2, L, nup2), d2 = dev_unrank(id2, L, ndn2);
    double out = 0.0;
    uint32_t occ = spin ? d2 : u2;
    // creation: target must hold the electron; destruction: must not.
    bool ok = (pm > 0) ? ((occ & m) != 0) : ((occ & m) == 0);
    if (ok) {
      uint32_t u = u2, d = d2;
      int par;
      if (!spin) {
        u = u2 ^ m;
        par = __popc(u2 & (m - 1u));
      } else {
        d = d2 ^ m;
        par = __popc(d2 & (m - 1u)) + __popc(u2);
      }
      size_t s = (size_t)dev_rank(u) + (size_t)du * dev_rank(d);
      out = z * ((par & 1) ? -x[s] : x[s]);
    }
    y[t] = accumulate ? y[t] + out : out;
  }
}

void launch_apply_c(int L, int orb, int spin, int pm, int nup, int ndn, const double* x, double* y,
                    double z, bool accumulate, cudaStream_t s) {
  uint32_t du = (uint32_t)binomial(L, nup), dd = (uint32_t)binomial(L, ndn);
  int nup2 = nup + (spin ? 0 : pm), ndn2 = ndn + (spin ? pm : 0);
  uint32_t du2 = (uint32_t)binomial(L, nup2), dd2 = (uint32_t)binomial(L, ndn2);
  size_t n2 = (size_t)du2 * dd2;
  if (!n2) return;
  k_apply_c<<<grid_for(n2, 256), 256, 0, s>>>(L, orb, spin, pm, nup, ndn, du, dd, du2, dd2, x, y,
                                               z, accumulate ? 1 : 0);
  QCMG_CUDA(cudaGetLastError());
}

}  // namespace qcmg
