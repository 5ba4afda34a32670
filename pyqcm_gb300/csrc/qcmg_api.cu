// C ABI entry points (declared in include/qcmg.h): argument checking, error
// reporting, host<->device staging, and the handle lifetime.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "qcmg.h"
#include "qcmg_internal.h"
#include "qcmg_fx.cuh"
#include "qcmg_fxpath.h"
#include "qcmg_krylov.h"
#include "qcmg_lattice.h"

namespace qcmg {

static thread_local std::string g_error;
static thread_local int g_device = 0;

void set_error(const std::string& msg) { g_error = msg; }
void clear_error() { g_error.clear(); }

template <class F>
static int guarded(F&& f) {
  try {
    clear_error();
    f();
    return QCMG_OK;
  } catch (const Error& e) {
    set_error(e.what());
    return e.code;
  } catch (const std::bad_alloc&) {
    set_error("host allocation failed");
    return QCMG_ERR_NOMEM;
  } catch (const std::exception& e) {
    set_error(e.what());
    return QCMG_ERR_CUDA;
  }
}

static void use_device() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0)
    throw Error(QCMG_ERR_DEVICE, std::string("no usable CUDA device: ") + cudaGetErrorString(e));
  if (g_device >= n) throw Error(QCMG_ERR_DEVICE, "device index out of range");
  QCMG_CUDA(cudaSetDevice(g_device));
  ensure_device_tables(g_device);
}

static unsigned classify_onsite(const std::vector<double>& W, int L, double* U, uint32_t* mask) {
  // Diagonal with a single nonzero value -> U * popcount(u & d & mask).
  double u = 0.0;
  uint32_t m = 0;
  for (int r = 0; r < L; ++r)
    for (int c = 0; c < L; ++c) {
      double w = W[(size_t)r * L + c];
      if (w == 0.0) continue;
      if (r != c) return QCMG_INTER_GENERAL;
      if (u == 0.0) u = w;
      if (w != u) return QCMG_INTER_GENERAL;
      m |= 1u << r;
    }
  if (u == 0.0) return QCMG_INTER_NONE;
  *U = u;
  *mask = m;
  return QCMG_INTER_ONSITE;
}

}  // namespace qcmg

using namespace qcmg;

// ---------------------------------------------------------------------------
// Same-spin density-density pairs are diagonal in one half basis: fold them
// into that spin's diagonal.  Cross-spin pairs W[r_up][c_dn] are evaluated in
// the product (on-site fast path) or tabulated per down state.

__global__ void k_pair_diag(uint32_t dim, const uint32_t* __restrict__ bin, int r, int c, double v,
                            double* __restrict__ diag) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < dim; i += gridDim.x * blockDim.x) {
    uint32_t b = bin[i];
    if (((b >> r) & 1u) && ((b >> c) & 1u)) diag[i] += v;
  }
}

__global__ void k_cross_table(uint32_t dd, int L, const uint32_t* __restrict__ bin_dn,
                              const double* __restrict__ W, double* __restrict__ wdn) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < dd; i += gridDim.x * blockDim.x) {
    uint32_t d = bin_dn[i];
    for (int r = 0; r < L; ++r) {
      double s = 0.0;
      for (int c = 0; c < L; ++c)
        if ((d >> c) & 1u) s += W[(size_t)r * L + c];
      wdn[(size_t)i * L + r] = s;
    }
  }
}

extern "C" {

const char* qcmg_version(void) { return "qcmg 0.1 (sm_103a)"; }

size_t qcmg_last_error(char* buf, size_t n) {
  if (buf && n) {
    size_t k = std::min(n - 1, g_error.size());
    std::memcpy(buf, g_error.data(), k);
    buf[k] = 0;
  }
  return g_error.size();
}

int qcmg_set_device(int device) {
  return guarded([&] {
    QCMG_CHECK_ARG(device >= 0, "negative device index");
    g_device = device;
    use_device();
  });
}

int qcmg_halfbasis(int L, int N, uint32_t* out, size_t cap, size_t* dim) {
  return guarded([&] {
    QCMG_CHECK_ARG(L >= 1 && L <= kMaxOrbitals, "L must be in 1..32");
    QCMG_CHECK_ARG(dim != nullptr, "dim is NULL");
    uint64_t d = (N < 0 || N > L) ? 0 : binomial(L, N);
    *dim = (size_t)d;
    if (!d || !out || !cap) return;
    QCMG_CHECK_ARG(d < (1ull << 31), "half basis too large");
    use_device();
    DevBuf<uint32_t> buf;
    buf.alloc(d);
    launch_halfbasis(L, N, (uint32_t)d, buf.p, 0);
    QCMG_CUDA(cudaMemcpy(out, buf.p, std::min<size_t>(cap, d) * 4, cudaMemcpyDeviceToHost));
  });
}

int qcmg_halfbasis_rank(int L, int N, const uint32_t* states, size_t n, uint32_t* ranks) {
  return guarded([&] {
    QCMG_CHECK_ARG(L >= 1 && L <= kMaxOrbitals, "L must be in 1..32");
    QCMG_CHECK_ARG(N >= 0 && N <= L, "N out of range");
    if (!n) return;
    QCMG_CHECK_ARG(states && ranks, "NULL array");
    use_device();
    uint32_t d = (uint32_t)binomial(L, N);
    // States with the wrong popcount are not in the basis: mark them first.
    std::vector<uint32_t> st(states, states + n);
    DevBuf<uint32_t> ds, dr;
    ds.upload(st.data(), n, 0);
    dr.alloc(n);
    launch_rank(L, ds.p, n, d, dr.p, 0);
    QCMG_CUDA(cudaMemcpy(ranks, dr.p, n * 4, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n; ++i)
      if (__builtin_popcount(st[i]) != N) ranks[i] = d;
  });
}

int qcmg_hamiltonian_create(int L, int n_up, int n_dn, int n_hop_up, const int32_t* up_r,
                            const int32_t* up_c, const double* up_v, int n_hop_dn,
                            const int32_t* dn_r, const int32_t* dn_c, const double* dn_v,
                            int n_pair, const int32_t* pair_r, const int32_t* pair_c,
                            const double* pair_v, qcmg_hamiltonian** out) {
  return guarded([&] {
    QCMG_CHECK_ARG(out != nullptr, "out is NULL");
    *out = nullptr;
    QCMG_CHECK_ARG(L >= 1 && L <= kMaxOrbitals, "L must be in 1..32");
    QCMG_CHECK_ARG(n_up >= 0 && n_up <= L && n_dn >= 0 && n_dn <= L, "electron count out of range");
    QCMG_CHECK_ARG(n_hop_up >= 0 && n_hop_dn >= 0 && n_pair >= 0, "negative element count");
    QCMG_CHECK_ARG((n_hop_up == 0 || (up_r && up_c && up_v)) &&
                       (n_hop_dn == 0 || (dn_r && dn_c && dn_v)) &&
                       (n_pair == 0 || (pair_r && pair_c && pair_v)),
                   "NULL element array");
    for (int k = 0; k < n_hop_up + n_hop_dn + n_pair; ++k) {
      double v = k < n_hop_up ? up_v[k]
                 : k < n_hop_up + n_hop_dn ? dn_v[k - n_hop_up]
                                           : pair_v[k - n_hop_up - n_hop_dn];
      QCMG_CHECK_ARG(std::isfinite(v), "non-finite matrix element");
    }
    use_device();
    auto* H = new qcmg_hamiltonian();
    try {
      H->device = g_device;
      H->L = L;
      H->nup = n_up;
      H->ndn = n_dn;
      QCMG_CUDA(cudaStreamCreateWithFlags(&H->own_stream, cudaStreamNonBlocking));
      H->stream = H->own_stream;
      std::vector<HopElement> eu, ed;
      for (int k = 0; k < n_hop_up; ++k) eu.push_back({up_r[k], up_c[k], up_v[k]});
      for (int k = 0; k < n_hop_dn; ++k) ed.push_back({dn_r[k], dn_c[k], dn_v[k]});
      build_halfop(H->up, L, n_up, eu, H->stream);
      build_halfop(H->dn, L, n_dn, ed, H->stream);
      H->du = H->up.dim;
      H->dd = H->dn.dim;
      H->dim = (size_t)H->du * H->dd;
      std::vector<double> W((size_t)L * L, 0.0);
      for (int k = 0; k < n_pair; ++k) {
        int r = pair_r[k], c = pair_c[k];
        double v = pair_v[k];
        QCMG_CHECK_ARG(r >= 0 && r < 2 * L && c >= 0 && c < 2 * L, "pair orbital out of range");
        if (v == 0.0) continue;
        bool ru = r < L, cu = c < L;
        if (ru && cu) {
          if (H->du)
            k_pair_diag<<<(H->du + 255) / 256, 256, 0, H->stream>>>(H->du, H->up.bin.p, r, c, v,
                                                                    H->up.diag.p);
        } else if (!ru && !cu) {
          if (H->dd)
            k_pair_diag<<<(H->dd + 255) / 256, 256, 0, H->stream>>>(H->dd, H->dn.bin.p, r - L,
                                                                    c - L, v, H->dn.diag.p);
        } else if (ru) {
          W[(size_t)r * L + (c - L)] += v;
        } else {
          W[(size_t)c * L + (r - L)] += v;
        }
        QCMG_CUDA(cudaGetLastError());
      }
      uint32_t mask = 0;
      H->inter_kind = (int)classify_onsite(W, L, &H->U, &mask);
      H->max_inter_abs = 0.0;
      for (int r = 0; r < L; ++r) {
        double s = 0.0;
        for (int c = 0; c < L; ++c) s += std::fabs(W[(size_t)r * L + c]);
        H->max_inter_abs += s;
      }
      if (H->inter_kind == QCMG_INTER_ONSITE && mask != (L >= 32 ? 0xffffffffu : (1u << L) - 1u)) {
        // masked on-site term (e.g. no U on bath orbitals): tabulate instead
        H->inter_kind = QCMG_INTER_GENERAL;
      }
      if (H->inter_kind == QCMG_INTER_GENERAL && H->dd) {
        DevBuf<double> dW;
        dW.upload(W.data(), W.size(), H->stream);
        H->wdn.alloc((size_t)H->dd * L);
        k_cross_table<<<(H->dd + 127) / 128, 128, 0, H->stream>>>(H->dd, L, H->dn.bin.p, dW.p,
                                                                  H->wdn.p);
        QCMG_CUDA(cudaGetLastError());
        QCMG_CUDA(cudaStreamSynchronize(H->stream));
      }
      QCMG_CUDA(cudaStreamSynchronize(H->stream));
    } catch (...) {
      if (H->own_stream) cudaStreamDestroy(H->own_stream);
      delete H;
      throw;
    }
    *out = H;
  });
}

int qcmg_hamiltonian_destroy(qcmg_hamiltonian* H) {
  return guarded([&] {
    if (!H) return;
    cudaSetDevice(H->device);
    if (H->stream) cudaStreamSynchronize(H->stream);
    if (H->copy_stream) {
      cudaStreamSynchronize(H->copy_stream);
      cudaStreamDestroy(H->copy_stream);
    }
    if (H->ev_x) cudaEventDestroy(H->ev_x);
    if (H->ev_y) cudaEventDestroy(H->ev_y);
    if (H->own_stream) cudaStreamDestroy(H->own_stream);
    delete H;
  });
}

int qcmg_hamiltonian_set_stream(qcmg_hamiltonian* H, void* stream) {
  return guarded([&] {
    QCMG_CHECK_ARG(H != nullptr, "NULL handle");
    std::lock_guard<std::mutex> lock(H->mu);
    H->stream = stream ? (cudaStream_t)stream : H->own_stream;
  });
}

int qcmg_hamiltonian_dims(const qcmg_hamiltonian* H, size_t* du, size_t* dd, size_t* dim) {
  return guarded([&] {
    QCMG_CHECK_ARG(H != nullptr, "NULL handle");
    if (du) *du = H->du;
    if (dd) *dd = H->dd;
    if (dim) *dim = H->dim;
  });
}

int qcmg_hamiltonian_halfop(const qcmg_hamiltonian* H, int spin, size_t* nnz, uint32_t* rowptr,
                            uint32_t* col, double* val, double* diag) {
  return guarded([&] {
    QCMG_CHECK_ARG(H != nullptr && nnz != nullptr, "NULL argument");
    QCMG_CHECK_ARG(spin == 0 || spin == 1, "spin must be 0 or 1");
    const HalfOp& op = spin ? H->dn : H->up;
    *nnz = op.nnz;
    if (!rowptr) return;
    QCMG_CUDA(cudaSetDevice(H->device));
    QCMG_CUDA(cudaMemcpy(rowptr, op.rowptr.p, (op.dim + 1) * 4, cudaMemcpyDeviceToHost));
    if (op.nnz && col) QCMG_CUDA(cudaMemcpy(col, op.col.p, op.nnz * 4, cudaMemcpyDeviceToHost));
    if (op.nnz && val) QCMG_CUDA(cudaMemcpy(val, op.val.p, op.nnz * 8, cudaMemcpyDeviceToHost));
    if (op.dim && diag) QCMG_CUDA(cudaMemcpy(diag, op.diag.p, op.dim * 8, cudaMemcpyDeviceToHost));
  });
}

// y (+)= d into page-locked host memory through its device-side address
// (zero copy: the old y is read and the new one written in one pass).
__global__ void k_add_to_host(const double* __restrict__ d, double* __restrict__ yh, size_t n,
                              int acc) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    yh[i] = acc ? yh[i] + d[i] : d[i];
}

// cuPointerGetAttribute through the runtime's driver entry point (no link
// against the driver library); null when the driver does not provide it.
typedef CUresult (*PointerGetAttributeFn)(void*, CUpointer_attribute, CUdeviceptr);
static PointerGetAttributeFn pointer_get_attribute() {
  static PointerGetAttributeFn fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuPointerGetAttribute", &f, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<PointerGetAttributeFn>(f);
  }();
  return fn;
}

// Device-side address of a page-locked host buffer when all n doubles from
// p lie inside one page-locked allocation made or registered against
// `device`; null otherwise (pageable or device memory, another device's
// allocation, a range the driver cannot report, or a buffer shorter than
// n), and the caller then stages the copies instead.
static double* pinned_device_address(double* p, size_t n, int device) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer || a.device != device) return nullptr;
  PointerGetAttributeFn get = pointer_get_attribute();
  CUdeviceptr start = 0;
  size_t size = 0;
  if (!get || get(&start, CU_POINTER_ATTRIBUTE_RANGE_START_ADDR, (CUdeviceptr)(uintptr_t)p) != 0 ||
      get(&size, CU_POINTER_ATTRIBUTE_RANGE_SIZE, (CUdeviceptr)(uintptr_t)p) != 0)
    return nullptr;
  const uintptr_t lo = (uintptr_t)p, hi = lo + n * sizeof(double);
  if (lo < (uintptr_t)start || hi > (uintptr_t)start + size) return nullptr;
  return (double*)a.devicePointer;
}

int qcmg_matvec(qcmg_hamiltonian* H, const double* x, double* y, unsigned flags) {
  return guarded([&] {
    QCMG_CHECK_ARG(H != nullptr && x != nullptr && y != nullptr, "NULL argument");
    QCMG_CHECK_ARG(x != y, "x and y must not alias");
    std::lock_guard<std::mutex> lock(H->mu);
    QCMG_CUDA(cudaSetDevice(H->device));
    const bool acc = (flags & QCMG_ACCUMULATE) != 0;
    const size_t n = H->dim;
    const bool fx = H->use_fx && fx_prepare(H);
    if (flags & QCMG_DEVICE_PTRS) {
      if (fx)
        fx_matvec_f64(H, x, y, acc);
      else
        matvec(H, x, y, acc);
      if (!(flags & QCMG_ASYNC)) {
        QCMG_CUDA(cudaStreamSynchronize(H->stream));
        if (fx) fx_check_error(H);
      }
      return;
    }
    H->xbuf.alloc(n);
    // QCMG_VERBOSE: which form ran, and its phases timed with events
    static const bool verbose = std::getenv("QCMG_VERBOSE") != nullptr;
    cudaEvent_t ev[4] = {};
    if (verbose)
      for (auto& e : ev) QCMG_CUDA(cudaEventCreate(&e));
    auto mark = [&](int i) {
      if (verbose) QCMG_CUDA(cudaEventRecord(ev[i], H->stream));
    };
    auto report = [&](const char* form) {
      if (!verbose) return;
      float a = 0.f, b = 0.f, c = 0.f;
      cudaEventElapsedTime(&a, ev[0], ev[1]);
      cudaEventElapsedTime(&b, ev[1], ev[2]);
      cudaEventElapsedTime(&c, ev[2], ev[3]);
      std::fprintf(stderr, "qcmg_matvec: %s, x in %.3f ms, product %.3f ms, y %.3f ms\n", form, a, b,
                   c);
      for (auto& e : ev) cudaEventDestroy(e);
    };
    if (double* yh = pinned_device_address(y, n, H->device)) {
      // page-locked y: x is copied in, and the result goes straight into y
      // (the old y read while the new one is written), so y crosses the
      // link once in each direction at the same time
      mark(0);
      QCMG_CUDA(cudaMemcpyAsync(H->xbuf.p, x, n * 8, cudaMemcpyHostToDevice, H->stream));
      mark(1);
      if (fx) {
        // While the product runs the host->device direction is idle: copy
        // the first part of the old y then (about what the link moves in
        // the product's time, half of y on the fixed-point path), so that
        // part of y only has to go out at the end.
        size_t m = 0;
        if (acc) {
          m = (n / 2) & ~(size_t)1;
          if (!H->copy_stream) {
            QCMG_CUDA(cudaStreamCreateWithFlags(&H->copy_stream, cudaStreamNonBlocking));
            QCMG_CUDA(cudaEventCreateWithFlags(&H->ev_x, cudaEventDisableTiming));
            QCMG_CUDA(cudaEventCreateWithFlags(&H->ev_y, cudaEventDisableTiming));
          }
          H->ybuf.alloc(n);
          QCMG_CUDA(cudaEventRecord(H->ev_x, H->stream));  // after x: no contention for the link
          QCMG_CUDA(cudaStreamWaitEvent(H->copy_stream, H->ev_x, 0));
          QCMG_CUDA(cudaMemcpyAsync(H->ybuf.p, y, m * 8, cudaMemcpyHostToDevice, H->copy_stream));
          QCMG_CUDA(cudaEventRecord(H->ev_y, H->copy_stream));
        }
        fx_matvec_to_host(H, H->xbuf.p, yh, acc, verbose ? ev[2] : nullptr, H->ybuf.p, m,
                          m ? H->ev_y : nullptr);
      } else {
        H->ybuf.alloc(n);
        matvec(H, H->xbuf.p, H->ybuf.p, false);
        mark(2);
        k_add_to_host<<<152 * 8, 256, 0, H->stream>>>(H->ybuf.p, yh, n, acc ? 1 : 0);
        QCMG_CUDA(cudaGetLastError());
      }
      mark(3);
      QCMG_CUDA(cudaStreamSynchronize(H->stream));
      if (fx) fx_check_error(H);
      report("zero-copy y");
      return;
    }
    H->ybuf.alloc(n);
    mark(0);
    QCMG_CUDA(cudaMemcpyAsync(H->xbuf.p, x, n * 8, cudaMemcpyHostToDevice, H->stream));
    if (acc) QCMG_CUDA(cudaMemcpyAsync(H->ybuf.p, y, n * 8, cudaMemcpyHostToDevice, H->stream));
    mark(1);
    if (fx)
      fx_matvec_f64(H, H->xbuf.p, H->ybuf.p, acc);
    else
      matvec(H, H->xbuf.p, H->ybuf.p, acc);
    mark(2);
    QCMG_CUDA(cudaMemcpyAsync(y, H->ybuf.p, n * 8, cudaMemcpyDeviceToHost, H->stream));
    mark(3);
    QCMG_CUDA(cudaStreamSynchronize(H->stream));
    if (fx) fx_check_error(H);
    report("staged copies");
  });
}

int qcmg_hamiltonian_set_path(qcmg_hamiltonian* H, int path) {
  return guarded([&] {
    QCMG_CHECK_ARG(H != nullptr, "NULL handle");
    QCMG_CHECK_ARG(path == 0 || path == 1, "path must be 0 (FP64) or 1 (fixed point)");
    std::lock_guard<std::mutex> lock(H->mu);
    H->use_fx = path;
  });
}

int qcmg_hamiltonian_fx_available(qcmg_hamiltonian* H, int* available) {
  return guarded([&] {
    QCMG_CHECK_ARG(H != nullptr && available != nullptr, "NULL argument");
    std::lock_guard<std::mutex> lock(H->mu);
    QCMG_CUDA(cudaSetDevice(H->device));
    *available = fx_prepare(H) ? 1 : 0;
  });
}

int qcmg_fx_from_f64(size_t n, const double* x, int64_t* q, int* E, int* mb, void* stream) {
  return guarded([&] {
    QCMG_CHECK_ARG(x && q && E && mb, "NULL argument");
    cudaStream_t s = (cudaStream_t)stream;
    FxVec v;
    DevBuf<unsigned long long> tmp;
    fx_from_f64(x, n, v, s, tmp);
    if (n) QCMG_CUDA(cudaMemcpyAsync(q, v.buf.p, n * 8, cudaMemcpyDeviceToDevice, s));
    QCMG_CUDA(cudaStreamSynchronize(s));
    *E = v.E;
    *mb = v.mb;
  });
}

int qcmg_fx_to_f64(size_t n, const int64_t* q, int E, double* x, void* stream) {
  return guarded([&] {
    QCMG_CHECK_ARG(x && q, "NULL argument");
    cudaStream_t s = (cudaStream_t)stream;
    FxVec v;
    v.buf.borrow(const_cast<int64_t*>(q), n);
    v.n = n;
    v.E = E;
    v.c = 1.0;
    fx_to_f64(v, x, s);
    QCMG_CUDA(cudaStreamSynchronize(s));
  });
}

int qcmg_matvec_fx(qcmg_hamiltonian* H, const int64_t* qx, int Ex, int mbx, int64_t* qy, int* Ey,
                   unsigned flags) {
  return guarded([&] {
    QCMG_CHECK_ARG(H && qx && qy && Ey, "NULL argument");
    QCMG_CHECK_ARG(qx != qy, "x and y must not alias");
    QCMG_CHECK_ARG(mbx >= 0 && mbx <= 62, "invalid bit length");
    std::lock_guard<std::mutex> lock(H->mu);
    QCMG_CUDA(cudaSetDevice(H->device));
    QCMG_CHECK_ARG(fx_prepare(H), "this Hamiltonian has no fixed-point form (hop magnitudes differ)");
    FxVec x, y;
    x.buf.borrow(const_cast<int64_t*>(qx), H->dim);
    x.n = H->dim;
    x.E = Ex;
    x.mb = mbx;
    x.c = 1.0;
    y.buf.borrow(qy, H->dim);
    y.n = H->dim;
    if (flags & QCMG_ACCUMULATE) {
      // the input y, in place: pass U reads and writes each entry once
      FxVec yin;
      yin.buf.borrow(qy, H->dim);
      yin.n = H->dim;
      yin.E = *Ey;
      yin.mb = kFxBits;
      yin.c = 1.0;
      fx_matvec(H, x, y, &yin, 1.0);
    } else {
      fx_matvec(H, x, y, nullptr, 0.0);
    }
    *Ey = y.E;
    if (!(flags & QCMG_ASYNC)) fx_check_error(H);
  });
}

int qcmg_multidot(int m, const double* const* V, const double* w, size_t n, double* out,
                  void* stream) {
  return guarded([&] {
    QCMG_CHECK_ARG(m >= 0 && (m == 0 || (V && w && out)), "NULL argument");
    QCMG_CHECK_ARG(m <= 4096, "at most 4096 vectors per call");
    if (m == 0) return;
    use_device();
    cudaStream_t s = (cudaStream_t)stream;
    DevBuf<double> part, res;
    part.alloc((size_t)m * multidot_blocks(n));
    res.alloc(m);
    multidot_launch(m, V, w, n, part.p, res.p, s);
    QCMG_CUDA(cudaMemcpyAsync(out, res.p, m * sizeof(double), cudaMemcpyDeviceToHost, s));
    QCMG_CUDA(cudaStreamSynchronize(s));
  });
}

int qcmg_seeded_vector(size_t dim, unsigned seed, double* out) {
  return guarded([&] {
    QCMG_CHECK_ARG(out != nullptr || dim == 0, "NULL output");
    seeded_vector(dim, seed, out);
  });
}

int qcmg_lanczos_ground_state(qcmg_hamiltonian* H, const double* x0, unsigned seed, double tol,
                              int max_iter, int reorth, double* E0, double* psi, int* niter,
                              double* alpha, double* beta, int cap) {
  return guarded([&] {
    QCMG_CHECK_ARG(H != nullptr && E0 != nullptr, "NULL argument");
    QCMG_CHECK_ARG(tol > 0.0 && max_iter > 0, "tol and max_iter must be positive");
    std::lock_guard<std::mutex> lock(H->mu);
    QCMG_CUDA(cudaSetDevice(H->device));
    LanczosResult r = lanczos_ground_state(H, x0, seed, tol, max_iter, reorth, psi);
    *E0 = r.energy;
    if (niter) *niter = r.niter;
    const int nc = (int)r.alpha.size();  // the last cycle's coefficients
    for (int k = 0; k < std::min<int>(cap, nc); ++k) {
      if (alpha) alpha[k] = r.alpha[k];
      if (beta) beta[k] = r.beta[k];
    }
    H->last_product_ms = r.product_ms;
    H->last_reorth_ms = r.reorth_ms;
    H->last_reorth_bytes = r.reorth_bytes;
    H->last_restarts = r.restarts;
    H->last_vectors = r.vectors;
    H->last_cycle = nc;
  });
}

// Eight independent FMA chains per thread; the values stay bounded (a < 1)
// and the result is written only when it equals an impossible value, so the
// chains are not removed.
__global__ void k_fp64_fma(double* out, int iters, double a, double b) {
  double x[8];
  for (int k = 0; k < 8; ++k) x[k] = 1e-3 * (threadIdx.x + k);
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
  double s = 0.0;
  for (int k = 0; k < 8; ++k) s += x[k];
  if (s == -1.0) out[0] = s;
}

int qcmg_fp64_fma_rate(double* tflops) {
  return guarded([&] {
    QCMG_CHECK_ARG(tflops != nullptr, "NULL argument");
    int dev = 0, sms = 0;
    QCMG_CUDA(cudaGetDevice(&dev));
    QCMG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    DevBuf<double> out;
    out.alloc(1);
    cudaStream_t s;
    QCMG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    cudaEvent_t e0, e1;
    QCMG_CUDA(cudaEventCreate(&e0));
    QCMG_CUDA(cudaEventCreate(&e1));
    const int blocks = sms * 8, threads = 256, iters = 4096;
    k_fp64_fma<<<blocks, threads, 0, s>>>(out.p, iters, 0.9999999, 1e-7);  // warm-up
    QCMG_CUDA(cudaEventRecord(e0, s));
    k_fp64_fma<<<blocks, threads, 0, s>>>(out.p, iters, 0.9999999, 1e-7);
    QCMG_CUDA(cudaEventRecord(e1, s));
    QCMG_CUDA(cudaEventSynchronize(e1));
    QCMG_CUDA(cudaGetLastError());
    float ms = 0.f;
    QCMG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
  });
}

int qcmg_lanczos_last_stats(qcmg_hamiltonian* H, double* product_ms, double* reorth_ms,
                            double* reorth_bytes, int* restarts, int* vectors, int* cycle) {
  return guarded([&] {
    QCMG_CHECK_ARG(H != nullptr, "NULL handle");
    std::lock_guard<std::mutex> lock(H->mu);
    if (product_ms) *product_ms = H->last_product_ms;
    if (reorth_ms) *reorth_ms = H->last_reorth_ms;
    if (reorth_bytes) *reorth_bytes = H->last_reorth_bytes;
    if (restarts) *restarts = H->last_restarts;
    if (vectors) *vectors = H->last_vectors;
    if (cycle) *cycle = H->last_cycle;
  });
}

int qcmg_lanczos_green(qcmg_hamiltonian* H, const double* psi, unsigned flags, double accur,
                       int max_iter, int* n, double* a, double* b, int cap) {
  return guarded([&] {
    QCMG_CHECK_ARG(H != nullptr && psi != nullptr && n != nullptr, "NULL argument");
    QCMG_CHECK_ARG(accur > 0.0 && max_iter > 0, "accur and max_iter must be positive");
    std::lock_guard<std::mutex> lock(H->mu);
    QCMG_CUDA(cudaSetDevice(H->device));
    *n = 0;
    const bool dev = (flags & QCMG_DEVICE_PTRS) != 0;
    if (dev) QCMG_CUDA(cudaDeviceSynchronize());  // the vector may come from any stream
    GreenResult r = lanczos_green(H, psi, dev, accur, max_iter);
    *n = (int)r.a.size();
    QCMG_CHECK_ARG(*n <= cap, "continued-fraction output capacity too small");
    if (a) std::copy(r.a.begin(), r.a.end(), a);
    if (b) std::copy(r.b.begin(), r.b.end(), b);
  });
}

int qcmg_block_lanczos(qcmg_hamiltonian* H, int p, const double* phi, unsigned flags,
                       int M_target, int max_iter, double acc_deflation, double acc_band, int* M,
                       int* p_actual, double* A, double* B, double* W, int cap) {
  return guarded([&] {
    QCMG_CHECK_ARG(H != nullptr && phi != nullptr && M != nullptr && p_actual != nullptr,
                   "NULL argument");
    QCMG_CHECK_ARG(p > 0 && M_target > 0 && max_iter > 0, "invalid block Lanczos sizes");
    std::lock_guard<std::mutex> lock(H->mu);
    QCMG_CUDA(cudaSetDevice(H->device));
    *M = 0;
    *p_actual = 0;
    if (H->dim == 0) return;
    const bool dev = (flags & QCMG_DEVICE_PTRS) != 0;
    if (dev) QCMG_CUDA(cudaDeviceSynchronize());  // start vectors may come from any stream
    BlockResult r = block_lanczos(H, p, phi, dev, M_target, max_iter, acc_deflation, acc_band);
    QCMG_CHECK_ARG(r.M <= cap, "block Lanczos output capacity too small");
    *M = r.M;
    *p_actual = r.pa;
    if (A) std::copy(r.A.begin(), r.A.end(), A);
    if (B) std::copy(r.B.begin(), r.B.end(), B);
    if (W) std::copy(r.W.begin(), r.W.end(), W);
  });
}

static int band_lanczos_entry(qcmg_hamiltonian* H, int p, const double* phi, bool on_device,
                              int M_target, int max_iter, double acc_deflation, double acc_band,
                              int* M, double* evals, double* Q, int cap) {
  return guarded([&] {
    QCMG_CHECK_ARG(H != nullptr && phi != nullptr && M != nullptr, "NULL argument");
    QCMG_CHECK_ARG(p > 0 && M_target > 1 && max_iter > 0, "invalid band Lanczos sizes");
    std::lock_guard<std::mutex> lock(H->mu);
    QCMG_CUDA(cudaSetDevice(H->device));
    *M = 0;
    if (H->dim == 0) return;
    // device start vectors may come from any stream: wait for the device
    if (on_device) QCMG_CUDA(cudaDeviceSynchronize());
    BandResult r = band_lanczos(H, p, phi, on_device, M_target, max_iter, acc_deflation, acc_band);
    *M = r.M;
    QCMG_CHECK_ARG(r.M <= cap, "band Lanczos output capacity too small");
    if (evals) std::copy(r.evals.begin(), r.evals.end(), evals);
    if (Q) std::copy(r.Q.begin(), r.Q.end(), Q);
  });
}

int qcmg_band_lanczos(qcmg_hamiltonian* H, int p, const double* phi, int M_target, int max_iter,
                      double acc_deflation, double acc_band, int* M, double* evals, double* Q,
                      int cap) {
  return band_lanczos_entry(H, p, phi, false, M_target, max_iter, acc_deflation, acc_band, M,
                            evals, Q, cap);
}

int qcmg_band_lanczos_ptrs(qcmg_hamiltonian* H, int p, const double* const* phi, int M_target,
                           int max_iter, double acc_deflation, double acc_band, int* M,
                           double* evals, double* Q, int cap) {
  // each host vector goes straight to its row of one device block
  DevBuf<double> dev;
  const int rc = guarded([&] {
    QCMG_CHECK_ARG(H != nullptr && phi != nullptr && M != nullptr, "NULL argument");
    QCMG_CHECK_ARG(p > 0, "invalid band Lanczos sizes");
    std::lock_guard<std::mutex> lock(H->mu);
    QCMG_CUDA(cudaSetDevice(H->device));
    if (H->dim == 0) return;
    dev.alloc((size_t)p * H->dim);
    for (int k = 0; k < p; ++k) {
      QCMG_CHECK_ARG(phi[k] != nullptr, "NULL start vector");
      QCMG_CUDA(cudaMemcpyAsync(dev.p + (size_t)k * H->dim, phi[k], H->dim * 8,
                                cudaMemcpyHostToDevice, H->stream));
    }
    QCMG_CUDA(cudaStreamSynchronize(H->stream));
  });
  if (rc != QCMG_OK) return rc;
  if (H->dim == 0) {
    *M = 0;
    return QCMG_OK;
  }
  return band_lanczos_entry(H, p, dev.p, true, M_target, max_iter, acc_deflation, acc_band, M,
                            evals, Q, cap);
}

int qcmg_band_lanczos_device(qcmg_hamiltonian* H, int p, const double* phi_dev, int M_target,
                             int max_iter, double acc_deflation, double acc_band, int* M,
                             double* evals, double* Q, int cap) {
  return band_lanczos_entry(H, p, phi_dev, true, M_target, max_iter, acc_deflation, acc_band, M,
                            evals, Q, cap);
}

int qcmg_apply_c(int L, int orb, int pm, int n_up, int n_dn, const double* x, double* y, double z,
                 unsigned flags) {
  return guarded([&] {
    QCMG_CHECK_ARG(L >= 1 && L <= kMaxOrbitals, "L must be in 1..32");
    QCMG_CHECK_ARG(orb >= 0 && orb < 2 * L, "orbital out of range");
    QCMG_CHECK_ARG(pm == 1 || pm == -1, "pm must be +1 or -1");
    QCMG_CHECK_ARG(n_up >= 0 && n_up <= L && n_dn >= 0 && n_dn <= L, "electron count out of range");
    QCMG_CHECK_ARG(x && y, "NULL vector");
    const int spin = orb >= L ? 1 : 0, o = spin ? orb - L : orb;
    const int nup2 = n_up + (spin ? 0 : pm), ndn2 = n_dn + (spin ? pm : 0);
    const size_t n1 = (size_t)binomial(L, n_up) * binomial(L, n_dn);
    const size_t n2 = (nup2 < 0 || ndn2 < 0 || nup2 > L || ndn2 > L)
                          ? 0
                          : (size_t)binomial(L, nup2) * binomial(L, ndn2);
    if (n2 == 0) return;
    use_device();
    const bool acc = (flags & QCMG_ACCUMULATE) != 0;
    if (flags & QCMG_DEVICE_PTRS) {
      launch_apply_c(L, o, spin, pm, n_up, n_dn, x, y, z, acc, 0);
      QCMG_CUDA(cudaStreamSynchronize(0));
      return;
    }
    DevBuf<double> dx, dy;
    dx.upload(x, n1, 0);
    if (acc)
      dy.upload(y, n2, 0);
    else
      dy.alloc(n2);
    launch_apply_c(L, o, spin, pm, n_up, n_dn, dx.p, dy.p, z, acc, 0);
    QCMG_CUDA(cudaMemcpy(y, dy.p, n2 * 8, cudaMemcpyDeviceToHost));
  });
}

int qcmg_green_function(int L, int M, const double* e, const double* v, int nz, const double* z,
                        double* G) {
  return guarded([&] {
    QCMG_CHECK_ARG(L > 0 && M >= 0 && nz >= 0, "invalid sizes");
    QCMG_CHECK_ARG(z && G && (M == 0 || (e && v)), "NULL argument");
    if (nz == 0) return;
    if (M == 0) {
      std::fill(G, G + (size_t)2 * L * L * nz, 0.0);
      return;
    }
    use_device();
    DevBuf<double> de, dv, dz, dG;
    de.upload(e, M, 0);
    dv.upload(v, (size_t)2 * L * M, 0);
    dz.upload(z, (size_t)2 * nz, 0);
    dG.alloc((size_t)2 * L * L * nz);
    green_function_batch(L, M, de.p, dv.p, nz, dz.p, dG.p, 0);
    QCMG_CUDA(cudaMemcpy(G, dG.p, (size_t)2 * L * L * nz * 8, cudaMemcpyDeviceToHost));
  });
}

int qcmg_self_energy(int L, int M, const double* e, const double* v, int nb, const double* tcb,
                     const double* eb, const double* tc, int nz, const double* z, double* sigma,
                     double* gamma) {
  return guarded([&] {
    QCMG_CHECK_ARG(L > 0 && L <= 32 && M >= 0 && nb >= 0 && nz >= 0, "invalid sizes");
    QCMG_CHECK_ARG(tc && z && sigma && (M == 0 || (e && v)) && (nb == 0 || (tcb && eb)),
                   "NULL argument");
    if (nz == 0) return;
    use_device();
    DevBuf<double> de, dv, dtcb, deb, dtc, dz, ds, dg;
    if (M) {
      de.upload(e, M, 0);
      dv.upload(v, (size_t)2 * L * M, 0);
    }
    if (nb) {
      dtcb.upload(tcb, (size_t)2 * L * nb, 0);
      deb.upload(eb, nb, 0);
    }
    dtc.upload(tc, (size_t)2 * L * L, 0);
    dz.upload(z, (size_t)2 * nz, 0);
    ds.alloc((size_t)2 * L * L * nz);
    if (gamma) dg.alloc((size_t)2 * L * L * nz);
    self_energy_batch(L, M, de.p, dv.p, nb, dtcb.p, deb.p, dtc.p, nz, dz.p, ds.p,
                      gamma ? dg.p : nullptr, 0);
    QCMG_CUDA(cudaMemcpy(sigma, ds.p, (size_t)2 * L * L * nz * 8, cudaMemcpyDeviceToHost));
    if (gamma) QCMG_CUDA(cudaMemcpy(gamma, dg.p, (size_t)2 * L * L * nz * 8, cudaMemcpyDeviceToHost));
  });
}

int qcmg_lattice_create(int L, int nR, const double* R, int nel, const int32_t* el_r,
                        const int32_t* el_c, const int32_t* el_n, const double* el_v,
                        const double* hdiff, const double* gpos, qcmg_lattice** out) {
  return guarded([&] {
    QCMG_CHECK_ARG(out != nullptr, "out is NULL");
    *out = nullptr;
    QCMG_CHECK_ARG(L >= 1 && L <= 32, "L must be in 1..32");
    QCMG_CHECK_ARG(nR >= 1 && R != nullptr, "at least one superlattice translation (R[0] = 0)");
    QCMG_CHECK_ARG(nel >= 0 && (nel == 0 || (el_r && el_c && el_n && el_v)), "NULL element array");
    QCMG_CHECK_ARG(hdiff && gpos, "NULL argument");
    for (int k = 0; k < nel; ++k)
      QCMG_CHECK_ARG(el_r[k] >= 0 && el_r[k] < L && el_c[k] >= 0 && el_c[k] < L && el_n[k] >= 0 &&
                         el_n[k] < nR,
                     "lattice element index out of range");
    use_device();
    auto* h = new qcmg_lattice();
    try {
      Lattice& t = h->lat;
      t.device = g_device;
      t.L = L;
      t.nR = nR;
      t.nel = nel;
      QCMG_CUDA(cudaStreamCreateWithFlags(&t.stream, cudaStreamNonBlocking));
      t.R.upload(R, (size_t)3 * nR, t.stream);
      t.gpos.upload(gpos, (size_t)3 * L, t.stream);
      t.hdiff.upload(hdiff, (size_t)2 * L * L, t.stream);
      // elements grouped by translation: each point then computes one phase
      // per translation instead of one per element
      std::vector<int> order(nel);
      for (int k = 0; k < nel; ++k) order[k] = k;
      std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return el_n[a] < el_n[b]; });
      std::vector<int> r(nel), c(nel), n(nel), start(nR + 1, 0);
      std::vector<double> v((size_t)2 * nel);
      for (int k = 0; k < nel; ++k) {
        const int o = order[k];
        r[k] = el_r[o];
        c[k] = el_c[o];
        n[k] = el_n[o];
        v[2 * k] = el_v[2 * o];
        v[2 * k + 1] = el_v[2 * o + 1];
        start[n[k] + 1]++;
      }
      for (int q = 0; q < nR; ++q) start[q + 1] += start[q];
      t.el_start.upload(start.data(), nR + 1, t.stream);
      t.R_host.assign(R, R + (size_t)3 * nR);
      if (nel) {
        t.el_r.upload(r.data(), nel, t.stream);
        t.el_c.upload(c.data(), nel, t.stream);
        t.el_n.upload(n.data(), nel, t.stream);
        t.el_v.upload(v.data(), (size_t)2 * nel, t.stream);
      }
      QCMG_CUDA(cudaStreamSynchronize(t.stream));
    } catch (...) {
      if (h->lat.stream) cudaStreamDestroy(h->lat.stream);
      delete h;
      throw;
    }
    *out = h;
  });
}

int qcmg_lattice_destroy(qcmg_lattice* h) {
  return guarded([&] {
    if (!h) return;
    cudaSetDevice(h->lat.device);
    if (h->lat.stream) {
      cudaStreamSynchronize(h->lat.stream);
      cudaStreamDestroy(h->lat.stream);
    }
    delete h;
  });
}

int qcmg_lattice_set_green(qcmg_lattice* h, int M, const double* e, const double* v, int nb,
                           const double* tcb, const double* eb) {
  return guarded([&] {
    QCMG_CHECK_ARG(h != nullptr, "NULL handle");
    QCMG_CHECK_ARG(M >= 0 && nb >= 0, "negative size");
    QCMG_CHECK_ARG((M == 0 || (e && v)) && (nb == 0 || (tcb && eb)), "NULL array");
    std::lock_guard<std::mutex> lock(h->mu);
    Lattice& t = h->lat;
    QCMG_CUDA(cudaSetDevice(t.device));
    t.M = M;
    if (M) {
      t.e.upload(e, M, t.stream);
      t.v.upload(v, (size_t)2 * t.L * M, t.stream);
    }
    t.nb = nb;
    if (nb) {
      t.tcb.upload(tcb, (size_t)2 * t.L * nb, t.stream);
      t.eb.upload(eb, nb, t.stream);
    } else {
      t.tcb.alloc(2);
      t.eb.alloc(1);
    }
    QCMG_CUDA(cudaStreamSynchronize(t.stream));
  });
}

int qcmg_sef_grid(qcmg_lattice* h, int nw, const double* w, const double* wt, int nkx, int nky,
                  int nkz, double* out) {
  return guarded([&] {
    QCMG_CHECK_ARG(h && w && wt && out, "NULL argument");
    QCMG_CHECK_ARG(nw > 0 && nkx > 0 && nky > 0 && nkz > 0, "invalid grid");
    std::lock_guard<std::mutex> lock(h->mu);
    QCMG_CHECK_ARG(h->lat.M >= 0, "the Green function was not set");
    QCMG_CUDA(cudaSetDevice(h->lat.device));
    *out = h->lat.sef_grid(nw, w, wt, nkx, nky, nkz, h->lat.stream);
  });
}

int qcmg_cpt_periodized(qcmg_lattice* h, int nz, const double* z, int nk, const double* K,
                        double* g) {
  return guarded([&] {
    QCMG_CHECK_ARG(h && z && K && g, "NULL argument");
    QCMG_CHECK_ARG(nz > 0 && nk > 0, "invalid sizes");
    std::lock_guard<std::mutex> lock(h->mu);
    QCMG_CHECK_ARG(h->lat.M >= 0, "the Green function was not set");
    QCMG_CUDA(cudaSetDevice(h->lat.device));
    h->lat.cpt(nz, z, nk, K, g, h->lat.stream);
  });
}

int qcmg_lattice_kmean(qcmg_lattice* h, int nz, const double* z, int nkx, int nky, int nkz,
                       double off, double* out) {
  return guarded([&] {
    QCMG_CHECK_ARG(h && z && out, "NULL argument");
    QCMG_CHECK_ARG(nz > 0 && nkx > 0 && nky > 0 && nkz > 0, "invalid sizes");
    std::lock_guard<std::mutex> lock(h->mu);
    QCMG_CHECK_ARG(h->lat.M >= 0, "the Green function was not set");
    QCMG_CUDA(cudaSetDevice(h->lat.device));
    h->lat.kmean(nz, z, nkx, nky, nkz, off, out, h->lat.stream);
  });
}

int qcmg_lattice_kmoments(qcmg_lattice* h, int nz, const double* z, int nkx, int nky, int nkz,
                          double off, int nmom, const double* R, double* out) {
  return guarded([&] {
    QCMG_CHECK_ARG(h && z && out && R, "NULL argument");
    QCMG_CHECK_ARG(nz > 0 && nkx > 0 && nky > 0 && nkz > 0, "invalid sizes");
    QCMG_CHECK_ARG(nmom >= 1 && nmom <= 16, "nmom must be 1..16");
    std::lock_guard<std::mutex> lock(h->mu);
    QCMG_CHECK_ARG(h->lat.M >= 0, "the Green function was not set");
    QCMG_CUDA(cudaSetDevice(h->lat.device));
    h->lat.kmoments(nz, z, nkx, nky, nkz, off, nmom, R, out, h->lat.stream);
  });
}

int qcmg_cdmft_projected(qcmg_lattice* h, int nw, const double* w, int kside, int dimk,
                         double* pgf) {
  return guarded([&] {
    QCMG_CHECK_ARG(h && w && pgf, "NULL argument");
    QCMG_CHECK_ARG(nw > 0 && kside > 0 && dimk >= 0 && dimk <= 3, "invalid sizes");
    std::lock_guard<std::mutex> lock(h->mu);
    QCMG_CHECK_ARG(h->lat.M >= 0, "the Green function was not set");
    QCMG_CUDA(cudaSetDevice(h->lat.device));
    h->lat.projected(nw, w, kside, dimk, pgf, h->lat.stream);
  });
}

}  // extern "C"
