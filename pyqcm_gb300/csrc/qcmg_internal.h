// Internal declarations of the qcmg engine (not part of the C ABI).
#pragma once

#include <tuple>
#include <utility>

#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "qcmg.h"

namespace qcmg {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void set_error(const std::string& msg);
void clear_error();

#define QCMG_CUDA(call)                                                                 \
  do {                                                                                  \
    cudaError_t err_ = (call);                                                          \
    if (err_ != cudaSuccess)                                                            \
      throw ::qcmg::Error(err_ == cudaErrorMemoryAllocation ? QCMG_ERR_NOMEM : QCMG_ERR_CUDA, \
                          std::string(#call) + ": " + cudaGetErrorString(err_));        \
  } while (0)

#define QCMG_CHECK_ARG(cond, msg) \
  do {                            \
    if (!(cond)) throw ::qcmg::Error(QCMG_ERR_ARG, msg); \
  } while (0)

// Owning device buffer.
template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  bool owned = true;  // false: p belongs to the caller and is never freed here
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p && owned) cudaFree(p);
    p = nullptr;
    n = 0;
    owned = true;
  }
  // Wraps caller-owned device memory.
  void borrow(T* ptr, size_t count) {
    release();
    p = ptr;
    n = count;
    owned = false;
  }
  void alloc(size_t count) {
    if (count <= n && p) return;
    QCMG_CHECK_ARG(owned, "cannot grow a borrowed buffer");
    release();
    size_t bytes = (count ? count : 1) * sizeof(T);
    QCMG_CUDA(cudaMalloc(&p, bytes));
    n = count;
  }
  void upload(const T* h, size_t count, cudaStream_t s) {
    alloc(count);
    if (count) QCMG_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
  }
};

// Largest orbital count a half-state can hold (uint32 bit masks).
constexpr int kMaxOrbitals = 32;

// Per-device one-time set-up (binomial table in constant memory).
void ensure_device_tables(int device);

// Half-operator of one spin on the device, CSR rows indexed by the input
// state: row I lists (J, value) for every hop I -> J, plus the diagonal.
struct HalfOp {
  int L = 0, N = 0;
  uint32_t dim = 0;
  size_t nnz = 0;
  DevBuf<uint32_t> bin;     // basis states, increasing
  DevBuf<uint32_t> rowptr;  // dim + 1
  DevBuf<uint32_t> col;     // nnz
  DevBuf<double> val;       // nnz
  DevBuf<double> diag;      // dim
  double max_row_abs = 0.0; // max_I sum_J |val| (for fixed-point headroom)
  double max_diag_abs = 0.0;
};

struct HopElement {
  int32_t r, c;
  double v;
};

// Device kernels launched from host code (defined in .cu files).
void launch_halfbasis(int L, int N, uint32_t dim, uint32_t* out, cudaStream_t s);
void launch_rank(int L, const uint32_t* states, size_t n, uint32_t dim, uint32_t* ranks,
                 cudaStream_t s);
void build_halfop(HalfOp& op, int L, int N, const std::vector<HopElement>& el, cudaStream_t s);

uint64_t binomial(int n, int k);

}  // namespace qcmg

// Interaction diagonal kinds.
enum { QCMG_INTER_NONE = 0, QCMG_INTER_ONSITE = 1, QCMG_INTER_GENERAL = 2 };

namespace qcmg {
// Device vector of the fixed-point fast path: value_i = c * 2^E * q_i with
// |q_i| < 2^mb.
struct FxVec {
  DevBuf<int64_t> buf;
  size_t n = 0;
  int E = 0;
  int mb = 0;
  double c = 1.0;
  void alloc(size_t count);
};

// Tables of the fixed-point product (built on first use by fx_prepare).
struct FxTables {
  int state = 0;  // 0 not built, 1 usable, -1 not applicable
  DevBuf<uint32_t> rp_up, rs_up, col_up, rp_dn, rs_dn, col_dn;
  double t_up = 0.0, t_dn = 0.0;  // hop magnitude of each spin
  int maxdeg_up = 0, maxdeg_dn = 0;
  DevBuf<int64_t> dup, ddn, wdn;  // diagonal in units of 2^-G
  int64_t U = 0;
  int G = 0;
  int dtz = -1;  // >= 0: every diagonal entry is a multiple of 2^dtz with |D| >> dtz < 2^6
  DevBuf<int32_t> dup32, ddn32, wdn32;  // the diagonal tables >> dtz (when dtz >= 0)
  int32_t U32 = 0;
  double bound = 0.0;  // bound on |H|_inf
  int b = 0;
  uint32_t band = 0;  // rows per band of the down-spin pass
  DevBuf<uint2> ell4;     // grouped ELL form of the up hops (pass U with bulk copies)
  DevBuf<uint16_t> cnt4;  // groups per row of ell4
  int ns = 0;             // slabs per pass U round: 0 (threads stage the slab), 1 or 2
  DevBuf<int> err;                  // bounded-wait failure flag of the kernels
  FxVec x, y;         // staging of the FP64-interface product
  DevBuf<unsigned long long> tmp;
};
}  // namespace qcmg

struct qcmg_hamiltonian {
  int device = 0;
  int L = 0, nup = 0, ndn = 0;
  uint32_t du = 0, dd = 0;
  size_t dim = 0;
  qcmg::HalfOp up, dn;
  int inter_kind = QCMG_INTER_NONE;
  double U = 0.0;                 // uniform on-site value (QCMG_INTER_ONSITE)
  qcmg::DevBuf<double> wdn;       // dd x L cross terms (QCMG_INTER_GENERAL)
  double max_inter_abs = 0.0;
  cudaStream_t stream = nullptr;      // stream the handle launches on
  cudaStream_t own_stream = nullptr;  // created with the handle
  // staging for host-pointer calls; the copy stream and its events prefetch
  // the old y while the product runs (created on first use)
  qcmg::DevBuf<double> xbuf, ybuf;
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_x = nullptr, ev_y = nullptr;
  // the seeded Lanczos start vector of the last seed used (generated once)
  qcmg::DevBuf<double> seed_vec;
  unsigned seed_key = 0;
  bool seed_ok = false;
  // deterministic reduction scratch
  qcmg::DevBuf<double> partials;
  qcmg::DevBuf<double> scalars;
  qcmg::FxTables fx;
  int use_fx = 1;  // 1: fixed-point fast path when applicable; 0: FP64 kernels
  // breakdown of the last reorthogonalized Lanczos solve on this handle
  double last_product_ms = 0.0, last_reorth_ms = 0.0, last_reorth_bytes = 0.0;
  int last_restarts = 0, last_vectors = 0, last_cycle = 0;
  std::mutex mu;   // serializes calls on one handle
};

namespace qcmg {
// Matrix-free factorized product y (+)= H x on the handle's stream.
void matvec(qcmg_hamiltonian* H, const double* x, double* y, bool accumulate);
// A chain of kernel nodes added to a CUDA graph explicitly (no stream
// capture, so no other host thread's device-wide synchronization can
// invalidate it): each node depends on the previous one.
struct GraphChain {
  cudaGraph_t graph = nullptr;
  cudaGraphNode_t last = nullptr;
  template <class... KArgs, class... Args>
  void add(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, Args... args) {
    static_assert(sizeof...(KArgs) == sizeof...(Args), "argument count");
    add_impl(kern, grid, block, smem, std::index_sequence_for<KArgs...>{},
             std::tuple<KArgs...>(args...));
  }

 private:
  template <class... KArgs, size_t... I>
  void add_impl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem,
                std::index_sequence<I...>, std::tuple<KArgs...> vals) {
    void* ptrs[sizeof...(KArgs) > 0 ? sizeof...(KArgs) : 1] = {(void*)&std::get<I>(vals)...};
    cudaKernelNodeParams p = {};
    p.func = (void*)kern;
    p.gridDim = grid;
    p.blockDim = block;
    p.sharedMemBytes = (unsigned)smem;
    p.kernelParams = ptrs;
    p.extra = nullptr;
    cudaGraphNode_t node;
    QCMG_CUDA(cudaGraphAddKernelNode(&node, graph, last ? &last : nullptr, last ? 1 : 0, &p));
    last = node;
  }
};

// The FP64 product y (+)= H x as one kernel node of a graph chain.
void matvec_node(qcmg_hamiltonian* H, const double* x, double* y, bool accumulate, GraphChain& gc);
}  // namespace qcmg
