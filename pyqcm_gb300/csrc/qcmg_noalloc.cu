// qcmg_multidot_noalloc: the multi-vector dot product of qcmg_multidot with
// no device allocation at all.
//
// Who needs it: a caller that may not call cudaMalloc.  Examples are a host
// framework that hands the whole GPU to its own memory pool (or runs under a
// hard memory cap), where a stray allocation fails or fragments the pool,
// and code that must not allocate while other work is in flight, since
// cudaMalloc/cudaFree can synchronize the device.  qcmg_multidot allocates
// its per-block partial sums for every call; this entry point runs the same
// two kernels with the partial sums kept in a fixed file-scope device array.
// The caller still owns every input and the output.
//
// Set-up: the first call on a device (with that device current) looks up
// the array's device address with cudaGetSymbolAddress and caches it,
// together with the device's current context; do that first call before any
// stream capture.  Later calls only launch.  The array itself is reserved
// when CUDA loads this library's module on the device: under lazy module
// loading (CUDA_MODULE_LOADING=LAZY, the default) that happens at this first
// call, so make it before handing the GPU's memory to a pool or a cap.  A
// new context on the device (after cudaDeviceReset) makes the next call look
// the address up again.
//
// The call runs on the calling thread's current CUDA device (it does not
// switch to the device chosen with qcmg_set_device, which may allocate).
//
// One scratch array per device: calls that overlap in time on one device
// (from several host threads or several streams) race on it and must be
// serialized by the caller.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "qcmg.h"
#include "qcmg_internal.h"
#include "qcmg_krylov.h"

namespace qcmg {

// Limits of the scratch: at most kNoAllocVectors vectors per call, and a
// multi-dot never uses more than kNoAllocBlocks blocks (multidot_blocks).
constexpr int kNoAllocVectors = 64;
constexpr int kNoAllocBlocks = 2 * 152;

// 64 x 304 doubles = 155,648 bytes of device memory, reserved when the
// module is loaded on a device (see above) and held until the process exits.
static __device__ __align__(256) double g_multidot_scratch[kNoAllocVectors * kNoAllocBlocks];

// In host code, g_multidot_scratch names a host-side shadow, not device
// memory: handing it to a kernel would read the wrong memory.  Kernels get
// the device address, looked up once per device with that device current.
static std::mutex g_scratch_mu;
static double* g_scratch_addr[256] = {nullptr};
static void* g_scratch_ctx[256] = {nullptr};

// cuCtxGetCurrent through the runtime's driver entry point (no link against
// the driver library); null when the driver does not provide it.
typedef int (*CtxGetCurrentFn)(void**);
static CtxGetCurrentFn ctx_get_current() {
  static CtxGetCurrentFn fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<CtxGetCurrentFn>(f);
  }();
  return fn;
}

static double* scratch_on(int device) {
  QCMG_CHECK_ARG(device >= 0 && device < 256, "device index out of range");
  void* ctx = nullptr;
  if (CtxGetCurrentFn f = ctx_get_current()) (void)f(&ctx);
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[device] || g_scratch_ctx[device] != ctx) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_multidot_scratch);
    if (e != cudaSuccess)
      throw Error(QCMG_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_scratch_addr[device] = static_cast<double*>(p);
    g_scratch_ctx[device] = ctx;
  }
  return g_scratch_addr[device];
}

}  // namespace qcmg

using namespace qcmg;

extern "C" int qcmg_multidot_noalloc(int m, const double* const* V, const double* w, size_t n,
                                     double* out, void* stream) {
  try {
    clear_error();
    QCMG_CHECK_ARG(m >= 0, "m must not be negative");
    if (m == 0) return QCMG_OK;  // as qcmg_multidot
    QCMG_CHECK_ARG(m <= kNoAllocVectors,
                   "qcmg_multidot_noalloc takes at most 64 vectors (its scratch is a fixed "
                   "device array); use qcmg_multidot for more");
    QCMG_CHECK_ARG(V && w && out, "NULL argument");
    QCMG_CHECK_ARG(multidot_blocks(n) <= kNoAllocBlocks, "block count exceeds the scratch");
    int device = 0;
    QCMG_CUDA(cudaGetDevice(&device));
    double* scratch = scratch_on(device);
    // Nothing starts at zero: the first kernel writes every partial sum the
    // second one reads, in this same call.
    multidot_launch(m, V, w, n, scratch, out, static_cast<cudaStream_t>(stream));
    return QCMG_OK;
  } catch (const Error& e) {
    set_error(e.what());
    return e.code;
  } catch (const std::exception& e) {
    set_error(e.what());
    return QCMG_ERR_CUDA;
  }
}
