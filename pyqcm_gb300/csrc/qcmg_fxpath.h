// FX64 fast path (fixed-point Krylov vectors): host-side declarations.
#pragma once

#include <cstdint>

#include "qcmg_internal.h"
#include "qcmg_krylov.h"

namespace qcmg {

struct I128;

struct FxReducer {
  DevBuf<I128> part;
  DevBuf<I128> out;
  DevBuf<unsigned long long> umax;
  double dot(const FxVec& a, const FxVec& b, cudaStream_t s);
};

// Prepares the fixed-point tables; false if the Hamiltonian does not have
// one hop magnitude per spin (then the FP64 path is used).
bool fx_prepare(qcmg_hamiltonian* H);
void fx_from_f64(const double* x, size_t n, FxVec& v, cudaStream_t s,
                 DevBuf<unsigned long long>& tmp);
void fx_to_f64(const FxVec& v, double* x, cudaStream_t s);
// With dot set, also returns <x, y> for the finished y (computed by the
// product's second pass, bit-identical to FxReducer::dot(x, y)).
void fx_matvec(qcmg_hamiltonian* H, const FxVec& x, FxVec& y, const FxVec* yin, double gamma,
               FxReducer* dot = nullptr, double* dot_out = nullptr);
// Throws if a kernel of the fast path reported a bounded-wait failure.
void fx_check_error(qcmg_hamiltonian* H);
// y (+)= H x on FP64 device vectors through the fixed-point product.
void fx_matvec_f64(qcmg_hamiltonian* H, const double* x, double* y, bool accumulate);
// y (+)= H x with x on the device and y in page-locked host memory, written
// through its device-side address yh (zero copy); product_done (optional) is
// recorded between the product and the pass into y.  With m > 0, the old
// values of y's first m elements are read from ypre on the device (a
// prefetched copy, complete once ypre_ready fires) instead of host memory.
void fx_matvec_to_host(qcmg_hamiltonian* H, const double* x, double* yh, bool accumulate,
                       cudaEvent_t product_done = nullptr, const double* ypre = nullptr,
                       size_t m = 0, cudaEvent_t ypre_ready = nullptr);
LanczosResult fx_lanczos(qcmg_hamiltonian* H, const double* x0_dev, double tol, int max_iter,
                         double* psi_dev);

}  // namespace qcmg
