// Vector kernels of the Krylov solvers (host launch wrappers).
#pragma once

#include <functional>

#include "qcmg_internal.h"

namespace qcmg {

constexpr int kRedThreads = 256;  // threads per reduction block
constexpr int kRedBlocks = 1024;  // fixed partial count of a reduction

// Deterministic dot products and norms: fixed grid, fixed-order final sum.
// Holds its own scratch: one Reducer per handle (not shared across threads).
struct Reducer {
  DevBuf<double> part;
  DevBuf<double> out;
  double* host = nullptr;  // pinned
  Reducer() = default;
  Reducer(const Reducer&) = delete;
  ~Reducer();
  void init();
  double dot(const double* x, const double* y, size_t n, cudaStream_t s);
  // x . y (same partials and summation order as dot) written to out_dev,
  // without a host round trip.
  void dot_dev(const double* x, const double* y, size_t n, double* out_dev, cudaStream_t s);
  // r -= alpha q; returns |r|^2.
  double axpy_norm2(double* r, const double* q, double alpha, size_t n, cudaStream_t s);
};

void axpy(double* y, const double* x, double a, size_t n, cudaStream_t s);
// y -= (*a_dev) x, bitwise the same as axpy(y, x, -(*a_dev), ...).
void axpy_neg_dev(double* y, const double* x, const double* a_dev, size_t n, cudaStream_t s);
void scale2(double* r, double s1, double* q, double s2, size_t n, cudaStream_t s);
void scale(double* x, double a, size_t n, cudaStream_t s);
void replay_step(double* r, double* q, double* gs, double alpha, double beta, double c, size_t n,
                 cudaStream_t s);

// Device state of a Lanczos recurrence whose step index and coefficients
// stay on the device (for step sequences captured in a CUDA graph).
struct LanczosDevState {
  double* alpha;  // cap
  double* beta;   // cap
  double* part;   // kRedBlocks partial sums
  int* j;         // steps done
  int* done;      // nonzero: every step kernel returns at once
  int cap;
};

// One recurrence step of LanczosEigenvalue on (r, q) with the scalars on
// the device, appended to a graph chain: r /= beta[j-1], q *= -beta[j-1]
// (j > 0); q += H r (product, which appends its own node); alpha[j] =
// <r, q>; q -= alpha[j] r; beta[j] = |q|; j += 1.  The next step takes
// (q, r): the two buffers swap roles every step.
void lanczos_step_nodes(const LanczosDevState& st, double* r, double* q, size_t n, GraphChain& gc,
                        const std::function<void(const double*, double*)>& product);

}  // namespace qcmg
