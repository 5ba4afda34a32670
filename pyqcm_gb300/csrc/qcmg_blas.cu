// Vector kernels of the Krylov solvers, FP64, with deterministic reductions:
// every reduction writes one partial per block of a fixed-size grid and a
// single block then sums the partials in a fixed tree order, so alpha/beta of
// a Lanczos run are bitwise reproducible run to run (replaces the BLAS-1 calls
// of src_util/vector_num.cpp:37-106 used by src_ed/Hamiltonian/Lanczos.hpp).
#include "qcmg_blas.h"

namespace qcmg {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum in a fixed order; result valid in thread 0.
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double ws[32];
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) ws[w] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  v = (threadIdx.x < nw) ? ws[threadIdx.x] : 0.0;
  if (w == 0) v = warp_sum(v);
  return v;
}

__global__ void __launch_bounds__(kRedThreads) k_dot_partial(const double* __restrict__ x,
                                                             const double* __restrict__ y,
                                                             size_t n, double* __restrict__ part) {
  double s = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    s = fma(x[i], y[i], s);
  s = block_sum(s);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kRedBlocks) k_reduce_final(const double* __restrict__ part,
                                                             int np, double* __restrict__ out) {
  double s = (threadIdx.x < np) ? part[threadIdx.x] : 0.0;
  s = block_sum(s);
  if (threadIdx.x == 0) *out = s;
}

// r -= alpha q, accumulating |r|^2 partials.
__global__ void __launch_bounds__(kRedThreads) k_axpy_norm(double* __restrict__ r,
                                                           const double* __restrict__ q,
                                                           double alpha, size_t n,
                                                           double* __restrict__ part) {
  double s = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    double v = fma(-alpha, q[i], r[i]);
    r[i] = v;
    s = fma(v, v, s);
  }
  s = block_sum(s);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void k_axpy(double* __restrict__ y, const double* __restrict__ x, double a, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    y[i] = fma(a, x[i], y[i]);
}

// y -= a x with a read from device memory (a scalar left there by a
// reduction, so the host need not wait for it).
__global__ void k_axpy_neg_dev(double* __restrict__ y, const double* __restrict__ x,
                               const double* __restrict__ a, size_t n) {
  const double c = -*a;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    y[i] = fma(c, x[i], y[i]);
}

__global__ void k_scale2(double* __restrict__ r, double s1, double* __restrict__ q, double s2,
                         size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    r[i] *= s1;
    q[i] *= s2;
  }
}

__global__ void k_scale(double* __restrict__ x, double s, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    x[i] *= s;
}

// One step of the eigenvector replay (LanczosEigenvector,
// src_ed/Hamiltonian/Lanczos.hpp:120-130) after q += H r:
//   q -= alpha r;  (r, q) = (q / beta, -beta r);  gs += c r
__global__ void k_replay(double* __restrict__ r, double* __restrict__ q, double* __restrict__ gs,
                         double alpha, double beta, double c, size_t n) {
  const double ib = 1.0 / beta;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    double ri = r[i];
    double qi = fma(-alpha, ri, q[i]);
    double rn = qi * ib;
    r[i] = rn;
    q[i] = -beta * ri;
    gs[i] = fma(c, rn, gs[i]);
  }
}

// Device-scalar forms of the Lanczos recurrence for captured step sequences:
// the step index *jp and the coefficients alpha[], beta[] live in device
// memory, and a set *done turns each kernel into a no-op.  Same arithmetic,
// grids and summation order as scale2 / Reducer::dot / Reducer::axpy_norm2,
// so a captured run reproduces the host-driven one bit for bit.
__global__ void k_lzb_scale2(double* __restrict__ r, double* __restrict__ q, size_t n,
                             const double* __restrict__ beta, const int* __restrict__ jp,
                             const int* __restrict__ done) {
  if (*done) return;
  const int j = *jp;
  if (j == 0) return;
  const double b = beta[j - 1], s1 = 1.0 / b, s2 = -b;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    r[i] *= s1;
    q[i] *= s2;
  }
}

__global__ void __launch_bounds__(kRedThreads) k_lzb_dot_partial(const double* __restrict__ x,
                                                                 const double* __restrict__ y,
                                                                 size_t n, double* __restrict__ part,
                                                                 const int* __restrict__ done) {
  if (*done) return;
  double s = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    s = fma(x[i], y[i], s);
  s = block_sum(s);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kRedBlocks) k_lzb_alpha(const double* __restrict__ part, int np,
                                                          double* __restrict__ alpha,
                                                          const int* __restrict__ jp,
                                                          const int* __restrict__ done) {
  if (*done) return;
  double s = (threadIdx.x < np) ? part[threadIdx.x] : 0.0;
  s = block_sum(s);
  if (threadIdx.x == 0) alpha[*jp] = s;
}

__global__ void __launch_bounds__(kRedThreads) k_lzb_axpy_norm(double* __restrict__ r,
                                                               const double* __restrict__ q,
                                                               size_t n,
                                                               const double* __restrict__ alpha,
                                                               const int* __restrict__ jp,
                                                               double* __restrict__ part,
                                                               const int* __restrict__ done) {
  if (*done) return;
  const double a = alpha[*jp];
  double s = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    double v = fma(-a, q[i], r[i]);
    r[i] = v;
    s = fma(v, v, s);
  }
  s = block_sum(s);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// beta[j] = sqrt(sum of the partials), then j <- j + 1; the run stops
// itself (done = 2) when j reaches the coefficient arrays' capacity.
__global__ void __launch_bounds__(kRedBlocks) k_lzb_beta(const double* __restrict__ part, int np,
                                                         double* __restrict__ beta,
                                                         int* __restrict__ jp, int* __restrict__ done,
                                                         int cap) {
  if (*done) return;
  double s = (threadIdx.x < np) ? part[threadIdx.x] : 0.0;
  s = block_sum(s);
  if (threadIdx.x == 0) {
    const int j = *jp;
    beta[j] = sqrt(s);
    *jp = j + 1;
    if (j + 1 >= cap) *done = 2;
  }
}

static unsigned ew_grid(size_t n) {
  size_t g = (n + 255) / 256;
  if (g < 1) g = 1;
  if (g > 152 * 16) g = 152 * 16;
  return (unsigned)g;
}

static unsigned red_grid(size_t n) {
  size_t g = (n + kRedThreads - 1) / kRedThreads;
  if (g < 1) g = 1;
  if (g > kRedBlocks) g = kRedBlocks;
  return (unsigned)g;
}

void Reducer::init() {
  part.alloc(kRedBlocks);
  out.alloc(8);
  QCMG_CUDA(cudaMallocHost(&host, 8 * sizeof(double)));
}

Reducer::~Reducer() {
  if (host) cudaFreeHost(host);
}

double Reducer::dot(const double* x, const double* y, size_t n, cudaStream_t s) {
  if (!part.p) init();
  unsigned g = red_grid(n);
  k_dot_partial<<<g, kRedThreads, 0, s>>>(x, y, n, part.p);
  k_reduce_final<<<1, kRedBlocks, 0, s>>>(part.p, (int)g, out.p);
  QCMG_CUDA(cudaGetLastError());
  QCMG_CUDA(cudaMemcpyAsync(host, out.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  QCMG_CUDA(cudaStreamSynchronize(s));
  return host[0];
}

double Reducer::axpy_norm2(double* r, const double* q, double alpha, size_t n, cudaStream_t s) {
  if (!part.p) init();
  unsigned g = red_grid(n);
  k_axpy_norm<<<g, kRedThreads, 0, s>>>(r, q, alpha, n, part.p);
  k_reduce_final<<<1, kRedBlocks, 0, s>>>(part.p, (int)g, out.p);
  QCMG_CUDA(cudaGetLastError());
  QCMG_CUDA(cudaMemcpyAsync(host, out.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  QCMG_CUDA(cudaStreamSynchronize(s));
  return host[0];
}

void Reducer::dot_dev(const double* x, const double* y, size_t n, double* out_dev,
                      cudaStream_t s) {
  if (!part.p) init();
  unsigned g = red_grid(n);
  k_dot_partial<<<g, kRedThreads, 0, s>>>(x, y, n, part.p);
  k_reduce_final<<<1, kRedBlocks, 0, s>>>(part.p, (int)g, out_dev);
  QCMG_CUDA(cudaGetLastError());
}

void axpy_neg_dev(double* y, const double* x, const double* a_dev, size_t n, cudaStream_t s) {
  if (!n) return;
  k_axpy_neg_dev<<<ew_grid(n), 256, 0, s>>>(y, x, a_dev, n);
  QCMG_CUDA(cudaGetLastError());
}

void axpy(double* y, const double* x, double a, size_t n, cudaStream_t s) {
  if (!n) return;
  k_axpy<<<ew_grid(n), 256, 0, s>>>(y, x, a, n);
  QCMG_CUDA(cudaGetLastError());
}

void scale2(double* r, double s1, double* q, double s2, size_t n, cudaStream_t s) {
  if (!n) return;
  k_scale2<<<ew_grid(n), 256, 0, s>>>(r, s1, q, s2, n);
  QCMG_CUDA(cudaGetLastError());
}

void scale(double* x, double a, size_t n, cudaStream_t s) {
  if (!n) return;
  k_scale<<<ew_grid(n), 256, 0, s>>>(x, a, n);
  QCMG_CUDA(cudaGetLastError());
}

void lanczos_step_nodes(const LanczosDevState& st, double* r, double* q, size_t n, GraphChain& gc,
                        const std::function<void(const double*, double*)>& product) {
  const unsigned g = red_grid(n);
  gc.add(k_lzb_scale2, dim3(ew_grid(n)), dim3(256), 0, r, q, n, (const double*)st.beta,
         (const int*)st.j, (const int*)st.done);
  product(r, q);  // q += H r, a node of the same chain
  // the roles swap: q is the new residual, r the current basis vector
  gc.add(k_lzb_dot_partial, dim3(g), dim3(kRedThreads), 0, (const double*)r, (const double*)q, n,
         st.part, (const int*)st.done);
  gc.add(k_lzb_alpha, dim3(1), dim3(kRedBlocks), 0, (const double*)st.part, (int)g, st.alpha,
         (const int*)st.j, (const int*)st.done);
  gc.add(k_lzb_axpy_norm, dim3(g), dim3(kRedThreads), 0, q, (const double*)r, n,
         (const double*)st.alpha, (const int*)st.j, st.part, (const int*)st.done);
  gc.add(k_lzb_beta, dim3(1), dim3(kRedBlocks), 0, (const double*)st.part, (int)g, st.beta, st.j,
         st.done, st.cap);
}

void replay_step(double* r, double* q, double* gs, double alpha, double beta, double c, size_t n,
                 cudaStream_t s) {
  if (!n) return;
  k_replay<<<ew_grid(n), 256, 0, s>>>(r, q, gs, alpha, beta, c, n);
  QCMG_CUDA(cudaGetLastError());
}

}  // namespace qcmg
