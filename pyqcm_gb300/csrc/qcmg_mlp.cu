// Multilayer perceptron for the learned CDMFT warm start: forward, backward
// and Adam training on the device.  No counterpart in the reference.
//
// Layers l = 0..L-1: z_l = a_l W_l^T + b_l, a_{l+1} = tanh(z_l) for hidden
// layers, identity for the last one.  Parameters are kept in FP32 (the Adam
// master copy, layout W_0, b_0, W_1, b_1, ... with W_l row-major
// [width_{l+1} x width_l]); the products use a BF16 copy of the weights with
// FP32 accumulation.  Loss: mean squared error over batch and outputs.
// The networks are small (~10^5 parameters, batches of a few thousand), so
// one tiled FP32 GEMM kernel on the CUDA cores serves all products: every
// layer is well under a GFLOP and launch-bound, not tensor-core-bound.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <numeric>
#include <random>
#include <string>
#include <vector>

#include "qcmg.h"
#include "qcmg_internal.h"

using namespace qcmg;

namespace {

constexpr int kBM = 64, kBN = 64, kBK = 16;

template <typename T>
__device__ __forceinline__ float as_f32(T v);
template <>
__device__ __forceinline__ float as_f32<float>(float v) {
  return v;
}
template <>
__device__ __forceinline__ float as_f32<__nv_bfloat16>(__nv_bfloat16 v) {
  return __bfloat162float(v);
}

// C[m, n] = sum_k A(m, k) B(k, n) + beta C[m, n], FP32 accumulation.
// A(m, k) = TA ? A[k lda + m] : A[m lda + k];  B(k, n) = TB ? B[n ldb + k] : B[k ldb + n].
// 64x64 tile per 256-thread block, 4x4 outputs per thread.
template <bool TA, bool TB, typename BT>
__global__ void __launch_bounds__(256) k_gemm(int M, int N, int K, const float* __restrict__ A,
                                              int lda, const BT* __restrict__ B, int ldb,
                                              float* __restrict__ C, int ldc, float beta) {
  __shared__ float As[kBK][kBM + 4];
  __shared__ float Bs[kBK][kBN + 4];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * kBN;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += kBK) {
    for (int e = threadIdx.x; e < kBM * kBK; e += 256) {
      const int mm = e / kBK, kk = e % kBK;
      const int m = m0 + mm, k = k0 + kk;
      float v = 0.f;
      if (m < M && k < K) v = TA ? A[(size_t)k * lda + m] : A[(size_t)m * lda + k];
      As[kk][mm] = v;
    }
    for (int e = threadIdx.x; e < kBN * kBK; e += 256) {
      const int nn = e / kBK, kk = e % kBK;
      const int n = n0 + nn, k = k0 + kk;
      float v = 0.f;
      if (n < N && k < K) v = as_f32<BT>(TB ? B[(size_t)n * ldb + k] : B[(size_t)k * ldb + n]);
      Bs[kk][nn] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kBK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int m = m0 + ty * 4 + i, n = n0 + tx * 4 + j;
      if (m < M && n < N) {
        float* c = C + (size_t)m * ldc + n;
        *c = acc[i][j] + (beta != 0.f ? beta * *c : 0.f);
      }
    }
}

// y[b, o] = act(y[b, o] + bias[o])
__global__ void k_bias_act(float* __restrict__ y, const float* __restrict__ bias, int rows, int cols,
                           int use_tanh) {
  const size_t n = (size_t)rows * cols;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const float v = y[i] + bias[i % cols];
    y[i] = use_tanh ? tanhf(v) : v;
  }
}

// d = 2 (y - t) / (rows cols), and the partial sums of (y - t)^2 per block
__global__ void k_mse(const float* __restrict__ y, const float* __restrict__ t, float* __restrict__ d,
                      size_t n, float* __restrict__ part) {
  __shared__ float s[256];
  float acc = 0.f;
  const float sc = 2.0f / (float)n;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const float r = y[i] - t[i];
    d[i] = sc * r;
    acc += r * r;
  }
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

// dz = dy * (1 - a^2) for a = tanh(z) (in place on dy)
__global__ void k_tanh_back(float* __restrict__ dy, const float* __restrict__ a, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    dy[i] *= 1.0f - a[i] * a[i];
}

// db[o] = sum_b dz[b, o]
__global__ void k_colsum(const float* __restrict__ dz, int rows, int cols, float* __restrict__ db) {
  for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < cols; o += gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int b = 0; b < rows; ++b) s += dz[(size_t)b * cols + o];
    db[o] = s;
  }
}

// Adam on the FP32 master copy; refreshes the BF16 copy.
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, __nv_bfloat16* __restrict__ pb, size_t n, float lr,
                       float b1, float b2, float eps, float c1, float c2) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    p[i] = pi;
    pb[i] = __float2bfloat16_rn(pi);
  }
}

__global__ void k_to_bf16(const float* __restrict__ p, __nv_bfloat16* __restrict__ pb, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    pb[i] = __float2bfloat16_rn(p[i]);
}

// rows of src selected by idx -> dst
__global__ void k_gather_rows(const float* __restrict__ src, const int* __restrict__ idx, int rows,
                              int cols, float* __restrict__ dst) {
  const size_t n = (size_t)rows * cols;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    dst[i] = src[(size_t)idx[i / cols] * cols + i % cols];
}

unsigned grid_for(size_t n) { return (unsigned)std::max<size_t>(1, std::min<size_t>((n + 255) / 256, 152 * 8)); }

template <bool TA, bool TB, typename BT>
void gemm(int M, int N, int K, const float* A, int lda, const BT* B, int ldb, float* C, int ldc,
          float beta, cudaStream_t s) {
  dim3 g((N + kBN - 1) / kBN, (M + kBM - 1) / kBM);
  k_gemm<TA, TB, BT><<<g, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, beta);
}

}  // namespace

struct qcmg_mlp {
  int device = 0;
  std::vector<int> w;              // widths, L + 1 entries
  std::vector<size_t> offW, offb;  // parameter offsets per layer
  size_t np = 0;
  DevBuf<float> p, g, m, v;
  DevBuf<__nv_bfloat16> pb;
  DevBuf<float> act[17];           // a_0 .. a_L (batch rows); at most 16 layers
  DevBuf<float> dA, dB, tgt, part, xdev;
  int cap = 0;                     // batch rows the activations hold
  long step = 0;
  cudaStream_t s = nullptr;
  std::mutex mu;
  int L() const { return (int)w.size() - 1; }
  void reserve(int rows) {
    if (rows <= cap) return;
    int wmax = *std::max_element(w.begin(), w.end());
    for (size_t l = 0; l < w.size(); ++l) act[l].alloc((size_t)rows * w[l]);
    dA.alloc((size_t)rows * wmax);
    dB.alloc((size_t)rows * wmax);
    tgt.alloc((size_t)rows * w.back());
    cap = rows;
  }
  // a_L = f(a_0) for `rows` rows of act[0]
  void forward(int rows) {
    for (int l = 0; l < L(); ++l) {
      gemm<false, true>(rows, w[l + 1], w[l], act[l].p, w[l], pb.p + offW[l], w[l], act[l + 1].p,
                        w[l + 1], 0.f, s);
      k_bias_act<<<grid_for((size_t)rows * w[l + 1]), 256, 0, s>>>(
          act[l + 1].p, p.p + offb[l], rows, w[l + 1], l + 1 < L() ? 1 : 0);
    }
  }
  // gradient of the MSE against tgt into g; returns the loss
  float backward(int rows) {
    const size_t n = (size_t)rows * w.back();
    const unsigned nb = std::min<unsigned>(grid_for(n), 256);
    part.alloc(256);
    k_mse<<<nb, 256, 0, s>>>(act[L()].p, tgt.p, dA.p, n, part.p);
    float* d = dA.p;
    float* e = dB.p;
    for (int l = L() - 1; l >= 0; --l) {
      if (l + 1 < L())
        k_tanh_back<<<grid_for((size_t)rows * w[l + 1]), 256, 0, s>>>(d, act[l + 1].p,
                                                                       (size_t)rows * w[l + 1]);
      // dW_l = dz^T a_l ; db_l = colsum dz ; da_l = dz W_l
      gemm<true, false>(w[l + 1], w[l], rows, d, w[l + 1], act[l].p, w[l], g.p + offW[l], w[l], 0.f,
                        s);
      k_colsum<<<(w[l + 1] + 127) / 128, 128, 0, s>>>(d, rows, w[l + 1], g.p + offb[l]);
      if (l > 0) {
        gemm<false, false>(rows, w[l], w[l + 1], d, w[l + 1], pb.p + offW[l], w[l], e, w[l], 0.f, s);
        std::swap(d, e);
      }
    }
    std::vector<float> h(nb);
    QCMG_CUDA(cudaMemcpyAsync(h.data(), part.p, nb * sizeof(float), cudaMemcpyDeviceToHost, s));
    QCMG_CUDA(cudaStreamSynchronize(s));
    double tot = 0.0;
    for (float x : h) tot += x;
    return (float)(tot / (double)n);
  }
};

namespace {
template <typename F>
int mlp_guarded(F&& f) {
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
}  // namespace

extern "C" {

int qcmg_mlp_create(int n_layers, const int* widths, qcmg_mlp** out) {
  return mlp_guarded([&] {
    QCMG_CHECK_ARG(out && widths && n_layers >= 1 && n_layers <= 16, "invalid layer count");
    *out = nullptr;
    for (int l = 0; l <= n_layers; ++l)
      QCMG_CHECK_ARG(widths[l] >= 1 && widths[l] <= 4096, "layer widths must be in 1..4096");
    auto* M = new qcmg_mlp();
    try {
      QCMG_CUDA(cudaGetDevice(&M->device));
      M->w.assign(widths, widths + n_layers + 1);
      size_t off = 0;
      for (int l = 0; l < n_layers; ++l) {
        M->offW.push_back(off);
        off += (size_t)M->w[l] * M->w[l + 1];
        M->offb.push_back(off);
        off += M->w[l + 1];
      }
      M->np = off;
      M->p.alloc(off);
      M->g.alloc(off);
      M->m.alloc(off);
      M->v.alloc(off);
      M->pb.alloc(off);
      QCMG_CUDA(cudaMemset(M->p.p, 0, off * sizeof(float)));
      QCMG_CUDA(cudaMemset(M->m.p, 0, off * sizeof(float)));
      QCMG_CUDA(cudaMemset(M->v.p, 0, off * sizeof(float)));
      QCMG_CUDA(cudaMemset(M->pb.p, 0, off * sizeof(__nv_bfloat16)));
      QCMG_CUDA(cudaStreamCreateWithFlags(&M->s, cudaStreamNonBlocking));
    } catch (...) {
      delete M;
      throw;
    }
    *out = M;
  });
}

int qcmg_mlp_destroy(qcmg_mlp* M) {
  return mlp_guarded([&] {
    if (!M) return;
    if (M->s) {
      cudaStreamSynchronize(M->s);
      cudaStreamDestroy(M->s);
    }
    delete M;
  });
}

int qcmg_mlp_num_params(qcmg_mlp* M, size_t* n) {
  return mlp_guarded([&] {
    QCMG_CHECK_ARG(M && n, "NULL argument");
    *n = M->np;
  });
}

int qcmg_mlp_set_params(qcmg_mlp* M, const float* params) {
  return mlp_guarded([&] {
    QCMG_CHECK_ARG(M && params, "NULL argument");
    std::lock_guard<std::mutex> lock(M->mu);
    QCMG_CUDA(cudaSetDevice(M->device));
    QCMG_CUDA(cudaMemcpyAsync(M->p.p, params, M->np * sizeof(float), cudaMemcpyHostToDevice, M->s));
    QCMG_CUDA(cudaMemsetAsync(M->m.p, 0, M->np * sizeof(float), M->s));
    QCMG_CUDA(cudaMemsetAsync(M->v.p, 0, M->np * sizeof(float), M->s));
    k_to_bf16<<<grid_for(M->np), 256, 0, M->s>>>(M->p.p, M->pb.p, M->np);
    QCMG_CUDA(cudaGetLastError());
    QCMG_CUDA(cudaStreamSynchronize(M->s));
    M->step = 0;
  });
}

int qcmg_mlp_get_params(qcmg_mlp* M, float* params) {
  return mlp_guarded([&] {
    QCMG_CHECK_ARG(M && params, "NULL argument");
    std::lock_guard<std::mutex> lock(M->mu);
    QCMG_CUDA(cudaSetDevice(M->device));
    QCMG_CUDA(cudaMemcpyAsync(params, M->p.p, M->np * sizeof(float), cudaMemcpyDeviceToHost, M->s));
    QCMG_CUDA(cudaStreamSynchronize(M->s));
  });
}

int qcmg_mlp_forward(qcmg_mlp* M, int batch, const float* x, float* y) {
  return mlp_guarded([&] {
    QCMG_CHECK_ARG(M && x && y && batch >= 1, "invalid arguments");
    std::lock_guard<std::mutex> lock(M->mu);
    QCMG_CUDA(cudaSetDevice(M->device));
    M->reserve(batch);
    QCMG_CUDA(cudaMemcpyAsync(M->act[0].p, x, (size_t)batch * M->w[0] * sizeof(float),
                              cudaMemcpyHostToDevice, M->s));
    M->forward(batch);
    QCMG_CUDA(cudaGetLastError());
    QCMG_CUDA(cudaMemcpyAsync(y, M->act[M->L()].p, (size_t)batch * M->w.back() * sizeof(float),
                              cudaMemcpyDeviceToHost, M->s));
    QCMG_CUDA(cudaStreamSynchronize(M->s));
  });
}

int qcmg_mlp_loss_grad(qcmg_mlp* M, int batch, const float* x, const float* t, float* loss,
                       float* grad) {
  return mlp_guarded([&] {
    QCMG_CHECK_ARG(M && x && t && loss && batch >= 1, "invalid arguments");
    std::lock_guard<std::mutex> lock(M->mu);
    QCMG_CUDA(cudaSetDevice(M->device));
    M->reserve(batch);
    QCMG_CUDA(cudaMemcpyAsync(M->act[0].p, x, (size_t)batch * M->w[0] * sizeof(float),
                              cudaMemcpyHostToDevice, M->s));
    QCMG_CUDA(cudaMemcpyAsync(M->tgt.p, t, (size_t)batch * M->w.back() * sizeof(float),
                              cudaMemcpyHostToDevice, M->s));
    M->forward(batch);
    *loss = M->backward(batch);
    QCMG_CUDA(cudaGetLastError());
    if (grad) {
      QCMG_CUDA(cudaMemcpyAsync(grad, M->g.p, M->np * sizeof(float), cudaMemcpyDeviceToHost, M->s));
      QCMG_CUDA(cudaStreamSynchronize(M->s));
    }
  });
}

int qcmg_mlp_train(qcmg_mlp* M, int n, const float* x, const float* t, int epochs, int batch,
                   float lr, unsigned seed, float* final_loss) {
  return mlp_guarded([&] {
    QCMG_CHECK_ARG(M && x && t && n >= 1 && epochs >= 0 && batch >= 1 && lr > 0.f,
                   "invalid arguments");
    std::lock_guard<std::mutex> lock(M->mu);
    QCMG_CUDA(cudaSetDevice(M->device));
    batch = std::min(batch, n);
    M->reserve(batch);
    const int ni = M->w[0], no = M->w.back();
    DevBuf<float> X, T;
    DevBuf<int> idx;
    X.upload(x, (size_t)n * ni, M->s);
    T.upload(t, (size_t)n * no, M->s);
    idx.alloc(n);
    std::mt19937 rng(seed);
    std::vector<int> perm(n);
    std::iota(perm.begin(), perm.end(), 0);
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    // the learning rate decays from lr to 0 along half a cosine over the
    // run's minibatch steps
    const double steps = (double)epochs * (n / batch);
    long long k = 0;
    double last = 0.0;
    for (int e = 0; e < epochs; ++e) {
      std::shuffle(perm.begin(), perm.end(), rng);
      QCMG_CUDA(cudaMemcpyAsync(idx.p, perm.data(), n * sizeof(int), cudaMemcpyHostToDevice, M->s));
      QCMG_CUDA(cudaStreamSynchronize(M->s));  // perm is rewritten next epoch
      double tot = 0.0;
      int cnt = 0;
      for (int b0 = 0; b0 + batch <= n; b0 += batch) {
        k_gather_rows<<<grid_for((size_t)batch * ni), 256, 0, M->s>>>(X.p, idx.p + b0, batch, ni,
                                                                        M->act[0].p);
        k_gather_rows<<<grid_for((size_t)batch * no), 256, 0, M->s>>>(T.p, idx.p + b0, batch, no,
                                                                        M->tgt.p);
        M->forward(batch);
        tot += M->backward(batch);
        ++cnt;
        ++M->step;
        const float c1 = 1.f / (1.f - std::pow(b1, (float)M->step));
        const float c2 = 1.f / (1.f - std::pow(b2, (float)M->step));
        const float lr_k = (float)(lr * 0.5 * (1.0 + std::cos(M_PI * (double)k++ / steps)));
        k_adam<<<grid_for(M->np), 256, 0, M->s>>>(M->p.p, M->g.p, M->m.p, M->v.p, M->pb.p, M->np,
                                                   lr_k, b1, b2, eps, c1, c2);
        QCMG_CUDA(cudaGetLastError());
      }
      last = cnt ? tot / cnt : 0.0;
    }
    QCMG_CUDA(cudaStreamSynchronize(M->s));
    if (final_loss) *final_loss = (float)last;
  });
}

}  // extern "C"
