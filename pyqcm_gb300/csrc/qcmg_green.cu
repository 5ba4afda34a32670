// Lehmann Green function of a Q-matrix, batched over frequencies:
//   G_w(b, a) = sum_i v(a,i) u_w(i) conj(v(b,i)),  u_w(i) = 1 / (z_w - e_i)
// (src_ed/Q_matrix.hpp:133-151 with VDVH_naive, src_util/VDVH_kernel.cpp:28-48).
// One CTA per frequency: u_w is computed once into shared memory, then each
// thread accumulates its (a, b) entries over the poles; v stays L2-resident
// across the frequency batch.
#include <cuComplex.h>

#include "qcmg_internal.h"
#include "qcmg_krylov.h"

namespace qcmg {

__global__ void k_green(int L, int M, const double* __restrict__ e,
                        const double2* __restrict__ v, const double2* __restrict__ z,
                        double2* __restrict__ G) {
  extern __shared__ double2 u[];
  const int w = blockIdx.x;
  const double2 zw = z[w];
  for (int i = threadIdx.x; i < M; i += blockDim.x) {
    double re = zw.x - e[i], im = zw.y;
    double den = re * re + im * im;
    u[i] = make_double2(re / den, -im / den);
  }
  __syncthreads();
  double2* Gw = G + (size_t)w * L * L;
  for (int ab = threadIdx.x; ab < L * L; ab += blockDim.x) {
    const int b = ab % L, a = ab / L;  // G[b + a*L]
    double sr = 0.0, si = 0.0;
    for (int i = 0; i < M; ++i) {
      const double2 va = v[a + (size_t)L * i], vb = v[b + (size_t)L * i], ui = u[i];
      // t = va * ui
      const double tr = va.x * ui.x - va.y * ui.y, ti = va.x * ui.y + va.y * ui.x;
      // += t * conj(vb)
      sr += tr * vb.x + ti * vb.y;
      si += ti * vb.x - tr * vb.y;
    }
    Gw[ab] = make_double2(sr, si);
  }
}

void green_function_batch(int L, int M, const double* e, const double* v, int nz, const double* z,
                          double* G, cudaStream_t s) {
  if (nz <= 0 || L <= 0) return;
  size_t smem = (size_t)std::max(M, 1) * sizeof(double2);
  QCMG_CHECK_ARG(smem <= 200 * 1024, "too many poles for one shared-memory pass");
  if (smem > 48 * 1024)
    QCMG_CUDA(cudaFuncSetAttribute(k_green, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_green<<<nz, 256, smem, s>>>(L, M, e, (const double2*)v, (const double2*)z, (double2*)G);
  QCMG_CUDA(cudaGetLastError());
}

}  // namespace qcmg
