// Factorized Hubbard matrix-vector product, FP64:
//   y[iu + du*id] (+)= sum_J T_up[iu,J] x[J + du*id]      (up hops, in-slab)
//                   + sum_J T_dn[id,J] x[iu + du*J]      (down hops, slab axpys)
//                   + (d_up[iu] + d_dn[id] + W(u, d)) x[iu + du*id]
// The vector is stored as the reference stores it (src_ed/ED_basis.cpp:142-165):
// column-major du x dd, the up index fastest, one contiguous "slab" per down
// index.  One CTA owns one slab at a time: it stages x's slab in shared
// memory (all up-hop gathers then hit shared memory), streams the down-hop
// neighbour slabs from global memory with coalesced loads (they are shared
// by up to ~2*bonds CTAs and mostly hit L2), and writes its y slab once.
// This is the arithmetic of HS_factorized_operator::multiply_add
// (src_ed/Operators/HS_factorized_operator.hpp:57-84) and
// HS_interaction_operator::multiply_add (HS_interaction_operator.hpp:62-70),
// reorganized per output element so that y is read and written once.
#include "qcmg_internal.h"

namespace qcmg {

template <int INTER, bool SMEM>
__global__ void __launch_bounds__(512)
k_matvec_f64(uint32_t du, uint32_t dd, int L,
             const uint32_t* __restrict__ rp_up, const uint32_t* __restrict__ col_up,
             const double* __restrict__ val_up, const double* __restrict__ diag_up,
             const uint32_t* __restrict__ rp_dn, const uint32_t* __restrict__ col_dn,
             const double* __restrict__ val_dn, const double* __restrict__ diag_dn,
             const uint32_t* __restrict__ bin_up, const uint32_t* __restrict__ bin_dn, double U,
             const double* __restrict__ wdn, const double* __restrict__ x, double* __restrict__ y,
             int accumulate) {
  extern __shared__ double xs[];
  for (uint32_t a = blockIdx.x; a < dd; a += gridDim.x) {
    const double* xa = x + (size_t)a * du;
    if (SMEM) {
      __syncthreads();
      for (uint32_t i = threadIdx.x; i < du; i += blockDim.x) xs[i] = xa[i];
      __syncthreads();
    }
    const double* xr = SMEM ? xs : xa;
    const uint32_t k0 = rp_dn[a], k1 = rp_dn[a + 1];
    const double dda = diag_dn[a];
    const uint32_t dbits = bin_dn[a];
    double* ya = y + (size_t)a * du;
    for (uint32_t i = threadIdx.x; i < du; i += blockDim.x) {
      double acc = 0.0;
      const uint32_t j0 = rp_up[i], j1 = rp_up[i + 1];
      for (uint32_t k = j0; k < j1; ++k) acc = fma(val_up[k], xr[col_up[k]], acc);
      for (uint32_t k = k0; k < k1; ++k) acc = fma(val_dn[k], x[(size_t)col_dn[k] * du + i], acc);
      double d = diag_up[i] + dda;
      if (INTER == QCMG_INTER_ONSITE) {
        d += U * (double)__popc(bin_up[i] & dbits);
      } else if (INTER == QCMG_INTER_GENERAL) {
        uint32_t u = bin_up[i];
        const double* w = wdn + (size_t)a * L;
        while (u) {
          d += w[__ffs(u) - 1];
          u &= u - 1;
        }
      }
      double out = fma(d, xr[i], acc);
      if (accumulate) out += ya[i];
      ya[i] = out;
    }
  }
}

template <int INTER>
static void launch_inter(qcmg_hamiltonian* H, const double* x, double* y, bool accumulate) {
  const size_t smem = (size_t)H->du * sizeof(double);
  const int threads = H->du >= 512 ? 512 : (H->du >= 256 ? 256 : 128);
  int sms = 0;
  QCMG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, H->device));
  unsigned grid = (unsigned)std::min<size_t>(H->dd, (size_t)sms * 8);
  if (grid < 1) grid = 1;
  int max_optin = 0;
  QCMG_CUDA(cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, H->device));
  auto& up = H->up;
  auto& dn = H->dn;
  if (smem <= (size_t)max_optin) {
    auto kern = k_matvec_f64<INTER, true>;
    if (smem > 48 * 1024)
      QCMG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<grid, threads, smem, H->stream>>>(H->du, H->dd, H->L, up.rowptr.p, up.col.p, up.val.p,
                                             up.diag.p, dn.rowptr.p, dn.col.p, dn.val.p, dn.diag.p,
                                             up.bin.p, dn.bin.p, H->U, H->wdn.p, x, y,
                                             accumulate ? 1 : 0);
  } else {
    k_matvec_f64<INTER, false><<<grid, threads, 0, H->stream>>>(
        H->du, H->dd, H->L, up.rowptr.p, up.col.p, up.val.p, up.diag.p, dn.rowptr.p, dn.col.p,
        dn.val.p, dn.diag.p, up.bin.p, dn.bin.p, H->U, H->wdn.p, x, y, accumulate ? 1 : 0);
  }
  QCMG_CUDA(cudaGetLastError());
}

template <int INTER>
static void node_inter(qcmg_hamiltonian* H, const double* x, double* y, bool accumulate,
                       GraphChain& gc) {
  const size_t smem = (size_t)H->du * sizeof(double);
  const int threads = H->du >= 512 ? 512 : (H->du >= 256 ? 256 : 128);
  int sms = 0;
  QCMG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, H->device));
  unsigned grid = (unsigned)std::min<size_t>(H->dd, (size_t)sms * 8);
  if (grid < 1) grid = 1;
  int max_optin = 0;
  QCMG_CUDA(cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, H->device));
  auto& up = H->up;
  auto& dn = H->dn;
  const bool in_smem = smem <= (size_t)max_optin;
  auto kern = in_smem ? k_matvec_f64<INTER, true> : k_matvec_f64<INTER, false>;
  if (in_smem && smem > 48 * 1024)
    QCMG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  gc.add(kern, dim3(grid), dim3(threads), in_smem ? smem : 0, H->du, H->dd, H->L,
         (const uint32_t*)up.rowptr.p, (const uint32_t*)up.col.p, (const double*)up.val.p,
         (const double*)up.diag.p, (const uint32_t*)dn.rowptr.p, (const uint32_t*)dn.col.p,
         (const double*)dn.val.p, (const double*)dn.diag.p, (const uint32_t*)up.bin.p,
         (const uint32_t*)dn.bin.p, H->U, (const double*)H->wdn.p, x, y, accumulate ? 1 : 0);
}

void matvec_node(qcmg_hamiltonian* H, const double* x, double* y, bool accumulate, GraphChain& gc) {
  switch (H->inter_kind) {
    case QCMG_INTER_NONE: node_inter<QCMG_INTER_NONE>(H, x, y, accumulate, gc); break;
    case QCMG_INTER_ONSITE: node_inter<QCMG_INTER_ONSITE>(H, x, y, accumulate, gc); break;
    default: node_inter<QCMG_INTER_GENERAL>(H, x, y, accumulate, gc); break;
  }
}

void matvec(qcmg_hamiltonian* H, const double* x, double* y, bool accumulate) {
  if (H->dim == 0) return;
  switch (H->inter_kind) {
    case QCMG_INTER_NONE: launch_inter<QCMG_INTER_NONE>(H, x, y, accumulate); break;
    case QCMG_INTER_ONSITE: launch_inter<QCMG_INTER_ONSITE>(H, x, y, accumulate); break;
    default: launch_inter<QCMG_INTER_GENERAL>(H, x, y, accumulate); break;
  }
}

}  // namespace qcmg
