// The factorized product y (+)= H x of the fixed-point path.
//
// The vector is stored like the reference's (up index fastest: slab a is the
// du up states of down state a, contiguous).  Two passes:
//   pass U  persistent CTAs take slabs of x into shared memory with bulk
//           (TMA) copies; every up-spin hop is an integer gather-add from
//           the staged slab; the diagonal (one-body diagonal + density-
//           density terms) and the accumulated input are added; y's slab is
//           written once.  With room for two slabs, one read of the hop
//           table serves both.
//   pass D  one warp per (row band, down state): every down-spin hop adds a
//           neighbour slab's segment of the band.  Warps sweep the down
//           states of one band at a time, so the band of x (~48 MB) stays
//           L2-resident and HBM sees x about once.
// Restates Hamiltonian_Factorized::mult_add (pyqcm
// src_ed/Hamiltonian/Hamiltonian_Factorized.hpp:118-170) on fixed-point
// vectors: hop values share one magnitude per spin (+-t), so a row's hops
// are a signed sum of gathered entries times t.
#include <algorithm>
#include <cstdlib>
#include <type_traits>
#include <vector>

#include "qcmg_fx.cuh"
#include "qcmg_fxprod.h"
#include "qcmg_tma.cuh"

namespace qcmg {

// ---------------------------------------------------------------------------
// pass U, small slabs: threads stage the slab, hops from the CSR

template <int INTER>
__global__ void __launch_bounds__(512) k_fx_passU(FxProdArgs A) {
  extern __shared__ int64_t xs[];
  const uint32_t du = A.du;
  for (uint32_t a = blockIdx.x; a < A.dd; a += gridDim.x) {
    const size_t base = (size_t)a * du;
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < du; i += blockDim.x) xs[i] = A.x[base + i];
    __syncthreads();
    const int64_t dda = A.ddn[a];
    const uint32_t dbits = A.bin_dn[a];
    for (uint32_t i = threadIdx.x; i < du; i += blockDim.x) {
      const uint32_t k0 = A.rp_up[i], ks = A.rs_up[i], k1 = A.rp_up[i + 1];
      int64_t sp = 0, sn = 0;
      for (uint32_t k = k0; k < ks; ++k) sp += xs[A.col_up[k]];
      for (uint32_t k = ks; k < k1; ++k) sn += xs[A.col_up[k]];
      int64_t out = mul_fix(sp - sn, A.mt_up, A.sh_up);
      int64_t D = A.dup[i] + dda;
      if (INTER == QCMG_INTER_ONSITE) {
        D += A.U * (int64_t)__popc(A.bin_up[i] & dbits);
      } else if (INTER == QCMG_INTER_GENERAL) {
        uint32_t u = A.bin_up[i];
        const int64_t* w = A.wdn + (size_t)a * A.L;
        while (u) {
          D += w[__ffs(u) - 1];
          u &= u - 1;
        }
      }
      out += mul_fix_diag(xs[i], D, A.sh_d, A.d_tz);
      if (A.yin) out += mul_fix(A.yin[base + i], A.m_in, A.sh_in);
      A.y[base + i] = out;
    }
  }
}

// ---------------------------------------------------------------------------
// pass U, bulk-copied slabs, grouped ELL hops

// Elements per slab buffer: even (16-byte multiple) and at least du + 2, so
// the zero slot view[du] lies inside the buffer for either view offset.
__host__ __device__ inline uint32_t slab_stride(uint32_t du) { return (du + 3u) & ~1u; }

// A slab starts at byte a*du*8, which is 8 mod 16 when du and a are odd.
// The copy moves the 16-byte-aligned interior [e0, e1); thread 0 loads the
// (at most one) element left over at either end.
__device__ __forceinline__ void slab_range(uint32_t a, uint32_t du, uint32_t* e0, uint32_t* e1) {
  const bool odd_start = (du & 1u) && (a & 1u);
  *e0 = odd_start ? 1u : 0u;
  *e1 = (du & 1u) ? (odd_start ? du : du - 1u) : du;
}

// Offset (elements) of the second slab buffer: a compile-time constant, so
// one address serves the gathers from both slabs.  Two slabs per round need
// slab_stride(du) <= kSlab1Off (du <= 14205).
constexpr uint32_t kSlab1Off = 14208;

// Groups of a row whose columns are requested together before the gathers.
constexpr int kPreGroups = 4;

// 8-byte load from shared memory at a 32-bit address plus a constant offset.
template <uint32_t OFF>
__device__ __forceinline__ int64_t lds64(uint32_t addr) {
  int64_t v;
  asm volatile("ld.shared.b64 %0, [%1+%2];" : "=l"(v) : "r"(addr), "n"(OFF));
  return v;
}

// Sums of the four staged entries named by one group of columns, in each of
// the NS slabs (the second slab kSlab1Off elements above the first).
template <int NS>
__device__ __forceinline__ void gather_group(uint32_t vbase, uint2 w, int64_t (&t)[NS]) {
  const uint32_t a0 = vbase + ((w.x & 0xffffu) << 3);
  const uint32_t a1 = vbase + ((w.x >> 16) << 3);
  const uint32_t a2 = vbase + ((w.y & 0xffffu) << 3);
  const uint32_t a3 = vbase + ((w.y >> 16) << 3);
  const int64_t x0 = lds64<0>(a0), x1 = lds64<0>(a1), x2 = lds64<0>(a2), x3 = lds64<0>(a3);
  if (NS == 2) {
    constexpr uint32_t O = kSlab1Off * 8;
    const int64_t y0 = lds64<O>(a0), y1 = lds64<O>(a1), y2 = lds64<O>(a2), y3 = lds64<O>(a3);
    t[NS - 1] = (y0 + y1) + (y2 + y3);
  }
  t[0] = (x0 + x1) + (x2 + x3);
}

// Each round a CTA stages NS slabs (a, a + G), then every thread takes rows
// i: one 8-byte load brings four 16-bit hop columns of row i, and each
// column is gathered from all NS staged slabs.  Row i lists its positive
// hops in its first groups and its negative hops after them; padding
// columns point at the zero slot du.  With NS = 2 the grid is even, so the
// two slabs of a round have the same alignment (view offset).  With NS = 1
// a second CTA on the SM computes while this one's copy is in flight.
template <int INTER, int NS, bool FAST>
__global__ void __launch_bounds__(NS == 1 ? 512 : 1024, NS == 1 ? 2 : 1) k_fx_passU4(FxProdArgs A) {
  extern __shared__ __align__(16) int64_t smem_slab[];
  __shared__ __align__(8) uint64_t bars[NS];
  const uint32_t du = A.du, dd = A.dd;
  const int tid = threadIdx.x;
  const uint32_t G = gridDim.x;
  if (NS == 2 && (G & 1u)) {  // launch contract: even grid
    if (tid == 0 && blockIdx.x == 0) atomicExch(A.err, 1);
    return;
  }
  if (tid == 0) {
#pragma unroll
    for (int s = 0; s < NS; ++s) mbar_init(&bars[s], 1);
    fence_barrier_init();
  }
  __syncthreads();
  unsigned parity = 0u;
  for (uint32_t a0 = blockIdx.x; a0 < dd; a0 += NS * G) {
    if (tid == 0) {
      fence_proxy_async_smem();  // earlier generic accesses before the copies
#pragma unroll
      for (int s = 0; s < NS; ++s) {
        const uint32_t a = a0 + s * G;
        if (a >= dd) break;
        uint32_t e0, e1;
        slab_range(a, du, &e0, &e1);
        const unsigned bytes = (e1 - e0) * 8u;
        mbar_arrive_expect_tx(&bars[s], bytes);
        bulk_g2s(smem_slab + s * kSlab1Off + 2 * e0, A.x + (size_t)a * du + e0, bytes, &bars[s]);
      }
    }
    bool ok = true;
#pragma unroll
    for (int s = 0; s < NS; ++s)
      if (a0 + s * G < dd) ok = mbar_wait_bounded(&bars[s], parity) && ok;
    if (__syncthreads_or(!ok)) {  // CTA-uniform decision: every thread leaves together
      if (tid == 0) {
        atomicExch(A.err, 1);
        // give copies still in flight a last bounded chance to land
#pragma unroll
        for (int s = 0; s < NS; ++s)
          if (a0 + s * G < dd) (void)mbar_wait_bounded(&bars[s], parity);
      }
      return;
    }
    parity ^= 1u;
    // element j of slab s is view[s * kSlab1Off + j]; the copy landed at
    // buf + 2*e0, so view = buf + e0 (e0 is the same for both slabs).
    uint32_t e0, e1;
    slab_range(a0, du, &e0, &e1);
    const int64_t* view = smem_slab + e0;
    int64_t dda[NS];
    int32_t dda32[NS];
    uint32_t dbits[NS];
    bool live[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      const uint32_t a = min(a0 + s * G, dd - 1u);
      live[s] = a0 + s * G < dd;
      dda[s] = FAST ? 0 : A.ddn[a];
      dda32[s] = FAST ? A.ddn32[a] : 0;
      dbits[s] = A.bin_dn[a];
      if (tid == 0 && a0 + s * G < dd) {
        int64_t* v = smem_slab + s * kSlab1Off + e0;
        const size_t base = (size_t)a * du;
        if (e0 == 1u) v[0] = A.x[base];
        if (e1 == du - 1u) v[du - 1] = A.x[base + du - 1];
        v[du] = 0;  // zero slot for padding columns
      }
    }
    __syncthreads();
    const uint32_t vbase = smem_u32(view);
    const uint32_t bd = blockDim.x;
    // the next row's group counts are loaded one row ahead; a row's group
    // columns, diagonal and accumulated input are all requested before its
    // first gather
    uint32_t c_next = tid < du ? __ldg(A.cnt4 + tid) : 0u;
    for (uint32_t i = tid; i < du; i += bd) {
      const uint32_t c = c_next;
      const uint32_t gp = c & 0xffu, gt = gp + (c >> 8);
      // the table holds at least kPreGroups groups per row (zero-slot padding),
      // so the first ones are loaded and gathered without a per-row test
      uint2 w[kPreGroups];
#pragma unroll
      for (int g = 0; g < kPreGroups; ++g) w[g] = __ldg(A.ell4 + (size_t)g * du + i);
      const int64_t dui = FAST ? 0 : __ldg(A.dup + i);
      const int32_t dui32 = FAST ? __ldg(A.dup32 + i) : 0;
      const uint32_t ubits = __ldg(A.bin_up + i);
      int64_t yv[NS];
#pragma unroll
      for (int s = 0; s < NS; ++s)
        yv[s] = (A.yin && live[s]) ? __ldcs(A.yin + (size_t)(a0 + s * G) * du + i) : 0;
      if (i + bd < du) c_next = __ldg(A.cnt4 + i + bd);
      int64_t sp[NS], sn[NS];
#pragma unroll
      for (int s = 0; s < NS; ++s) sp[s] = sn[s] = 0;
#pragma unroll
      for (int g = 0; g < kPreGroups; ++g) {
        int64_t t[NS];
        gather_group<NS>(vbase, w[g], t);
#pragma unroll
        for (int s = 0; s < NS; ++s) {
          if ((uint32_t)g < gp)
            sp[s] += t[s];
          else
            sn[s] += t[s];
        }
      }
      for (uint32_t g = kPreGroups; g < gt; ++g) {  // rows with more than kPreGroups groups
        int64_t t[NS];
        gather_group<NS>(vbase, __ldg(A.ell4 + (size_t)g * du + i), t);
#pragma unroll
        for (int s = 0; s < NS; ++s) {
          if (g < gp)
            sp[s] += t[s];
          else
            sn[s] += t[s];
        }
      }
#pragma unroll
      for (int s = 0; s < NS; ++s) {
        if (!live[s]) break;
        const uint32_t a = a0 + s * G;
        int64_t out;
        if (FAST) {
          // small-integer diagonal D >> tz in 32 bits, shifts fixed per launch
          out = rshift_fixed(sp[s] - sn[s], A.t_up, A.r_up);
          int32_t Dn = dui32 + dda32[s];
          if (INTER == QCMG_INTER_ONSITE) {
            Dn += A.U32 * __popc(ubits & dbits[s]);
          } else if (INTER == QCMG_INTER_GENERAL) {
            uint32_t u = ubits;
            const int32_t* wt = A.wdn32 + (size_t)a * A.L;
            while (u) {
              Dn += wt[__ffs(u) - 1];
              u &= u - 1;
            }
          }
          out += rshift_fixed(view[s * kSlab1Off + i] * (int64_t)Dn, A.t_d, A.r_d);
          if (A.yin) out += rshift_fixed(A.neg_in ? -yv[s] : yv[s], A.t_in, A.r_in);
        } else {
          out = mul_fix(sp[s] - sn[s], A.mt_up, A.sh_up);
          int64_t D = dui + dda[s];
          if (INTER == QCMG_INTER_ONSITE) {
            D += A.U * (int64_t)__popc(ubits & dbits[s]);
          } else if (INTER == QCMG_INTER_GENERAL) {
            uint32_t u = ubits;
            const int64_t* wt = A.wdn + (size_t)a * A.L;
            while (u) {
              D += wt[__ffs(u) - 1];
              u &= u - 1;
            }
          }
          out += mul_fix(view[s * kSlab1Off + i], D, A.sh_d);
          if (A.yin) out += mul_fix(yv[s], A.m_in, A.sh_in);
        }
        __stcs(A.y + (size_t)a * du + i, out);
      }
    }
    __syncthreads();  // every buffer is free again
  }
}

// ---------------------------------------------------------------------------
// pass D: one warp per (band, down state)

// Adds, for the neighbours k in [kf, kt) of the current chunk (columns held
// one per lane in ccol), the band segments at rows ia.. and ib.. (VEC
// consecutive elements each) into acc.
template <int VEC>
__device__ __forceinline__ void passD_accum(const int64_t* __restrict__ x, uint32_t du,
                                            uint32_t ccol, uint32_t kf, uint32_t kt, uint32_t ia,
                                            uint32_t ib, bool va, bool vb, int64_t (&acc)[2 * VEC]) {
#pragma unroll 4
  for (uint32_t k = kf; k < kt; ++k) {
    const uint32_t b = __shfl_sync(0xffffffffu, ccol, (int)k);
    const int64_t* src = x + (size_t)b * du;
    if (VEC == 2) {
      if (va) {
        const longlong2 v = __ldcg(reinterpret_cast<const longlong2*>(src + ia));
        acc[0] += v.x;
        acc[1] += v.y;
      }
      if (vb) {
        const longlong2 v = __ldcg(reinterpret_cast<const longlong2*>(src + ib));
        acc[2] += v.x;
        acc[3] += v.y;
      }
    } else {
      if (va) acc[0] += __ldcg(src + ia);
      if (vb) acc[1] += __ldcg(src + ib);
    }
  }
}

// VEC = 2 needs du even (every slab segment at an even row is 16-byte
// aligned); bands start at multiples of 256 rows.  DOT: also the dot
// product of the finished y with A.dot_x (the element of x at the same
// place is in the band of x that L2 holds).
template <int VEC, bool FAST, bool DOT>
__global__ void __launch_bounds__(256) k_fx_passD4(FxProdArgs A) {
  const uint32_t du = A.du, dd = A.dd;
  const uint32_t lane = threadIdx.x & 31u;
  const size_t warp = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const size_t nwarps = ((size_t)gridDim.x * blockDim.x) >> 5;
  const size_t items = (size_t)A.nbands * dd;
  constexpr uint32_t kSweep = 64u * VEC;  // rows per warp sweep: two VEC-chunks per lane
  I128 dot = {0, 0};
  for (size_t it = warp; it < items; it += nwarps) {
    const uint32_t band = (uint32_t)(it / dd), a = (uint32_t)(it % dd);
    const uint32_t r0 = band * A.band, r1 = min(du, r0 + A.band);
    const uint32_t k0 = A.rp_dn[a], np = A.rs_dn[a] - k0, nt = A.rp_dn[a + 1] - k0;
    int64_t* yrow = A.y + (size_t)a * du;
    for (uint32_t i0 = r0; i0 < r1; i0 += kSweep) {
      const uint32_t ia = i0 + lane * VEC, ib = ia + 32u * VEC;
      const bool va = ia < r1, vb = ib < r1;
      int64_t P[2 * VEC], N[2 * VEC];
#pragma unroll
      for (int e = 0; e < 2 * VEC; ++e) P[e] = N[e] = 0;
      for (uint32_t kc = 0; kc < nt; kc += 32u) {
        const uint32_t ccol = (kc + lane < nt) ? A.col_dn[k0 + kc + lane] : 0u;
        const uint32_t e = min(32u, nt - kc);
        const uint32_t spos = np > kc ? min(e, np - kc) : 0u;
        passD_accum<VEC>(A.x, du, ccol, 0u, spos, ia, ib, va, vb, P);
        passD_accum<VEC>(A.x, du, ccol, spos, e, ia, ib, va, vb, N);
      }
      // y streams through once (evict-first), leaving L2 to the band of x
      auto term = [&](int64_t v) {
        return FAST ? rshift_fixed(v, A.t_dn, A.r_dn) : mul_fix(v, A.mt_dn, A.sh_dn);
      };
      const int64_t* xrow = DOT ? A.dot_x + (size_t)a * du : nullptr;
      auto acc_dot = [&](int64_t yv, int64_t xv) {
        dot = add128(dot, shr128(mul_s64(yv, xv), kDotShift));
      };
      if constexpr (VEC == 2) {
        if (va) {
          longlong2* yp = reinterpret_cast<longlong2*>(yrow + ia);
          longlong2 v = __ldcs(yp);
          v.x += term(P[0] - N[0]);
          v.y += term(P[1] - N[1]);
          __stcs(yp, v);
          if (DOT) {
            const longlong2 xv = __ldcg(reinterpret_cast<const longlong2*>(xrow + ia));
            acc_dot(v.x, xv.x);
            acc_dot(v.y, xv.y);
          }
        }
        if (vb) {
          longlong2* yp = reinterpret_cast<longlong2*>(yrow + ib);
          longlong2 v = __ldcs(yp);
          v.x += term(P[2] - N[2]);
          v.y += term(P[3] - N[3]);
          __stcs(yp, v);
          if (DOT) {
            const longlong2 xv = __ldcg(reinterpret_cast<const longlong2*>(xrow + ib));
            acc_dot(v.x, xv.x);
            acc_dot(v.y, xv.y);
          }
        }
      } else {
        if (va) {
          const int64_t v = __ldcs(yrow + ia) + term(P[0] - N[0]);
          __stcs(yrow + ia, v);
          if (DOT) acc_dot(v, __ldcg(xrow + ia));
        }
        if (vb) {
          const int64_t v = __ldcs(yrow + ib) + term(P[1] - N[1]);
          __stcs(yrow + ib, v);
          if (DOT) acc_dot(v, __ldcg(xrow + ib));
        }
      }
    }
  }
  if (DOT) block_store128(dot, A.dot_part);  // every thread of the block gets here
}

// ---------------------------------------------------------------------------
// tables

// Grouped ELL: row i holds ceil(np/4) groups of its positive hop columns,
// then ceil(nn/4) groups of its negative ones, four 16-bit columns per
// group, padded with dim (the zero slot behind each staged slab);
// ell4[g * dim + i] is group g of row i and cnt4[i] = positive groups |
// (negative groups << 8).
bool build_ell4(const DevBuf<uint32_t>& rp, const DevBuf<uint32_t>& rs, const DevBuf<uint32_t>& col,
                uint32_t dim, cudaStream_t s, DevBuf<uint2>& ell4, DevBuf<uint16_t>& cnt4) {
  if (dim == 0 || dim > 65534u) return false;
  std::vector<uint32_t> hrp(dim + 1), hrs(dim);
  QCMG_CUDA(cudaMemcpyAsync(hrp.data(), rp.p, (dim + 1) * 4, cudaMemcpyDeviceToHost, s));
  QCMG_CUDA(cudaMemcpyAsync(hrs.data(), rs.p, dim * 4, cudaMemcpyDeviceToHost, s));
  QCMG_CUDA(cudaStreamSynchronize(s));
  const size_t nnz = hrp[dim];
  std::vector<uint32_t> hcol(std::max<size_t>(nnz, 1));
  if (nnz) QCMG_CUDA(cudaMemcpyAsync(hcol.data(), col.p, nnz * 4, cudaMemcpyDeviceToHost, s));
  QCMG_CUDA(cudaStreamSynchronize(s));
  uint32_t groups = 1;
  for (uint32_t i = 0; i < dim; ++i) {
    const uint32_t np = hrs[i] - hrp[i], nn = hrp[i + 1] - hrs[i];
    const uint32_t gp = (np + 3) / 4, gn = (nn + 3) / 4;
    if (gp > 255 || gn > 255) return false;
    groups = std::max(groups, gp + gn);
  }
  groups = std::max<uint32_t>(groups, kPreGroups);  // pass U loads the first kPreGroups unconditionally
  const uint16_t Z = (uint16_t)dim;
  std::vector<uint16_t> cols((size_t)groups * 4 * dim, Z), hc(dim);
  // cols is laid out as [group][row][4].  Slot k of a row (group k/4,
  // position k%4) is gathered by 16 lanes at once: the rows of one
  // half-warp, 16 consecutive rows from a multiple of 16.  An 8-byte shared
  // load costs one wavefront per distinct address on its busiest bank pair
  // (column mod 16), and a row's columns may take any order within its
  // positive and its negative list.  So, slot by slot, each row of a
  // half-warp takes the remaining column of the slot's sign list whose bank
  // pair is least used so far in that slot; rows with the fewest choices go
  // first.  On the 4x4 half bases this cuts the wavefronts from ~1.8x to
  // ~1.55x the conflict-free count.
  for (uint32_t i = 0; i < dim; ++i) {
    const uint32_t np = hrs[i] - hrp[i], nn = hrp[i + 1] - hrs[i];
    hc[i] = (uint16_t)(((np + 3) / 4) | (((nn + 3) / 4) << 8));
  }
  std::vector<std::vector<uint32_t>> remp(16), remn(16);
  std::vector<uint32_t> order;
  for (uint32_t b0 = 0; b0 < dim; b0 += 16) {
    const uint32_t nr = std::min<uint32_t>(16, dim - b0);
    uint32_t kmax = 0;
    for (uint32_t r = 0; r < nr; ++r) {
      const uint32_t i = b0 + r;
      remp[r].assign(hcol.begin() + hrp[i], hcol.begin() + hrs[i]);
      remn[r].assign(hcol.begin() + hrs[i], hcol.begin() + hrp[i + 1]);
      std::sort(remp[r].begin(), remp[r].end());
      std::sort(remn[r].begin(), remn[r].end());
      kmax = std::max<uint32_t>(kmax, 4u * ((hc[i] & 0xffu) + (hc[i] >> 8)));
    }
    for (uint32_t k = 0; k < kmax; ++k) {
      // the list slot k draws from, for row r (null: padding)
      auto list = [&](uint32_t r) -> std::vector<uint32_t>* {
        const uint32_t c = hc[b0 + r], gp = c & 0xffu, gt = gp + (c >> 8);
        if (k < 4 * gp) return &remp[r];
        if (k < 4 * gt) return &remn[r];
        return nullptr;
      };
      order.resize(nr);
      for (uint32_t r = 0; r < nr; ++r) order[r] = r;
      std::stable_sort(order.begin(), order.end(), [&](uint32_t p, uint32_t q) {
        const std::vector<uint32_t>* lp = list(p);
        const std::vector<uint32_t>* lq = list(q);
        const size_t np = (lp && !lp->empty()) ? lp->size() : SIZE_MAX;
        const size_t nq = (lq && !lq->empty()) ? lq->size() : SIZE_MAX;
        return np < nq;
      });
      uint32_t used[16] = {0};
      bool zero_used = false;
      for (uint32_t r : order) {
        std::vector<uint32_t>* l = list(r);
        uint32_t j = Z;
        if (l && !l->empty()) {
          size_t best = 0;
          for (size_t q = 1; q < l->size(); ++q)
            if (used[(*l)[q] % 16] < used[(*l)[best] % 16]) best = q;
          j = (*l)[best];
          l->erase(l->begin() + best);
          ++used[j % 16];
        } else if (!zero_used) {  // padding: every padded lane reads the same zero slot
          zero_used = true;
          ++used[Z % 16];
        }
        cols[((size_t)(k / 4) * dim + b0 + r) * 4 + (k % 4)] = (uint16_t)j;
      }
    }
  }
  std::vector<uint2> he((size_t)groups * dim);
  for (size_t q = 0; q < he.size(); ++q) {
    he[q].x = (uint32_t)cols[4 * q] | ((uint32_t)cols[4 * q + 1] << 16);
    he[q].y = (uint32_t)cols[4 * q + 2] | ((uint32_t)cols[4 * q + 3] << 16);
  }
  ell4.upload(he.data(), he.size(), s);
  cnt4.upload(hc.data(), hc.size(), s);
  QCMG_CUDA(cudaStreamSynchronize(s));  // host staging vectors go out of scope
  return true;
}

int pow2_exponent(int64_t m) {
  if (m == 0 || m == INT64_MIN) return -1;
  const uint64_t a = (uint64_t)(m < 0 ? -m : m);
  if (a & (a - 1)) return -1;
  int p = 0;
  while ((1ull << p) != a) ++p;
  return p;
}

int choose_slabs_per_pass(uint32_t du, int max_optin_smem) {
  if (du < 64 || du > 65534u) return 0;
  const size_t one = (size_t)slab_stride(du) * 8;
  if (one > (size_t)max_optin_smem) return 0;
  const bool two_fit = slab_stride(du) <= kSlab1Off &&
                       ((size_t)kSlab1Off + slab_stride(du)) * 8 <= (size_t)max_optin_smem;
  int ns = two_fit ? 2 : 1;
  if (const char* e = std::getenv("QCMG_FX_SLABS")) {
    const int v = std::atoi(e);
    if (v == 1) ns = 1;
    if (v == 2 && two_fit) ns = 2;
  }
  return ns;
}

// ---------------------------------------------------------------------------
// launcher

template <int NS, typename Kern>
static void launch_passU4(Kern kern, const qcmg_hamiltonian* H, const FxProdArgs& A, int sms,
                          cudaStream_t s) {
  const size_t smem = ((NS == 2 ? (size_t)kSlab1Off : 0) + slab_stride(H->du)) * 8;
  QCMG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int tmax = NS == 1 ? 512 : 1024;
  const int threads = std::min<int>(tmax, (int)((H->du + 127) / 128 * 128));
  int per_sm = 0;
  QCMG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem));
  per_sm = std::max(per_sm, 1);
  const size_t rounds = ((size_t)H->dd + NS - 1) / NS;
  size_t grid = std::max<size_t>(1, std::min<size_t>(rounds, (size_t)sms * per_sm));
  if (NS == 2 && (grid & 1)) ++grid;  // even: the two slabs of a round share their alignment
  kern<<<(unsigned)grid, threads, smem, s>>>(A);
}

unsigned launch_product(const qcmg_hamiltonian* H, const FxProdArgs& A, cudaStream_t s) {
  const FxTables& T = H->fx;
  int sms = 0;
  QCMG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, H->device));
  const int ik = H->inter_kind;
  // FAST kernels: hop magnitudes and accumulation factor are powers of two
  // and the diagonal is narrow (the Hubbard form with t = 1 and small-integer
  // energies); everything else uses the 128-bit products
  const bool fast = A.d_tz >= 0 && A.p2_up >= 0 && A.p2_dn >= 0 && (!A.yin || A.p2_in >= 0);
  auto passU4 = [&](auto ns_tag, auto fast_tag) {
    constexpr int NS = decltype(ns_tag)::value;
    constexpr bool F = decltype(fast_tag)::value;
    if (ik == QCMG_INTER_NONE) launch_passU4<NS>(k_fx_passU4<QCMG_INTER_NONE, NS, F>, H, A, sms, s);
    else if (ik == QCMG_INTER_ONSITE) launch_passU4<NS>(k_fx_passU4<QCMG_INTER_ONSITE, NS, F>, H, A, sms, s);
    else launch_passU4<NS>(k_fx_passU4<QCMG_INTER_GENERAL, NS, F>, H, A, sms, s);
  };
  using One = std::integral_constant<int, 1>;
  using Two = std::integral_constant<int, 2>;
  using Fast = std::true_type;
  using Full = std::false_type;
  // pass U
  if (T.ns == 2) {
    if (fast) passU4(Two{}, Fast{});
    else passU4(Two{}, Full{});
  } else if (T.ns == 1) {
    if (fast) passU4(One{}, Fast{});
    else passU4(One{}, Full{});
  } else {
    const size_t smem = (size_t)H->du * 8;
    const int threads = H->du >= 512 ? 512 : (H->du >= 256 ? 256 : 128);
    const unsigned g = (unsigned)std::max<size_t>(1, std::min<size_t>(H->dd, (size_t)sms * 2));
    auto go = [&](auto kern) {
      if (smem > 48 * 1024)
        QCMG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      kern<<<g, threads, smem, s>>>(A);
    };
    if (ik == QCMG_INTER_NONE) go(k_fx_passU<QCMG_INTER_NONE>);
    else if (ik == QCMG_INTER_ONSITE) go(k_fx_passU<QCMG_INTER_ONSITE>);
    else go(k_fx_passU<QCMG_INTER_GENERAL>);
  }
  QCMG_CUDA(cudaGetLastError());
  // pass D
  const size_t items = (size_t)A.nbands * H->dd;
  const unsigned gD = (unsigned)std::max<size_t>(1, std::min<size_t>((items + 7) / 8, (size_t)sms * 8));
  auto passD = [&](auto vec_tag, auto fast_tag) {
    constexpr int V = decltype(vec_tag)::value;
    constexpr bool F = decltype(fast_tag)::value;
    if (A.dot_part) k_fx_passD4<V, F, true><<<gD, 256, 0, s>>>(A);
    else k_fx_passD4<V, F, false><<<gD, 256, 0, s>>>(A);
  };
  if ((H->du & 1u) == 0u) {
    if (fast) passD(Two{}, Fast{});
    else passD(Two{}, Full{});
  } else {
    if (fast) passD(One{}, Fast{});
    else passD(One{}, Full{});
  }
  QCMG_CUDA(cudaGetLastError());
  return gD;
}

}  // namespace qcmg
