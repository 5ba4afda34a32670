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
//           states of one band at a time, so the band of x (~26 MB at
//           L = 16) stays L2-resident and HBM sees x about once; the
//           gathers run at the L2's throughput, so the kernel is lean in
//           registers (six blocks per SM) to keep many loads in flight.
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

// Zero slots behind each staged slab: view[du + j] = 0 for j < kZeroSlots,
// one per bank pair, so padding columns can read a zero from whichever bank
// pair the real columns of their slot leave free.
constexpr uint32_t kZeroSlots = 16;

// Elements per slab buffer: even (16-byte multiple) and at least
// du + 1 + kZeroSlots, so the zero slots lie inside the buffer for either
// view offset.
__host__ __device__ inline uint32_t slab_stride(uint32_t du) { return (du + kZeroSlots + 1u + 1u) & ~1u; }

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
// slab_stride(du) <= kSlab1Off (du <= 14190).
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
// columns point at zero slots du..du+15.  With NS = 2 the grid is even, so the
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
      }
      if (tid < (int)kZeroSlots && a0 + s * G < dd)
        smem_slab[s * kSlab1Off + e0 + du + tid] = 0;  // zero slots for padding columns
    }
    __syncthreads();
    const uint32_t vbase = smem_u32(view);
    const uint32_t bd = blockDim.x;
    // the next row's group counts are loaded one row ahead; a row's group
    // columns, diagonal and accumulated input are all requested before its
    // first gather
    uint32_t c_next = tid < du ? __ldg(A.cnt4 + tid) : 0u;
    // the table holds at least kPreGroups groups per row (zero-slot padding),
    // so the first ones are loaded and gathered without a per-row test; they
    // are requested one row ahead, off the gathers' critical path
    uint2 w_next[kPreGroups];
#pragma unroll
    for (int g = 0; g < kPreGroups; ++g)
      w_next[g] = tid < du ? __ldg(A.ell4 + (size_t)g * du + tid) : make_uint2(0u, 0u);
    for (uint32_t i = tid; i < du; i += bd) {
      const uint32_t c = c_next;
      const uint32_t gp = c & 0xffu, gt = gp + (c >> 8);
      uint2 w[kPreGroups];
#pragma unroll
      for (int g = 0; g < kPreGroups; ++g) w[g] = w_next[g];
      if (i + bd < du) {
#pragma unroll
        for (int g = 0; g < kPreGroups; ++g) w_next[g] = __ldg(A.ell4 + (size_t)g * du + i + bd);
      }
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
// pass D, lean form: one VEC-chunk per lane per sweep (32*VEC rows), so a
// thread holds few registers and eight 256-thread blocks fit on an SM; the
// neighbour columns of an item (at most 32 of them in one register per lane)
// are read once per item, not once per sweep.

template <int VEC, bool NEG>
__device__ __forceinline__ void passD5_accum(const int64_t* __restrict__ x, uint32_t du,
                                             uint32_t ccol, uint32_t kf, uint32_t kt, uint32_t ir,
                                             int64_t (&acc)[VEC]) {
#pragma unroll 4
  for (uint32_t k = kf; k < kt; ++k) {
    const uint32_t b = __shfl_sync(0xffffffffu, ccol, (int)k);
    const int64_t* src = x + (size_t)b * du + ir;
    if (VEC == 2) {
      const longlong2 v = __ldcg(reinterpret_cast<const longlong2*>(src));
      acc[0] += NEG ? -v.x : v.x;
      acc[VEC - 1] += NEG ? -v.y : v.y;
    } else {
      const int64_t v = __ldcg(src);
      acc[0] += NEG ? -v : v;
    }
  }
}

// Items (band, down state) are numbered in 32 bits (launch contract:
// nbands * dd < 2^32).  A row's hops are summed with their signs into one
// accumulator per element (exact: |sum| < 2^61).
template <int VEC, bool FAST, bool DOT, int MINB>
__global__ void __launch_bounds__(256, MINB) k_fx_passD5(FxProdArgs A) {
  const uint32_t du = A.du, dd = A.dd;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const uint32_t items = A.nbands * dd;
  constexpr uint32_t kSweep = 32u * VEC;
  I128 dot = {0, 0};
  for (uint32_t it = warp; it < items; it += nwarps) {
    const uint32_t band = it / dd, a = it - band * dd;
    const uint32_t r0 = band * A.band, r1 = min(du, r0 + A.band);
    const uint32_t k0 = A.rp_dn[a], np = A.rs_dn[a] - k0, nt = A.rp_dn[a + 1] - k0;
    for (uint32_t i0 = r0; i0 < r1; i0 += kSweep) {
      const uint32_t ia = i0 + lane * VEC;
      // lanes past the band's end read a valid row of the band (r0) and drop it
      const uint32_t ir = ia < r1 ? ia : r0;
      int64_t acc[VEC];
#pragma unroll
      for (int e = 0; e < VEC; ++e) acc[e] = 0;
      for (uint32_t kc = 0; kc < nt; kc += 32u) {  // neighbour columns, 32 at a time
        const uint32_t ccol = (kc + lane < nt) ? __ldg(A.col_dn + k0 + kc + lane) : 0u;
        const uint32_t e = min(32u, nt - kc);
        const uint32_t spos = np > kc ? min(e, np - kc) : 0u;
        passD5_accum<VEC, false>(A.x, du, ccol, 0u, spos, ir, acc);
        passD5_accum<VEC, true>(A.x, du, ccol, spos, e, ir, acc);
      }
      if (ia >= r1) continue;
      const size_t at = (size_t)a * du + ia;
      auto term = [&](int64_t v) {
        return FAST ? rshift_fixed(v, A.t_dn, A.r_dn) : mul_fix(v, A.mt_dn, A.sh_dn);
      };
      if constexpr (VEC == 2) {
        longlong2* yp = reinterpret_cast<longlong2*>(A.y + at);
        longlong2 v = __ldcs(yp);
        v.x += term(acc[0]);
        v.y += term(acc[1]);
        __stcs(yp, v);
        if (DOT) {
          const longlong2 xv = __ldcg(reinterpret_cast<const longlong2*>(A.dot_x + at));
          dot = add128(dot, shr128(mul_s64(v.x, xv.x), kDotShift));
          dot = add128(dot, shr128(mul_s64(v.y, xv.y), kDotShift));
        }
      } else {
        const int64_t v = __ldcs(A.y + at) + term(acc[0]);
        __stcs(A.y + at, v);
        if (DOT) dot = add128(dot, shr128(mul_s64(v, __ldcg(A.dot_x + at)), kDotShift));
      }
    }
  }
  if (DOT) block_store128(dot, A.dot_part);  // every thread of the block gets here
}

// ---------------------------------------------------------------------------
// tables

// Grouped ELL: row i holds ceil(np/4) groups of its positive hop columns,
// then ceil(nn/4) groups of its negative ones, four 16-bit columns per
// group, padded with zero slots (dim..dim+15, behind each staged slab);
// ell4[g * dim + i] is group g of row i and cnt4[i] = positive groups |
// (negative groups << 8).
bool build_ell4(const DevBuf<uint32_t>& rp, const DevBuf<uint32_t>& rs, const DevBuf<uint32_t>& col,
                uint32_t dim, cudaStream_t s, DevBuf<uint2>& ell4, DevBuf<uint16_t>& cnt4) {
  if (dim == 0 || dim + kZeroSlots > 65536u) return false;
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
  // (column mod 16).  A row's columns may take any order within its positive
  // and its negative slot range, and a row may read a zero slot (one per
  // bank pair) in any slot of its range that it does not need.  So, slot by
  // slot, rows are matched to distinct bank pairs (a maximum bipartite
  // matching by augmenting paths, rows whose remaining columns leave them the
  // least slack first); an unmatched row with no slack left takes a column
  // anyway (a conflict), and the others read the zero slot of a bank pair
  // the slot leaves free.  On the 4x4 half bases this brings the wavefronts
  // from ~1.55x to ~1.06x the slot count (a per-slot greedy choice of the
  // least-used bank pair got ~1.55x).
  for (uint32_t i = 0; i < dim; ++i) {
    const uint32_t np = hrs[i] - hrp[i], nn = hrp[i + 1] - hrs[i];
    hc[i] = (uint16_t)(((np + 3) / 4) | (((nn + 3) / 4) << 8));
  }
  // the zero slot on bank pair p
  auto zero_on = [&](uint32_t p) { return (uint16_t)(dim + (p + 16u - dim % 16u) % 16u); };
  std::vector<std::vector<uint32_t>> remp(16), remn(16);
  std::vector<uint32_t>* lst[16] = {};
  uint32_t order[16];
  double slack[16];
  int owner[16], choice[16];
  auto augment = [&](auto&& self, int r, uint32_t& seen) -> bool {
    for (uint32_t c : *lst[r]) {
      const uint32_t b = c % 16u;
      if ((seen >> b) & 1u) continue;
      seen |= 1u << b;
      if (owner[b] < 0 || self(self, owner[b], seen)) {
        owner[b] = r;
        choice[r] = (int)c;
        return true;
      }
    }
    return false;
  };
  for (uint32_t b0 = 0; b0 < dim; b0 += 16) {
    const uint32_t nr = std::min<uint32_t>(16, dim - b0);
    uint32_t kmax = 4u * kPreGroups;
    for (uint32_t r = 0; r < nr; ++r) {
      const uint32_t i = b0 + r;
      remp[r].assign(hcol.begin() + hrp[i], hcol.begin() + hrs[i]);
      remn[r].assign(hcol.begin() + hrs[i], hcol.begin() + hrp[i + 1]);
      kmax = std::max<uint32_t>(kmax, 4u * ((hc[i] & 0xffu) + (hc[i] >> 8)));
    }
    for (uint32_t k = 0; k < kmax; ++k) {
      uint32_t nl = 0;
      for (uint32_t r = 0; r < nr; ++r) {
        const uint32_t c = hc[b0 + r], gp = c & 0xffu, gt = gp + (c >> 8);
        lst[r] = nullptr;
        if (k < 4 * gp) {
          lst[r] = &remp[r];
          slack[r] = (double)(4 * gp - k) - (double)remp[r].size();
        } else if (k < 4 * gt) {
          lst[r] = &remn[r];
          slack[r] = (double)(4 * gt - k) - (double)remn[r].size();
        }
        if (lst[r] && lst[r]->empty()) lst[r] = nullptr;
        choice[r] = -1;
        if (lst[r]) order[nl++] = r;
      }
      std::stable_sort(order, order + nl, [&](uint32_t p, uint32_t q) { return slack[p] < slack[q]; });
      for (int b = 0; b < 16; ++b) owner[b] = -1;
      for (uint32_t q = 0; q < nl; ++q) {
        uint32_t seen = 0;
        augment(augment, (int)order[q], seen);
      }
      uint32_t used = 0;
      for (uint32_t r = 0; r < nr; ++r) {
        if (!lst[r]) continue;
        if (choice[r] < 0 && slack[r] > 0.5) continue;  // pads this slot, places later
        const uint32_t c = choice[r] >= 0 ? (uint32_t)choice[r] : lst[r]->front();
        lst[r]->erase(std::find(lst[r]->begin(), lst[r]->end(), c));
        used |= 1u << (c % 16u);
        cols[((size_t)(k / 4) * dim + b0 + r) * 4 + (k % 4)] = (uint16_t)c;
        choice[r] = (int)c;
      }
      // padding lanes of this slot read one zero slot, on a bank pair the slot
      // leaves free when there is one
      uint32_t p = (uint32_t)__builtin_ctz(~used | 0x10000u) & 15u;
      const uint16_t zp = zero_on(p);
      for (uint32_t r = 0; r < nr; ++r) {
        const uint32_t c = hc[b0 + r], gt = (c & 0xffu) + (c >> 8);
        const bool active = k < 4u * std::max<uint32_t>(gt, kPreGroups);
        if (active && choice[r] < 0) cols[((size_t)(k / 4) * dim + b0 + r) * 4 + (k % 4)] = zp;
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
  if (du < 64 || du + kZeroSlots > 65536u) return 0;
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
  if (items >= (1ull << 32)) throw Error(QCMG_ERR_ARG, "sector too large for pass D's 32-bit item numbers");
  auto go = [&](auto kern) {
    int per_sm = 0;
    QCMG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, 0));
    per_sm = std::max(1, std::min(per_sm, 8));  // dot partials: at most 8 blocks per SM
    const unsigned g = (unsigned)std::max<size_t>(1, std::min<size_t>((items + 7) / 8, (size_t)sms * per_sm));
    kern<<<g, 256, 0, s>>>(A);
    return g;
  };
  // six 256-thread blocks per SM (40 registers) for the product; five for
  // the Lanczos form, whose 128-bit dot accumulator needs the registers
  const bool even = (H->du & 1u) == 0u;
  unsigned gD;
  if (A.dot_part) {
    if (even) gD = fast ? go(k_fx_passD5<2, true, true, 5>) : go(k_fx_passD5<2, false, true, 5>);
    else gD = fast ? go(k_fx_passD5<1, true, true, 5>) : go(k_fx_passD5<1, false, true, 5>);
  } else {
    if (even) gD = fast ? go(k_fx_passD5<2, true, false, 6>) : go(k_fx_passD5<2, false, false, 6>);
    else gD = fast ? go(k_fx_passD5<1, true, false, 6>) : go(k_fx_passD5<1, false, false, 6>);
  }
  QCMG_CUDA(cudaGetLastError());
  return gD;
}

}  // namespace qcmg
