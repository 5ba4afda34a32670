// FX64 fast path: the factorized product and the Lanczos recurrence on
// fixed-point vectors (see qcmg_fx.cuh for the number format).
//
// Product y (+)= H x in two passes over the sector, stored like the
// reference's vector (up index fastest, one contiguous slab per down state):
//   pass U  one CTA per slab: the slab of x is staged in shared memory and
//           every up-spin hop is an integer gather-add from it; the
//           diagonal (one-body diagonal + density-density terms) and the
//           accumulated input are added; the slab of y is written once.
//   pass D  row bands: the CTAs sweep the down states of one band of rows at
//           a time, so the band of x (~48 MB) stays L2-resident while every
//           down-spin hop adds a neighbour slab segment.
// Both passes read 8 B and write 8 B per state from HBM; the hop gathers hit
// shared memory and L2.  Hop values must share one magnitude per spin
// (the Hubbard form: hops are +-t); other Hamiltonians use the FP64 path.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "qcmg_fx.cuh"
#include "qcmg_tma.cuh"
#include "qcmg_fxpath.h"
#include "qcmg_fxprod.h"
#include "qcmg_internal.h"
#include "qcmg_tridiag.h"

namespace qcmg {

// ---------------------------------------------------------------------------
// host helpers

// x = m * 2^e with |m| < 2^53 (m = 0 for x = 0).
static void split_double(double x, int64_t* m, int* e) {
  if (x == 0.0 || !std::isfinite(x)) {
    *m = 0;
    *e = 0;
    return;
  }
  int ex;
  double f = std::frexp(x, &ex);  // x = f 2^ex, 0.5 <= |f| < 1
  *m = (int64_t)std::llround(std::ldexp(f, 53));
  *e = ex - 53;
}

static int ceil_log2(double x) {
  if (x <= 0.0) return 0;
  int ex;
  double f = std::frexp(x, &ex);  // x = f 2^ex
  return (f == 0.5) ? ex - 1 : ex;
}

static int bitlen(uint64_t v) {
  int n = 0;
  while (v) {
    ++n;
    v >>= 1;
  }
  return n;
}

static unsigned grid_ew(size_t n, int per_sm = 8) {
  size_t g = (n + 255) / 256;
  g = std::max<size_t>(1, std::min<size_t>(g, (size_t)152 * per_sm));
  return (unsigned)g;
}

// ---------------------------------------------------------------------------
// device kernels: conversions and reductions

__global__ void k_absmax_f64(const double* __restrict__ x, size_t n,
                             unsigned long long* __restrict__ out) {
  unsigned long long m = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    unsigned long long b = (unsigned long long)__double_as_longlong(x[i]) & 0x7fffffffffffffffull;
    m = max(m, b);
  }
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

__global__ void k_f64_to_fx(const double* __restrict__ x, int64_t* __restrict__ q, size_t n,
                            int E) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    q[i] = f64_to_fx(x[i], E);
}

__global__ void k_fx_to_f64(const int64_t* __restrict__ q, double* __restrict__ x, size_t n,
                            int E, double c) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    x[i] = c * fx_to_f64(q[i], E);
}

// y (+)= c q 2^E straight into the caller's page-locked host vector (zero
// copy).  Elements below m take their old value from ypre, a device copy
// prefetched while the product ran, and are only written (one link
// direction); the others are read and written in host memory (both
// directions at once).  V2: y is 16-byte aligned and m even, two elements
// per access.
template <bool V2>
__global__ void k_fx_to_host(const int64_t* __restrict__ q, double* __restrict__ yh,
                             const double* __restrict__ ypre, size_t m, size_t n, int E, double c,
                             int acc) {
  const size_t step = (size_t)gridDim.x * blockDim.x;
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (V2) {
    double2* y2 = reinterpret_cast<double2*>(yh);
    const double2* p2 = reinterpret_cast<const double2*>(ypre);
    for (; i < n / 2; i += step) {
      double2 v = make_double2(c * fx_to_f64(q[2 * i], E), c * fx_to_f64(q[2 * i + 1], E));
      if (acc) {
        const double2 o = 2 * i < m ? p2[i] : y2[i];
        v.x += o.x;
        v.y += o.y;
      }
      y2[i] = v;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && (n & 1)) {
      const double v = c * fx_to_f64(q[n - 1], E);
      yh[n - 1] = acc ? (n - 1 < m ? ypre[n - 1] : yh[n - 1]) + v : v;
    }
  } else {
    for (; i < n; i += step) {
      const double v = c * fx_to_f64(q[i], E);
      yh[i] = acc ? (i < m ? ypre[i] : yh[i]) + v : v;
    }
  }
}

constexpr int kRedBlocksFx = 1024;

// Exact <a, b> partials, two elements per 16-byte load (the fixed-point
// vectors come from cudaMalloc, so even indices are 16-byte aligned); the
// integer sums are exact, so the summation order does not matter.
__global__ void __launch_bounds__(256) k_fx_dot(const int64_t* __restrict__ a,
                                                const int64_t* __restrict__ b, size_t n,
                                                I128* __restrict__ part) {
  I128 s = {0, 0};
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t n2 = n / 2;
  const longlong2* a2 = reinterpret_cast<const longlong2*>(a);
  const longlong2* b2 = reinterpret_cast<const longlong2*>(b);
#pragma unroll 2
  for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n2; j += stride) {
    const longlong2 x = __ldcs(a2 + j), y = __ldcs(b2 + j);
    s = add128(s, shr128(mul_s64(x.x, y.x), kDotShift));
    s = add128(s, shr128(mul_s64(x.y, y.y), kDotShift));
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0)
    s = add128(s, shr128(mul_s64(a[n - 1], b[n - 1]), kDotShift));
  block_store128(s, part);
}

// Sum of the block partials by one warp (launched with 32 threads).
__global__ void k_fx_final(const I128* __restrict__ part, int np, I128* __restrict__ out) {
  I128 s = {0, 0};
  for (int i = threadIdx.x; i < np; i += blockDim.x) s = add128(s, part[i]);
  s = warp_sum128(s);
  if (threadIdx.x == 0) *out = s;
}

// Fused Lanczos update:
//   q_o = round(q_w * 2^-sw) - round(q_v * ma 2^-sa) - round(q_p * mb 2^-sb)
// written over q_w, with exact |q_o|^2 partials and max|q_o|.
__global__ void __launch_bounds__(256) k_fx_update(int64_t* __restrict__ w,
                                                   const int64_t* __restrict__ v,
                                                   const int64_t* __restrict__ p, size_t n, int sw,
                                                   int64_t ma, int sa, int64_t mb, int sb,
                                                   I128* __restrict__ part,
                                                   unsigned long long* __restrict__ qmax) {
  I128 s = {0, 0};
  unsigned long long m = 0;
  auto one = [&](int64_t wi, int64_t vi, int64_t pi) {
    int64_t o = shr_round(wi, sw);
    if (ma) o -= mul_fix(vi, ma, sa);
    if (p && mb) o -= mul_fix(pi, mb, sb);
    s = add128(s, shr128(mul_s64(o, o), kDotShift));
    m = max(m, (unsigned long long)(o < 0 ? -o : o));
    return o;
  };
  // two elements per 16-byte load (cudaMalloc'd vectors: even indices are
  // 16-byte aligned); w, v and p are each read once and streamed
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t n2 = n / 2;
  longlong2* w2 = reinterpret_cast<longlong2*>(w);
  const longlong2* v2 = reinterpret_cast<const longlong2*>(v);
  const longlong2* p2 = reinterpret_cast<const longlong2*>(p);
#pragma unroll 2
  for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n2; j += stride) {
    const longlong2 wv = __ldcs(w2 + j), vv = __ldcs(v2 + j);
    const longlong2 pv = p ? __ldcs(p2 + j) : make_longlong2(0, 0);
    longlong2 o;
    o.x = one(wv.x, vv.x, pv.x);
    o.y = one(wv.y, vv.y, pv.y);
    __stcs(w2 + j, o);
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0)
    w[n - 1] = one(w[n - 1], v[n - 1], p ? p[n - 1] : 0);
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(qmax, m);
  block_store128(s, part);
}

// g = round(g * 2^-sg) + round(q * m 2^-s)   (eigenvector accumulation)
__global__ void k_fx_axpy(int64_t* __restrict__ g, const int64_t* __restrict__ q, size_t n, int sg,
                          int64_t m, int s) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    g[i] = shr_round(g[i], sg) + mul_fix(q[i], m, s);
}

// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// tables

static void build_unit_csr(const HalfOp& op, cudaStream_t s, DevBuf<uint32_t>& rp,
                           DevBuf<uint32_t>& rs, DevBuf<uint32_t>& col, double* tmag,
                           int* maxdeg, bool* ok) {
  std::vector<uint32_t> hrp(op.dim + 1), hcol(op.nnz);
  std::vector<double> hval(op.nnz);
  if (op.dim) QCMG_CUDA(cudaMemcpyAsync(hrp.data(), op.rowptr.p, (op.dim + 1) * 4, cudaMemcpyDeviceToHost, s));
  if (op.nnz) {
    QCMG_CUDA(cudaMemcpyAsync(hcol.data(), op.col.p, op.nnz * 4, cudaMemcpyDeviceToHost, s));
    QCMG_CUDA(cudaMemcpyAsync(hval.data(), op.val.p, op.nnz * 8, cudaMemcpyDeviceToHost, s));
  }
  QCMG_CUDA(cudaStreamSynchronize(s));
  double t = 0.0;
  for (double v : hval) {
    if (t == 0.0) t = std::fabs(v);
    if (std::fabs(v) != t) {
      *ok = false;
      return;
    }
  }
  *tmag = t;
  std::vector<uint32_t> nrp(op.dim + 1), nrs(std::max<uint32_t>(op.dim, 1)), ncol(op.nnz);
  int md = 0;
  for (uint32_t i = 0; i < op.dim; ++i) {
    uint32_t pos = hrp[i];
    nrp[i] = pos;
    for (uint32_t k = hrp[i]; k < hrp[i + 1]; ++k)
      if (hval[k] > 0) ncol[pos++] = hcol[k];
    nrs[i] = pos;
    for (uint32_t k = hrp[i]; k < hrp[i + 1]; ++k)
      if (hval[k] < 0) ncol[pos++] = hcol[k];
    md = std::max<int>(md, (int)(hrp[i + 1] - hrp[i]));
  }
  nrp[op.dim] = hrp[op.dim];
  *maxdeg = md;
  rp.upload(nrp.data(), op.dim + 1, s);
  rs.upload(nrs.data(), nrs.size(), s);
  if (op.nnz)
    col.upload(ncol.data(), op.nnz, s);
  else
    col.alloc(1);
  QCMG_CUDA(cudaStreamSynchronize(s));  // host staging vectors go out of scope
}

__global__ void k_diag_to_fx(const double* __restrict__ d, int64_t* __restrict__ out, size_t n,
                             double scale) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = (int64_t)llrint(d[i] * scale);  // set-up only
}

bool fx_prepare(qcmg_hamiltonian* H) {
  FxTables& T = H->fx;
  if (T.state != 0) return T.state > 0;
  T.state = -1;
  if (H->dim == 0 || H->du >= (1u << 31) || H->dd >= (1u << 31)) return false;
  int max_optin = 0;
  QCMG_CUDA(cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, H->device));
  if ((size_t)H->du * 8 > (size_t)max_optin) return false;  // slab must fit in shared memory
  cudaStream_t s = H->stream;
  bool ok = true;
  build_unit_csr(H->up, s, T.rp_up, T.rs_up, T.col_up, &T.t_up, &T.maxdeg_up, &ok);
  if (!ok) return false;
  build_unit_csr(H->dn, s, T.rp_dn, T.rs_dn, T.col_dn, &T.t_dn, &T.maxdeg_dn, &ok);
  if (!ok) return false;
  // pass U with bulk-copied slabs: grouped ELL table and slabs per round
  T.ns = choose_slabs_per_pass(H->du, max_optin);
  if (T.ns > 0 && !build_ell4(T.rp_up, T.rs_up, T.col_up, H->du, s, T.ell4, T.cnt4)) T.ns = 0;
  T.err.alloc(1);
  QCMG_CUDA(cudaMemsetAsync(T.err.p, 0, sizeof(int), s));
  // diagonal bound and fixed-point scale 2^-G
  std::vector<double> hdu(H->du), hdd(H->dd), hw;
  QCMG_CUDA(cudaMemcpyAsync(hdu.data(), H->up.diag.p, H->du * 8, cudaMemcpyDeviceToHost, s));
  QCMG_CUDA(cudaMemcpyAsync(hdd.data(), H->dn.diag.p, H->dd * 8, cudaMemcpyDeviceToHost, s));
  if (H->inter_kind == QCMG_INTER_GENERAL) {
    hw.resize((size_t)H->dd * H->L);
    QCMG_CUDA(cudaMemcpyAsync(hw.data(), H->wdn.p, hw.size() * 8, cudaMemcpyDeviceToHost, s));
  }
  QCMG_CUDA(cudaStreamSynchronize(s));
  double mu = 0.0, md = 0.0, mw = 0.0;
  for (double v : hdu) mu = std::max(mu, std::fabs(v));
  for (double v : hdd) md = std::max(md, std::fabs(v));
  if (H->inter_kind == QCMG_INTER_ONSITE) mw = std::fabs(H->U) * H->L;
  if (H->inter_kind == QCMG_INTER_GENERAL)
    for (uint32_t i = 0; i < H->dd; ++i) {
      double s2 = 0.0;
      for (int r = 0; r < H->L; ++r) s2 += std::fabs(hw[(size_t)i * H->L + r]);
      mw = std::max(mw, s2);
    }
  const double dmax = mu + md + mw;
  T.G = 61 - ceil_log2(std::max(dmax, 1.0));
  const double scale = std::ldexp(1.0, T.G);
  T.dup.alloc(H->du);
  T.ddn.alloc(H->dd);
  k_diag_to_fx<<<grid_ew(H->du), 256, 0, s>>>(H->up.diag.p, T.dup.p, H->du, scale);
  k_diag_to_fx<<<grid_ew(H->dd), 256, 0, s>>>(H->dn.diag.p, T.ddn.p, H->dd, scale);
  T.U = (int64_t)std::llrint(H->U * scale);
  if (H->inter_kind == QCMG_INTER_GENERAL) {
    T.wdn.alloc(hw.size());
    k_diag_to_fx<<<grid_ew(hw.size()), 256, 0, s>>>(H->wdn.p, T.wdn.p, hw.size(), scale);
  }
  QCMG_CUDA(cudaGetLastError());
  // Narrow diagonal: when every diagonal entry at scale 2^-G is a multiple of
  // 2^tz and |D| >> tz stays below 2^6 (small-integer energies such as the
  // Hubbard model's), x * (D >> tz) fits in 63 bits and the diagonal term is
  // one 64-bit product and a rounding shift, bit-identical to the 128-bit one.
  {
    int tz = 63;
    auto fold = [&](double v) {
      const long long q = std::llrint(v * scale);  // the value k_diag_to_fx stores
      if (q != 0) tz = std::min(tz, __builtin_ctzll((unsigned long long)q));
    };
    for (double v : hdu) fold(v);
    for (double v : hdd) fold(v);
    for (double v : hw) fold(v);
    if (H->inter_kind == QCMG_INTER_ONSITE) fold(H->U);
    const double dbound = std::ceil(dmax * scale);
    T.dtz = (std::ldexp(dbound, -tz) < 64.0) ? tz : -1;
    if (T.dtz >= 0) {
      auto narrow = [&](const std::vector<double>& src, DevBuf<int32_t>& dst) {
        std::vector<int32_t> h(std::max<size_t>(src.size(), 1), 0);
        for (size_t k = 0; k < src.size(); ++k) h[k] = (int32_t)(std::llrint(src[k] * scale) >> T.dtz);
        dst.upload(h.data(), h.size(), s);
      };
      narrow(hdu, T.dup32);
      narrow(hdd, T.ddn32);
      narrow(hw, T.wdn32);
      T.U32 = (int32_t)(std::llrint(H->U * scale) >> T.dtz);
      QCMG_CUDA(cudaStreamSynchronize(s));  // host staging vectors go out of scope
    }
  }
  T.bound = dmax + T.t_up * T.maxdeg_up + T.t_dn * T.maxdeg_dn;
  T.b = ceil_log2(std::max(T.bound, 1.0));
  // rows per band of pass D: ~48 MB of x per band (QCMG_FX_BAND_MB overrides)
  double band_mb = 48.0;
  if (const char* v = std::getenv("QCMG_FX_BAND_MB")) band_mb = std::max(1.0, std::atof(v));
  size_t band = (size_t)(band_mb * 1.0e6 / (8.0 * std::max<uint32_t>(H->dd, 1)));
  band = std::max<size_t>(256, (band / 256) * 256);
  T.band = (uint32_t)std::min<size_t>(band, H->du);
  T.state = 1;
  return true;
}

// ---------------------------------------------------------------------------
// FX vectors

void FxVec::alloc(size_t count) {
  buf.alloc(count);
  n = count;
}

void fx_from_f64(const double* x, size_t n, FxVec& v, cudaStream_t s, DevBuf<unsigned long long>& tmp) {
  v.alloc(n);
  tmp.alloc(1);
  QCMG_CUDA(cudaMemsetAsync(tmp.p, 0, 8, s));
  k_absmax_f64<<<grid_ew(n), 256, 0, s>>>(x, n, tmp.p);
  unsigned long long hb = 0;
  QCMG_CUDA(cudaMemcpyAsync(&hb, tmp.p, 8, cudaMemcpyDeviceToHost, s));
  QCMG_CUDA(cudaStreamSynchronize(s));
  double mx;
  std::memcpy(&mx, &hb, 8);
  v.c = 1.0;
  if (mx == 0.0) {
    v.E = 0;
    v.mb = 0;
    QCMG_CUDA(cudaMemsetAsync(v.buf.p, 0, n * 8, s));
    return;
  }
  v.E = ceil_log2(mx) - kFxBits;  // |q| <= 2^56
  k_f64_to_fx<<<grid_ew(n), 256, 0, s>>>(x, v.buf.p, n, v.E);
  QCMG_CUDA(cudaGetLastError());
  v.mb = kFxBits;
}

void fx_to_f64(const FxVec& v, double* x, cudaStream_t s) {
  k_fx_to_f64<<<grid_ew(v.n), 256, 0, s>>>(v.buf.p, x, v.n, v.E, v.c);
  QCMG_CUDA(cudaGetLastError());
}

// exact <a, b> as a double
double FxReducer::dot(const FxVec& a, const FxVec& b, cudaStream_t s) {
  part.alloc(kRedBlocksFx);
  out.alloc(1);
  unsigned g = (unsigned)std::min<size_t>(kRedBlocksFx, std::max<size_t>(1, (a.n + 255) / 256));
  k_fx_dot<<<g, 256, 0, s>>>(a.buf.p, b.buf.p, a.n, part.p);
  k_fx_final<<<1, 32, 0, s>>>(part.p, (int)g, out.p);
  QCMG_CUDA(cudaGetLastError());
  I128 h;
  QCMG_CUDA(cudaMemcpyAsync(&h, out.p, sizeof(I128), cudaMemcpyDeviceToHost, s));
  QCMG_CUDA(cudaStreamSynchronize(s));
  double r = std::ldexp((double)h.hi, 64) + (double)h.lo;
  return a.c * b.c * std::ldexp(r, kDotShift + a.E + b.E);
}

// ---------------------------------------------------------------------------
// the product

// y = H x  (or y = H x + gamma * yin with yin != nullptr, yin may be &y).
// The output exponent follows from the bound |H|_inf (T.b) and the input's
// largest component; c_y = c_x.
void fx_matvec(qcmg_hamiltonian* H, const FxVec& x, FxVec& y, const FxVec* yin, double gamma,
               FxReducer* dot, double* dot_out) {
  FxTables& T = H->fx;
  cudaStream_t s = H->stream;
  const size_t n = H->dim;
  if (y.n != n) y.alloc(n);
  // bound on the output's real magnitude, in units of c_x
  double bound = std::ldexp(T.bound, x.E + x.mb);
  if (yin && yin->mb > 0) bound += std::fabs(gamma * yin->c / x.c) * std::ldexp(1.0, yin->E + yin->mb);
  int Eo = ceil_log2(bound) - kFxBits;
  FxProdArgs A;
  A.du = H->du;
  A.dd = H->dd;
  A.L = H->L;
  A.rp_up = T.rp_up.p;
  A.rs_up = T.rs_up.p;
  A.col_up = T.col_up.p;
  A.rp_dn = T.rp_dn.p;
  A.rs_dn = T.rs_dn.p;
  A.col_dn = T.col_dn.p;
  A.dup = T.dup.p;
  A.ddn = T.ddn.p;
  A.bin_up = H->up.bin.p;
  A.bin_dn = H->dn.bin.p;
  A.U = T.U;
  A.wdn = T.wdn.p;
  int e;
  split_double(T.t_up, &A.mt_up, &e);
  A.sh_up = Eo - x.E - e;
  split_double(T.t_dn, &A.mt_dn, &e);
  A.sh_dn = Eo - x.E - e;
  A.sh_d = Eo - x.E + T.G;
  A.d_tz = T.dtz;
  A.p2_up = pow2_exponent(A.mt_up);
  A.p2_dn = pow2_exponent(A.mt_dn);
  A.yin = nullptr;
  A.m_in = 0;
  A.sh_in = 0;
  A.p2_in = -1;
  if (yin && yin->mb > 0 && gamma != 0.0) {
    A.yin = yin->buf.p;
    split_double(gamma * yin->c / x.c, &A.m_in, &e);
    A.sh_in = Eo - yin->E - e;
    A.p2_in = pow2_exponent(A.m_in);
  }
  // fixed shifts of the FAST kernels (used only when every multiplier is a
  // power of two and the diagonal is narrow)
  auto fixed = [](int t, int* to, int64_t* ro) {
    t = std::min(t, 63);
    *to = t;
    *ro = t > 0 ? (int64_t)(1ull << (t - 1)) : 0;
  };
  fixed(A.sh_up - A.p2_up, &A.t_up, &A.r_up);
  fixed(A.sh_dn - A.p2_dn, &A.t_dn, &A.r_dn);
  fixed(A.sh_d - T.dtz, &A.t_d, &A.r_d);
  fixed(A.sh_in - A.p2_in, &A.t_in, &A.r_in);
  A.neg_in = A.m_in < 0;
  A.dup32 = T.dup32.p;
  A.ddn32 = T.ddn32.p;
  A.wdn32 = T.wdn32.p;
  A.U32 = T.U32;
  A.x = x.buf.p;
  A.y = y.buf.p;
  A.band = T.band;
  A.nbands = (H->du + T.band - 1) / T.band;
  A.ell4 = T.ell4.p;
  A.cnt4 = T.cnt4.p;
  A.err = T.err.p;
  A.dot_x = nullptr;
  A.dot_part = nullptr;
  if (dot) {
    int sms = 0;
    QCMG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, H->device));
    dot->part.alloc(std::max<size_t>(kRedBlocksFx, product_dot_partials(sms)));
    dot->out.alloc(1);
    A.dot_x = x.buf.p;
    A.dot_part = dot->part.p;
  }
  const unsigned np = launch_product(H, A, s);
  y.E = Eo;
  y.mb = kFxBits;
  y.c = x.c;
  if (dot) {
    k_fx_final<<<1, 32, 0, s>>>(dot->part.p, (int)np, dot->out.p);
    QCMG_CUDA(cudaGetLastError());
    I128 h;
    QCMG_CUDA(cudaMemcpyAsync(&h, dot->out.p, sizeof(I128), cudaMemcpyDeviceToHost, s));
    QCMG_CUDA(cudaStreamSynchronize(s));
    const double r = std::ldexp((double)h.hi, 64) + (double)h.lo;
    *dot_out = x.c * y.c * std::ldexp(r, kDotShift + x.E + y.E);
  }
}

void fx_check_error(qcmg_hamiltonian* H) {
  int err = 0;
  if (!H->fx.err.p) return;
  QCMG_CUDA(cudaMemcpyAsync(&err, H->fx.err.p, sizeof(int), cudaMemcpyDeviceToHost, H->stream));
  QCMG_CUDA(cudaStreamSynchronize(H->stream));
  if (err) throw Error(QCMG_ERR_CUDA, "a bulk copy into shared memory did not complete in time");
}

void fx_matvec_f64(qcmg_hamiltonian* H, const double* x, double* y, bool accumulate) {
  FxTables& T = H->fx;
  cudaStream_t s = H->stream;
  fx_from_f64(x, H->dim, T.x, s, T.tmp);
  if (accumulate) {
    fx_from_f64(y, H->dim, T.y, s, T.tmp);
    fx_matvec(H, T.x, T.y, &T.y, 1.0);
  } else {
    fx_matvec(H, T.x, T.y, nullptr, 0.0);
  }
  fx_to_f64(T.y, y, s);
}

// y_host (+)= H x for x on the device and y in page-locked host memory (its
// device-side address yh): H x in fixed point, then one pass that converts
// and accumulates into the host vector, the first m elements' old values
// read from ypre (device) once the event ypre_ready has fired.
void fx_matvec_to_host(qcmg_hamiltonian* H, const double* x, double* yh, bool accumulate,
                       cudaEvent_t product_done, const double* ypre, size_t m,
                       cudaEvent_t ypre_ready) {
  FxTables& T = H->fx;
  cudaStream_t s = H->stream;
  const size_t n = H->dim;
  fx_from_f64(x, n, T.x, s, T.tmp);
  fx_matvec(H, T.x, T.y, nullptr, 0.0);
  if (product_done) QCMG_CUDA(cudaEventRecord(product_done, s));
  if (m && ypre_ready) QCMG_CUDA(cudaStreamWaitEvent(s, ypre_ready, 0));
  const unsigned g = 152u * 8u;
  const int acc = accumulate ? 1 : 0;
  if (((uintptr_t)yh & 15u) == 0 && (m % 2) == 0)
    k_fx_to_host<true><<<g, 256, 0, s>>>(T.y.buf.p, yh, ypre, m, n, T.y.E, T.y.c, acc);
  else
    k_fx_to_host<false><<<g, 256, 0, s>>>(T.y.buf.p, yh, ypre, m, n, T.y.E, T.y.c, acc);
  QCMG_CUDA(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// Lanczos on FX vectors: the reference's recurrence (Lanczos.hpp:64-93)
// written with normalized vectors, w = H v_j - alpha v_j - beta v_{j-1}.

static void fx_update(qcmg_hamiltonian* H, FxVec& w, const FxVec& v, const FxVec* p, double alpha,
                      double beta, FxReducer& red, double* norm2) {
  cudaStream_t s = H->stream;
  const size_t n = w.n;
  // bound of the result in units of c_w
  double bw = std::ldexp(1.0, w.E + w.mb);
  double bv = std::fabs(alpha * v.c / w.c) * std::ldexp(1.0, v.E + v.mb);
  double bp = p ? std::fabs(beta * p->c / w.c) * std::ldexp(1.0, p->E + p->mb) : 0.0;
  int Eo = ceil_log2(bw + bv + bp) - kFxBits;
  int e;
  int64_t ma = 0, mb = 0;
  int sa = 0, sb = 0;
  split_double(alpha * v.c / w.c, &ma, &e);
  sa = Eo - v.E - e;
  if (p) {
    split_double(beta * p->c / w.c, &mb, &e);
    sb = Eo - p->E - e;
  }
  red.part.alloc(kRedBlocksFx);
  red.out.alloc(1);
  red.umax.alloc(1);
  QCMG_CUDA(cudaMemsetAsync(red.umax.p, 0, 8, s));
  unsigned g = (unsigned)std::min<size_t>(kRedBlocksFx, std::max<size_t>(1, (n + 255) / 256));
  k_fx_update<<<g, 256, 0, s>>>(w.buf.p, v.buf.p, p ? p->buf.p : nullptr, n, Eo - w.E, ma, sa, mb,
                                sb, red.part.p, red.umax.p);
  k_fx_final<<<1, 32, 0, s>>>(red.part.p, (int)g, red.out.p);
  QCMG_CUDA(cudaGetLastError());
  I128 h;
  unsigned long long um = 0;
  int err = 0;
  QCMG_CUDA(cudaMemcpyAsync(&h, red.out.p, sizeof(I128), cudaMemcpyDeviceToHost, s));
  QCMG_CUDA(cudaMemcpyAsync(&um, red.umax.p, 8, cudaMemcpyDeviceToHost, s));
  if (H->fx.err.p) QCMG_CUDA(cudaMemcpyAsync(&err, H->fx.err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  QCMG_CUDA(cudaStreamSynchronize(s));
  if (err) throw Error(QCMG_ERR_CUDA, "a bulk copy into shared memory did not complete in time");
  w.E = Eo;
  w.mb = bitlen(um);
  double r = std::ldexp((double)h.hi, 64) + (double)h.lo;
  *norm2 = w.c * w.c * std::ldexp(r, kDotShift + 2 * Eo);
}

LanczosResult fx_lanczos(qcmg_hamiltonian* H, const double* x0_dev, double tol, int max_iter,
                         double* psi_dev) {
  LanczosResult res;
  cudaStream_t s = H->stream;
  FxReducer red;
  DevBuf<unsigned long long> tmp;
  FxVec vbuf[3];
  FxVec x0;
  fx_from_f64(x0_dev, H->dim, x0, s, tmp);
  auto run = [&](bool replay, const std::vector<double>* z, FxVec* gs) {
    FxVec* v = &vbuf[0];
    FxVec* p = &vbuf[1];
    FxVec* w = &vbuf[2];
    v->alloc(H->dim);
    QCMG_CUDA(cudaMemcpyAsync(v->buf.p, x0.buf.p, H->dim * 8, cudaMemcpyDeviceToDevice, s));
    v->E = x0.E;
    v->mb = x0.mb;
    v->c = x0.c;
    bool have_p = false;
    double beta_prev = 0.0;
    std::vector<double> zz;
    const int nsteps = replay ? (int)z->size() : max_iter + 1;
    for (int j = 0; j < nsteps; ++j) {
      if (replay) {
        // gs += z_j v_j
        if (j == 0) {
          gs->alloc(H->dim);
          QCMG_CUDA(cudaMemsetAsync(gs->buf.p, 0, H->dim * 8, s));
          double bnd = 0.0;
          for (double zj : *z) bnd += std::fabs(zj);
          gs->E = ceil_log2(bnd) - kFxBits;  // |psi_i| <= sum_j |z_j| |v_j|_max <= sum |z_j|
          gs->c = 1.0;
          gs->mb = kFxBits;
        }
        int64_t m;
        int e;
        split_double((*z)[j] * v->c, &m, &e);
        k_fx_axpy<<<grid_ew(H->dim), 256, 0, s>>>(gs->buf.p, v->buf.p, H->dim, 0, m,
                                                  gs->E - v->E - e);
        QCMG_CUDA(cudaGetLastError());
        if (j + 1 == nsteps) break;
      }
      // alpha = <v, H v> comes out of the product's second pass
      double a = 0.0;
      if (replay) {
        fx_matvec(H, *v, *w, nullptr, 0.0);
        a = res.alpha[j];
      } else {
        fx_matvec(H, *v, *w, nullptr, 0.0, &red, &a);
      }
      double n2 = 0.0;
      fx_update(H, *w, *v, have_p ? p : nullptr, a, beta_prev, red, &n2);
      double b = replay ? res.beta[j] : std::sqrt(n2);
      if (!replay) {
        res.alpha.push_back(a);
        res.beta.push_back(b);
        res.energy = tridiag_lowest(res.alpha, res.beta, zz);
        double ritz = std::fabs(zz.back() * b);
        if (!std::isfinite(res.energy) || !std::isfinite(ritz))
          throw Error(QCMG_ERR_NUMERIC, "Lanczos produced a non-finite value");
        if (ritz <= tol || b == 0.0) break;
        if ((int)res.alpha.size() > max_iter)
          throw Error(QCMG_ERR_NOCONV,
                      "Lanczos procedure exceeded " + std::to_string(max_iter) + " iterations");
      }
      // rotate: p <- v, v <- w / beta, w <- old p.  The division only changes
      // the lazy scale; its power of two moves into the exponent (exact), so
      // c stays in [0.5, 1) and neither c nor 2^E drifts out of double range
      // over hundreds of iterations.
      int k2 = 0;
      w->c = std::frexp(w->c / b, &k2);
      w->E += k2;
      FxVec* t = p;
      p = v;
      v = w;
      w = t;
      have_p = true;
      beta_prev = b;
    }
    if (!replay) res.niter = (int)res.alpha.size();
    return zz;
  };
  std::vector<double> z = run(false, nullptr, nullptr);
  if (psi_dev) {
    FxVec gs;
    run(true, &z, &gs);
    fx_to_f64(gs, psi_dev, s);
    QCMG_CUDA(cudaStreamSynchronize(s));
  }
  return res;
}

}  // namespace qcmg
