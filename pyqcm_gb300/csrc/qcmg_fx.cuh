// Fixed-point (FX64) arithmetic for device-resident Krylov vectors.
//
// GB300 executes FP64 at ~1/64 of its FP32/INT32 rate (about 1 TFLOP/s),
// which makes every FP64 operation on a length-1e8 vector slower than the
// HBM stream it belongs to.  The Krylov vectors of the fast path are
// therefore held as 64-bit integers q_i with one binary exponent E per
// vector (value_i = c * 2^E * q_i, c a host-side double scale):
//   - the Hamiltonian's hops become exact integer additions;
//   - products by doubles use an exact 64x64 -> 128-bit product and one
//     rounding shift (mul_fix);
//   - dot products and norms accumulate exact 128-bit products.
// With |q_i| < 2^56 the representation error of a unit vector is below
// 2^-56 per component, i.e. at or below FP64's own normwise rounding.
#pragma once

#include <cstdint>

namespace qcmg {

constexpr int kFxBits = 56;  // |q| < 2^kFxBits for every stored vector

// 128-bit signed integer as (hi, lo).
struct I128 {
  int64_t hi;
  uint64_t lo;
};

__device__ __forceinline__ I128 mul_s64(int64_t a, int64_t b) {
  I128 r;
  r.lo = (uint64_t)a * (uint64_t)b;
  r.hi = __mul64hi(a, b);
  return r;
}

__device__ __forceinline__ I128 add128(I128 a, I128 b) {
  I128 r;
  r.lo = a.lo + b.lo;
  r.hi = a.hi + b.hi + (r.lo < a.lo ? 1 : 0);
  return r;
}

// Arithmetic right shift of a 128-bit value by s (s < 128), rounding to
// nearest (ties toward +infinity); s <= 0 shifts left by -s.  The caller
// guarantees that the result fits in 63 bits.
__device__ __forceinline__ int64_t shr128_round(I128 v, int s) {
  if (s <= 0) return (int64_t)(v.lo << (-s));
  if (s >= 127) return 0;
  // add 2^(s-1)
  I128 h;
  if (s - 1 < 64) {
    h.hi = 0;
    h.lo = 1ull << (s - 1);
  } else {
    h.hi = (int64_t)(1ull << (s - 1 - 64));
    h.lo = 0;
  }
  v = add128(v, h);
  if (s < 64) return (int64_t)((v.lo >> s) | ((uint64_t)v.hi << (64 - s)));
  return v.hi >> (s - 64);
}

// Dot products sum_i (a_i b_i >> kDotShift), accumulated as 128-bit integers
// (order-independent, so any split of the sum gives the same bits).
__device__ __forceinline__ I128 warp_sum128(I128 v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    I128 w;
    w.hi = __shfl_xor_sync(0xffffffffu, v.hi, o);
    w.lo = __shfl_xor_sync(0xffffffffu, v.lo, o);
    v = add128(v, w);
  }
  return v;
}

__device__ __forceinline__ I128 shr128(I128 v, int s) {  // arithmetic, 0 < s < 64
  I128 r;
  r.lo = (v.lo >> s) | ((uint64_t)v.hi << (64 - s));
  r.hi = v.hi >> s;
  return r;
}

constexpr int kDotShift = 20;

__device__ __forceinline__ void block_store128(I128 s, I128* part) {
  __shared__ int64_t shi[32];
  __shared__ uint64_t slo[32];
  s = warp_sum128(s);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) {
    shi[w] = s.hi;
    slo[w] = s.lo;
  }
  __syncthreads();
  if (w == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    I128 t;
    t.hi = lane < nw ? shi[lane] : 0;
    t.lo = lane < nw ? slo[lane] : 0;
    t = warp_sum128(t);
    if (lane == 0) part[blockIdx.x] = t;
  }
}

// round(a * m / 2^s)
__device__ __forceinline__ int64_t mul_fix(int64_t a, int64_t m, int s) {
  return shr128_round(mul_s64(a, m), s);
}

// mul_fix with a multiplier known to be +-2^p when p >= 0 (hop magnitude 1,
// accumulation factor 1): a shift with the same rounding, bit-identical to
// mul_fix for |a| < 2^62.  p < 0 falls back to the 128-bit product.
// round(v / 2^t) with mul_fix's rounding, for |v| < 2^62 (t <= 0: v * 2^-t).
__device__ __forceinline__ int64_t round_shift(int64_t v, int t) {
  if (t <= 0) return (int64_t)((uint64_t)v << (-t));
  if (t >= 63) return 0;
  return (v + (1ll << (t - 1))) >> t;
}

// round_shift with the shift t and the round term r = 2^(t-1) fixed for a
// launch (t <= 0: v * 2^-t).  The host clamps t to 63, where |v| < 2^62
// gives 0 as round_shift does.
__device__ __forceinline__ int64_t rshift_fixed(int64_t v, int t, int64_t r) {
  return t > 0 ? (v + r) >> t : (int64_t)((uint64_t)v << (-t));
}

__device__ __forceinline__ int64_t mul_fix_p2(int64_t a, int64_t m, int s, int p) {
  if (p >= 0) return round_shift(m < 0 ? -a : a, s - p);
  return mul_fix(a, m, s);
}

// Compile-time forms for kernels specialized on the multipliers: FAST = the
// multiplier is +-2^p and the diagonal is narrow, so no 128-bit code is
// generated at all (a runtime test alone leaves both forms in the kernel).
template <bool FAST>
__device__ __forceinline__ int64_t scale_term(int64_t a, int64_t m, int s, int p) {
  if (FAST) return round_shift(m < 0 ? -a : a, s - p);
  return mul_fix(a, m, s);
}

template <bool FAST>
__device__ __forceinline__ int64_t diag_term(int64_t x, int64_t D, int s, int tz) {
  if (FAST) return round_shift(x * (D >> tz), s - tz);
  return mul_fix(x, D, s);
}

// The diagonal term round(x * D / 2^s).  tz >= 0 means D is a multiple of
// 2^tz with |D >> tz| < 2^6, so x * (D >> tz) fits in 63 bits and one 64-bit
// product replaces the 128-bit one (bit-identical result); tz < 0 takes the
// 128-bit product.
__device__ __forceinline__ int64_t mul_fix_diag(int64_t x, int64_t D, int s, int tz) {
  if (tz >= 0) return round_shift(x * (D >> tz), s - tz);
  return mul_fix(x, D, s);
}

// Rounding arithmetic right shift of an int64 (s >= 0; s >= 63 gives 0 or -1 -> 0).
__device__ __forceinline__ int64_t shr_round(int64_t a, int s) {
  if (s <= 0) return a;
  if (s >= 63) return 0;
  return (a + (1ll << (s - 1))) >> s;
}

// double -> round(x * 2^-E) using integer operations only.
__device__ __forceinline__ int64_t f64_to_fx(double x, int E) {
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  const int ex = (int)((b >> 52) & 0x7ff);
  if (ex == 0) return 0;  // zero or subnormal (below any fixed-point quantum used here)
  const int64_t mant = (int64_t)((b & ((1ull << 52) - 1)) | (1ull << 52));
  const int sh = ex - 1075 - E;  // value = mant * 2^(ex-1075)
  int64_t q;
  if (sh >= 0)
    q = (sh < 11) ? (mant << sh) : 0x7fffffffffffffffll;  // caller keeps |x| * 2^-E < 2^62
  else
    q = shr_round(mant, -sh);
  return (b >> 63) ? -q : q;
}

// q * 2^E -> double with round-to-nearest, integer operations only.
__device__ __forceinline__ double fx_to_f64(int64_t q, int E) {
  if (q == 0) return 0.0;
  const uint64_t sign = q < 0 ? (1ull << 63) : 0;
  uint64_t m = q < 0 ? (uint64_t)(-q) : (uint64_t)q;
  const int lz = __clzll((long long)m);
  const int top = 63 - lz;  // index of the leading bit
  int ex = top + E;         // value = m * 2^E, leading bit at 2^(top+E)
  uint64_t frac;
  if (top > 52) {
    const int s = top - 52;
    uint64_t r = m >> s;
    const uint64_t rem = m & ((1ull << s) - 1);
    const uint64_t half = 1ull << (s - 1);
    if (rem > half || (rem == half && (r & 1))) {
      r += 1;
      if (r >> 53) {
        r >>= 1;
        ex += 1;
      }
    }
    frac = r;
  } else {
    frac = m << (52 - top);
  }
  const int bexp = ex + 1023;
  if (bexp <= 0) return 0.0;  // below the normal range: flush (never reached in practice)
  const uint64_t bits = sign | ((uint64_t)bexp << 52) | (frac & ((1ull << 52) - 1));
  return __longlong_as_double((long long)bits);
}

}  // namespace qcmg
