// Factorized product kernels of the fixed-point path: arguments, tables and
// the launcher (qcmg_fxprod.cu).
#pragma once

#include <cstdint>

#include "qcmg_internal.h"

namespace qcmg {

struct I128;

struct FxProdArgs {
  uint32_t du, dd;
  int L;
  // up half-operator: row i has positive hops cols[rp[i]..rs[i]) and negative
  // hops cols[rs[i]..rp[i+1]) (used for slabs too small to bulk-copy)
  const uint32_t* rp_up;
  const uint32_t* rs_up;
  const uint32_t* col_up;
  const uint32_t* rp_dn;
  const uint32_t* rs_dn;
  const uint32_t* col_dn;
  const int64_t* dup;  // fixed-point diagonal of each half basis (scale 2^-G)
  const int64_t* ddn;
  const uint32_t* bin_up;
  const uint32_t* bin_dn;
  int64_t U;           // on-site interaction (scale 2^-G)
  const int64_t* wdn;  // dd x L cross table (scale 2^-G), general interactions
  int64_t mt_up, mt_dn;  // hop magnitudes (mantissas)
  int sh_up, sh_dn;      // shifts of the hop terms
  int p2_up, p2_dn;      // log2 |mt| when |mt| is a power of two, else -1
  int sh_d;              // shift of the diagonal term
  int d_tz;              // >= 0: narrow diagonal (see FxTables::dtz), -1: 128-bit products
  const int64_t* yin;    // accumulated input (may alias y) or null
  int64_t m_in;
  int sh_in;
  int p2_in;
  const int64_t* x;
  int64_t* y;
  uint32_t band;  // rows per band (pass D)
  uint32_t nbands;
  // FAST kernels (powers-of-two multipliers, narrow diagonal): the diagonal
  // tables shifted right by d_tz as int32, and each term's shift t with its
  // round term r = 2^(t-1) (rshift_fixed)
  const int32_t* dup32;
  const int32_t* ddn32;
  const int32_t* wdn32;
  int32_t U32;
  int t_up, t_dn, t_d, t_in;
  int64_t r_up, r_dn, r_d, r_in;
  int neg_in;  // the accumulation factor is negative
  // grouped ELL form of the up half-operator (see build_ell4)
  const uint2* ell4;
  const uint16_t* cnt4;
  int* err;  // set to 1 when a bounded wait gives up
  // optional: pass D also accumulates sum_i (y_i dot_x_i >> kDotShift), one
  // 128-bit partial per pass-D block into dot_part (the Lanczos alpha)
  const int64_t* dot_x;
  I128* dot_part;
};

// Builds the grouped ELL form of the up-spin hops from the unit-magnitude
// CSR (positive hops first in each row).  False when the half basis is too
// large for 16-bit columns.
bool build_ell4(const DevBuf<uint32_t>& rp, const DevBuf<uint32_t>& rs, const DevBuf<uint32_t>& col,
                uint32_t dim, cudaStream_t s, DevBuf<uint2>& ell4, DevBuf<uint16_t>& cnt4);

// Slabs staged per table read by pass U: 1 or 2 (0 when the slab is not
// bulk-copied).  QCMG_FX_SLABS=1|2 overrides the choice.
int choose_slabs_per_pass(uint32_t du, int max_optin_smem);

// log2 |m| when |m| is a power of two, else -1 (for FxProdArgs::p2_*).
int pow2_exponent(int64_t m);

// Launches pass U then pass D for y (+)= H x; returns pass D's block count
// (the number of dot partials when A.dot_part is set).
unsigned launch_product(const qcmg_hamiltonian* H, const FxProdArgs& A, cudaStream_t s);

// Upper bound of launch_product's return value on a device with sms SMs.
inline unsigned product_dot_partials(int sms) { return (unsigned)sms * 8u; }

}  // namespace qcmg
