// te_fixed.cuh -- fixed-point SpMV for real matrices on the integer pipes.
//
// GB300 issues FP64 at 1/58 of its FP32 rate, so a complex-vector SpMV with
// two DFMAs per stored entry is bound by FP64 issue long before HBM.  This
// path multiplies in integers instead:
//
//  * H (real, SELL slots): h~ = round(h 2^sh), sh chosen so that the largest
//    row 1-norm R maps below 2^61; stored as two int32 limbs {h0, h1},
//    h~ = h1 2^31 + h0 with 0 <= h0 < 2^31 (8 bytes per slot, as the double).
//  * the Krylov vector u_j: X = round(u 2^xs) per component, xs chosen from a
//    rigorous bound U on max|u| so that |X| < 2^61; stored as int4
//    {re0, re1, im0, im1} with the same limb split (16 bytes per row).
//  * a row sum is accumulated in one int64 per component from int32 limb
//    products (te_sell_row_fix) and rounded to the nearest double once.
//
// Error of a row of k slots: below (1.25 k 2^-56 + (k + 1) 2^-61) R U +
// 2^-53 |y|, an absolute bound at the scale R U; an FP64 SpMV's bound is
// k 2^-53 sum|h||u| <= k 2^-53 R U, so normwise the fixed-point product is the
// more accurate one, while rows whose sum|h||u| lies far below R U get the
// absolute bound instead of a relative one.  Everything else (the recurrence,
// the reductions, the Krylov-space arithmetic) stays FP64.
#pragma once
#include <cstdint>

#include "te_internal.cuh"

// Fixed-point value with |v 2^xs| < 2^61 (caller's bound), rounded half away
// from zero; zeros and subnormals give 0.  Integer instructions only.
__device__ __forceinline__ int64_t te_fix_encode(double v, int xs) {
  const uint64_t b = (uint64_t)__double_as_longlong(v);
  const int e = (int)((b >> 52) & 0x7ff);
  if (e == 0) return 0;
  const uint64_t m = (b & 0xfffffffffffffull) | (1ull << 52);
  const int sft = e - 1075 + xs;  // |v| 2^xs = m 2^sft
  uint64_t mag;
  if (sft >= 0) {
    mag = m << min(sft, 8);  // the bound keeps sft <= 8
  } else if (sft > -64) {
    const int r = -sft;
    mag = (m >> r) + ((m >> (r - 1)) & 1ull);
  } else {
    mag = 0;
  }
  return (b >> 63) ? -(int64_t)mag : (int64_t)mag;
}

// x 2^k rounded to the nearest integer (half away from zero) as a signed
// 128-bit two's complement {lo, hi}; zeros and subnormals give 0.  The caller
// keeps |x| 2^k below 2^126.  Integer instructions only.
__device__ __forceinline__ void te_fix_encode128(double x, int k, unsigned long long& lo, unsigned long long& hi) {
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7ff);
  lo = hi = 0ull;
  if (e == 0) return;
  const uint64_t m = (b & 0xfffffffffffffull) | (1ull << 52);
  const int sft = e - 1075 + k;  // |x| 2^k = m 2^sft
  if (sft >= 64) {
    hi = m << min(sft - 64, 63);
  } else if (sft > 0) {
    lo = m << sft;
    hi = m >> (64 - sft);
  } else if (sft == 0) {
    lo = m;
  } else if (sft > -64) {
    const int r = -sft;
    lo = (m >> r) + ((m >> (r - 1)) & 1ull);
  }
  if (b >> 63) {  // negate
    lo = ~lo + 1ull;
    hi = ~hi + (lo == 0ull ? 1ull : 0ull);
  }
}

// Signed 128-bit {lo, hi} times 2^e2, rounded to the nearest double.
__device__ __forceinline__ double te_i128_to_double(unsigned long long lo, unsigned long long hi, int e2);

// Limb split v = v1 2^31 + v0, 0 <= v0 < 2^31 (|v| < 2^61 keeps |v1| < 2^30).
__device__ __forceinline__ int2 te_fix_split(int64_t v) {
  return make_int2((int)(v & 0x7fffffffll), (int)(v >> 31));
}

// v 2^e2 rounded to the nearest double (ties to even), integers only.
// Results below the normal range flush to zero.
__device__ __forceinline__ double te_i64_to_double(int64_t v, int e2) {
  if (v == 0) return 0.0;
  const uint64_t sign = (uint64_t)v & 0x8000000000000000ull;
  const uint64_t a = sign ? 0ull - (uint64_t)v : (uint64_t)v;
  const int lz = __clzll((long long)a);
  const uint64_t top = a << lz;  // leading one at bit 63
  uint64_t mant = top >> 11;
  const uint64_t rb = top & 0x7ffull;
  mant += (rb > 0x400ull || (rb == 0x400ull && (mant & 1ull))) ? 1ull : 0ull;
  int ex = 63 - lz + e2;
  if (mant >> 53) {
    mant >>= 1;
    ++ex;
  }
  if (ex < -1022) return 0.0;
  return __longlong_as_double((long long)(sign | ((uint64_t)(ex + 1023) << 52) | (mant & 0xfffffffffffffull)));
}

// (hi:lo) 2^e2 for an unsigned 128-bit value, rounded to the nearest double
// (ties to even), integers only; results below the normal range flush to zero.
__device__ __forceinline__ double te_u128_to_double(unsigned long long hi, unsigned long long lo, int e2) {
  if ((hi | lo) == 0ull) return 0.0;
  const int lz = hi ? __clzll((long long)hi) : 64 + __clzll((long long)lo);
  uint64_t top, rest;
  if (lz >= 64) {
    top = lo << (lz - 64);
    rest = 0;
  } else if (lz == 0) {
    top = hi;
    rest = lo;
  } else {
    top = (hi << lz) | (lo >> (64 - lz));
    rest = lo << lz;
  }
  uint64_t mant = top >> 11;
  const uint64_t rb = top & 0x7ffull;
  mant += (rb > 0x400ull || (rb == 0x400ull && (rest != 0ull || (mant & 1ull)))) ? 1ull : 0ull;
  int ex = 127 - lz + e2;
  if (mant >> 53) {
    mant >>= 1;
    ++ex;
  }
  if (ex < -1022) return 0.0;
  return __longlong_as_double((long long)(((uint64_t)(ex + 1023) << 52) | (mant & 0xfffffffffffffull)));
}

__device__ __forceinline__ double te_i128_to_double(unsigned long long lo, unsigned long long hi, int e2) {
  if (hi >> 63) {
    const unsigned long long nlo = ~lo + 1ull, nhi = ~hi + (nlo == 0ull ? 1ull : 0ull);
    return -te_u128_to_double(nhi, nlo, e2);
  }
  return te_u128_to_double(hi, lo, e2);
}

// {lo, hi} added to the 128-bit integer at p (two atomics, the carry of the
// low word into the high word; any order of additions gives the same total).
__device__ __forceinline__ void te_atomic_add128(unsigned long long* p, unsigned long long lo, unsigned long long hi) {
  const unsigned long long old = atomicAdd(p, lo);
  atomicAdd(p + 1, hi + (old + lo < old ? 1ull : 0ull));
}

// v^2 / 2^62 for |v| < 2^61 from 31-bit limbs of |v| (a1^2 + 4 hi32(a1 a0),
// the a0^2 term dropped): below the exact value by less than 5.
__device__ __forceinline__ unsigned long long te_fix_sq(int64_t v) {
  const uint64_t a = v < 0 ? 0ull - (uint64_t)v : (uint64_t)v;
  const unsigned int a1 = (unsigned int)(a >> 31), a0 = (unsigned int)(a & 0x7fffffffull);
  return (unsigned long long)a1 * a1 + 4ull * __umulhi(a1, a0);
}

// Upper bound of |v| from the high word of its bit pattern (sign cleared):
// the double whose high word is one larger.
__device__ __forceinline__ unsigned int te_fix_hiword(double v) {
  return (unsigned int)__double2hiint(v) & 0x7fffffffu;
}
__device__ __forceinline__ double te_fix_upper(unsigned int hiword) {
  return hiword ? __hiloint2double((int)(hiword + 1u), 0) : 0.0;
}

// Scale exponent for a vector bounded by B: |v| 2^xs <= B 2^xs < 2^61.
__device__ __forceinline__ int te_fix_scale(double bound) {
  if (!(bound > 0.0) || !(bound < 1e300)) return 0;
  int E;
  frexp(bound, &E);  // bound < 2^E
  return 61 - E;
}

#ifndef TE_FIX_UNROLL
#define TE_FIX_UNROLL 2
#endif
constexpr int kTeFixUnroll = TE_FIX_UNROLL;  // slots per lane in flight
// Slots per lane in flight in the column-block passes: 3 measured 2.437 ms
// per apply of the dim-1e7 Zipf matrix against 2.478 (2) and 2.451 (4), all
// at 6 blocks of 256 per SM without spills.
constexpr int kTeFixBlockUnroll = 3;

// hi-part product of two limb-split values c = c1 2^31 + c0, x = x1 2^31 + x0
// in units of 2^62: c1 x1 + 2 (hi32(c1 x0) + hi32(c0 x1)), below c x / 2^62 by
// less than 5.
__device__ __forceinline__ int64_t te_fix_prod(int c0, int c1, int x0, int x1) {
  int t;
  asm("mul.hi.s32 %0, %1, %2;" : "=r"(t) : "r"(c1), "r"(x0));
  asm("mad.hi.s32 %0, %1, %2, %0;" : "+r"(t) : "r"(c0), "r"(x1));
  return (int64_t)c1 * x1 + 2 * (int64_t)t;
}

// One slot: S += h~ X (see te_sell_row_fix).
__device__ __forceinline__ void te_fix_mac(const int2 h, const int4 x, int64_t& sr, int64_t& si) {
  int tr, ti;
  asm("mul.hi.s32 %0, %1, %2;" : "=r"(tr) : "r"(h.y), "r"(x.x));
  asm("mad.hi.s32 %0, %1, %2, %0;" : "+r"(tr) : "r"(h.x), "r"(x.y));
  asm("mul.hi.s32 %0, %1, %2;" : "=r"(ti) : "r"(h.y), "r"(x.z));
  asm("mad.hi.s32 %0, %1, %2, %0;" : "+r"(ti) : "r"(h.x), "r"(x.w));
  sr += (int64_t)h.y * x.y + 2 * (int64_t)tr;
  si += (int64_t)h.y * x.w + 2 * (int64_t)ti;
}

// One lane's row of a real SELL-32 matrix times the fixed-point vector X: the
// lane's slots s, s + 32, ... below e of its chunk; returns the row sum as a
// double, given the total scale shift = sh + xs (y = sum h~ X 2^-shift).
//
// Per slot and component, with h~ = h1 2^31 + h0 and X = x1 2^31 + x0:
//   S += h1 x1 + 2 (hi32(h1 x0) + hi32(h0 x1))      (y = S 2^(62 - shift))
// i.e. the cross products are taken at their high 32 bits (floored) and h0 x0
// is left out: at most 5 units of 2^62 per slot of a total below 2^122, so
// the row error is below k 1.25 2^-56 R U + (k + 1) 2^-61 R U + 2^-53 |y|
// for k slots, R the largest row 1-norm and U the bound on max|u|.
template <int U = kTeFixUnroll>
__device__ __forceinline__ longlong2 te_sell_row_fix_sum(int64_t s, int64_t e, const int32_t* __restrict__ col,
                                                         const int2* __restrict__ hv, const int4* __restrict__ X) {
  int64_t sr = 0, si = 0;
#pragma unroll(U)
  for (; s < e; s += 32) te_fix_mac(__ldcs(hv + s), __ldg(X + __ldcs(col + s)), sr, si);  // {h0, h1}, {re0, re1, im0, im1}
  return make_longlong2(sr, si);
}
__device__ __forceinline__ double2 te_fix_to_double(longlong2 S, int shift) {
  return make_double2(te_i64_to_double(S.x, 62 - shift), te_i64_to_double(S.y, 62 - shift));
}
__device__ __forceinline__ double2 te_sell_row_fix(int64_t s, int64_t e, const int32_t* __restrict__ col,
                                                   const int2* __restrict__ hv, const int4* __restrict__ X,
                                                   int shift) {
  return te_fix_to_double(te_sell_row_fix_sum(s, e, col, hv, X), shift);
}

// te_sell_row_fix over packed slots: word = column | (value index << cbits),
// the values' limbs in tab (shared memory).
__device__ __forceinline__ double2 te_sell_row_fix_packed(int64_t s, int64_t e, const uint32_t* __restrict__ pk,
                                                          const int2* tab, int cbits, const int4* __restrict__ X,
                                                          int shift) {
  const uint32_t cmask = (1u << cbits) - 1u;
  int64_t sr = 0, si = 0;
#pragma unroll(kTeFixUnroll)
  for (; s < e; s += 32) {
    const uint32_t wd = __ldcs(pk + s);
    te_fix_mac(tab[wd >> cbits], __ldg(X + (wd & cmask)), sr, si);
  }
  return make_double2(te_i64_to_double(sr, 62 - shift), te_i64_to_double(si, 62 - shift));
}

// Complex H: slot value {Re h~ limbs, Im h~ limbs} as int4; R is then the
// largest row sum of |Re h| + |Im h|.  Four limb products per slot
// (Re = hr xr - hi xi, Im = hr xi + hi xr), so the per-slot term of the
// error bound is four times the real one: below (5 k 2^-56 + (2 k + 1) 2^-61)
// R U + 2^-53 |y|.
template <int U = kTeFixUnroll>
__device__ __forceinline__ longlong2 te_sell_row_fix_c_sum(int64_t s, int64_t e, const int32_t* __restrict__ col,
                                                           const int4* __restrict__ hv, const int4* __restrict__ X) {
  int64_t sr = 0, si = 0;
#pragma unroll(U)
  for (; s < e; s += 32) {
    const int4 h = __ldcs(hv + s);
    const int4 x = __ldg(X + __ldcs(col + s));
    sr += te_fix_prod(h.x, h.y, x.x, x.y) - te_fix_prod(h.z, h.w, x.z, x.w);
    si += te_fix_prod(h.x, h.y, x.z, x.w) + te_fix_prod(h.z, h.w, x.x, x.y);
  }
  return make_longlong2(sr, si);
}
__device__ __forceinline__ double2 te_sell_row_fix_c(int64_t s, int64_t e, const int32_t* __restrict__ col,
                                                     const int4* __restrict__ hv, const int4* __restrict__ X,
                                                     int shift) {
  return te_fix_to_double(te_sell_row_fix_c_sum(s, e, col, hv, X), shift);
}
