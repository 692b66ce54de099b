// te_sell.cuh -- one SELL-32 row (one lane of a warp) times a complex vector.
//
// All 32 lanes of a warp work on the 32 rows of one chunk; rows were sorted by
// length so the chunk's trip count (its longest row) wastes almost no FP64
// issue slots on padding, and slot s + 32k is contiguous across lanes, so
// values and column indices are read fully coalesced with streaming (evict
// first) loads that keep the L2 for the Krylov vectors.
#pragma once
#include "te_internal.cuh"

// Loads of x (XCG): 0 through the read-only (non-coherent) cache; 1 ordinary
// cached loads (ld.global.ca) for x written earlier in the same kernel by
// other SMs and read after a grid barrier, with no copy of it in this SM's L1
// from before the write (the persistent Lanczos kernel: each basis vector is
// written once per launch, then read); 2 L2-only loads (ld.global.cg) for
// vectors rewritten again and again within one launch (the persistent batched
// kernel), where this SM's L1 could still hold an earlier copy.
template <int XCG>
__device__ __forceinline__ double2 te_load_x(const double2* __restrict__ x, int32_t c) {
  return XCG == 2 ? __ldcg(x + c) : (XCG == 1 ? __ldca(x + c) : __ldg(x + c));
}

template <bool REAL, int XCG = 0>
__device__ __forceinline__ double2 te_sell_row(const int64_t* __restrict__ chunk_off,
                                               const int32_t* __restrict__ col, const double* __restrict__ val,
                                               const double2* __restrict__ x, int64_t chunk, int lane) {
  const int64_t e = __ldg(chunk_off + chunk + 1);
  int64_t s = __ldg(chunk_off + chunk) + lane;
  double re = 0.0, im = 0.0;
  if (REAL) {
    for (; s + 96 < e; s += 128) {
      int32_t c0 = __ldcs(col + s), c1 = __ldcs(col + s + 32), c2 = __ldcs(col + s + 64), c3 = __ldcs(col + s + 96);
      double a0 = __ldcs(val + s), a1 = __ldcs(val + s + 32), a2 = __ldcs(val + s + 64), a3 = __ldcs(val + s + 96);
      double2 x0 = te_load_x<XCG>(x, c0), x1 = te_load_x<XCG>(x, c1), x2 = te_load_x<XCG>(x, c2),
              x3 = te_load_x<XCG>(x, c3);
      re = fma(a0, x0.x, re);
      im = fma(a0, x0.y, im);
      re = fma(a1, x1.x, re);
      im = fma(a1, x1.y, im);
      re = fma(a2, x2.x, re);
      im = fma(a2, x2.y, im);
      re = fma(a3, x3.x, re);
      im = fma(a3, x3.y, im);
    }
    for (; s < e; s += 32) {
      double a = __ldcs(val + s);
      double2 xv = te_load_x<XCG>(x, __ldcs(col + s));
      re = fma(a, xv.x, re);
      im = fma(a, xv.y, im);
    }
  } else {
    const double2* __restrict__ v2 = reinterpret_cast<const double2*>(val);
    for (; s + 32 < e; s += 64) {
      int32_t c0 = __ldcs(col + s), c1 = __ldcs(col + s + 32);
      double2 a0 = __ldcs(v2 + s), a1 = __ldcs(v2 + s + 32);
      double2 x0 = te_load_x<XCG>(x, c0), x1 = te_load_x<XCG>(x, c1);
      re = fma(a0.x, x0.x, re);
      re = fma(-a0.y, x0.y, re);
      im = fma(a0.x, x0.y, im);
      im = fma(a0.y, x0.x, im);
      re = fma(a1.x, x1.x, re);
      re = fma(-a1.y, x1.y, re);
      im = fma(a1.x, x1.y, im);
      im = fma(a1.y, x1.x, im);
    }
    for (; s < e; s += 32) {
      double2 a = __ldcs(v2 + s);
      double2 xv = te_load_x<XCG>(x, __ldcs(col + s));
      re = fma(a.x, xv.x, re);
      re = fma(-a.y, xv.y, re);
      im = fma(a.x, xv.y, im);
      im = fma(a.y, xv.x, im);
    }
  }
  return make_double2(re, im);
}

// K lanes per row (K = 2 or 4), for matrices too small to fill the GPU with
// one lane per row: a warp owns the part-th group of 32/K rows of a chunk;
// lane l works on row part * (32/K) + l/K and takes that row's entries
// k = l%K, l%K + K, ...; the K partial sums are combined by xor shuffles, so
// every lane of the row ends with the same value.  The entries are summed in
// a different order than te_sell_row (interleaved by K): results differ from
// the K = 1 kernel by rounding only.
template <bool REAL, int K>
__device__ __forceinline__ double2 te_sell_row_k(const int64_t* __restrict__ chunk_off,
                                                 const int32_t* __restrict__ col, const double* __restrict__ val,
                                                 const double2* __restrict__ x, int64_t chunk, int part, int lane) {
  const int64_t off = __ldg(chunk_off + chunk);
  const int64_t len = (__ldg(chunk_off + chunk + 1) - off) >> 5;
  const int rloc = part * (32 / K) + lane / K;
  double re = 0.0, im = 0.0;
  int64_t k = lane % K;
  if (REAL) {
    for (; k + K < len; k += 2 * K) {
      const int64_t s0 = off + 32 * k + rloc, s1 = s0 + 32 * K;
      const int32_t c0 = __ldcs(col + s0), c1 = __ldcs(col + s1);
      const double a0 = __ldcs(val + s0), a1 = __ldcs(val + s1);
      const double2 x0 = __ldg(x + c0), x1 = __ldg(x + c1);
      re = fma(a0, x0.x, re);
      im = fma(a0, x0.y, im);
      re = fma(a1, x1.x, re);
      im = fma(a1, x1.y, im);
    }
    for (; k < len; k += K) {
      const int64_t s = off + 32 * k + rloc;
      const double a = __ldcs(val + s);
      const double2 xv = __ldg(x + __ldcs(col + s));
      re = fma(a, xv.x, re);
      im = fma(a, xv.y, im);
    }
  } else {
    const double2* __restrict__ v2 = reinterpret_cast<const double2*>(val);
    for (; k < len; k += K) {
      const int64_t s = off + 32 * k + rloc;
      const double2 a = __ldcs(v2 + s);
      const double2 xv = __ldg(x + __ldcs(col + s));
      re = fma(a.x, xv.x, re);
      re = fma(-a.y, xv.y, re);
      im = fma(a.x, xv.y, im);
      im = fma(a.y, xv.x, im);
    }
  }
#pragma unroll
  for (int o = 1; o < K; o <<= 1) {
    re += __shfl_xor_sync(0xffffffffu, re, o);
    im += __shfl_xor_sync(0xffffffffu, im, o);
  }
  return make_double2(re, im);
}

// Entries [b, e) of the long-row CSR times x by a whole warp: lanes stride
// over the entries, then a warp sum (lane 0's value is the one used).
template <bool REAL, int XCG = 0>
__device__ __forceinline__ double2 te_long_range(const TeLongRows& L, int64_t b, int64_t e,
                                                 const double2* __restrict__ x, int lane) {
  double re = 0.0, im = 0.0;
  if (REAL) {
    for (int64_t p = b + lane; p < e; p += 32) {
      const double a = __ldcs(L.val + p);
      const double2 xv = te_load_x<XCG>(x, __ldcs(L.col + p));
      re = fma(a, xv.x, re);
      im = fma(a, xv.y, im);
    }
  } else {
    const double2* __restrict__ v2 = reinterpret_cast<const double2*>(L.val);
    for (int64_t p = b + lane; p < e; p += 32) {
      const double2 a = __ldcs(v2 + p);
      const double2 xv = te_load_x<XCG>(x, __ldcs(L.col + p));
      re = fma(a.x, xv.x, re);
      re = fma(-a.y, xv.y, re);
      im = fma(a.x, xv.y, im);
      im = fma(a.y, xv.x, im);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    re += __shfl_xor_sync(0xffffffffu, re, o);
    im += __shfl_xor_sync(0xffffffffu, im, o);
  }
  return make_double2(re, im);
}

// Merge-path segment s of the long rows by one warp.  Returns non-zero when
// this warp completes its row (then *row and *y hold the row and its sum,
// lane 0's value being the one used): 1 at once for a row of one segment
// (warp-per-row); 2 for a split row, where every warp publishes its segment's
// partial sum and the warp that arrives last adds the row's partials in
// segment order (lane k takes segments k, k + 32, ..., then a fixed shuffle
// tree), so the sum does not depend on which warps ran which segments, and
// resets the row's count.  Which warp completes a split row varies from run
// to run, so a pass that reduces over rows must not fold a split row's terms
// into that warp's sums: te_split_row_publish / te_split_rows_add move them
// to a fixed place in the final reduction.
template <bool REAL, int XCG = 0>
__device__ __forceinline__ int te_long_segment(const TeLongRows& L, int64_t s, const double2* __restrict__ x,
                                               int lane, int64_t* row, double2* y) {
  const int32_t i = __ldg(L.seg_row + s);
  const double2 part = te_long_range<REAL, XCG>(L, __ldg(L.seg_begin + s), __ldg(L.seg_begin + s + 1), x, lane);
  *row = i;
  const int32_t s0 = __ldg(L.row_seg + i), s1 = __ldg(L.row_seg + i + 1);
  if (s1 - s0 == 1) {
    *y = part;
    return 1;
  }
  int last = 0;
  if (lane == 0) {
    __stcg(L.part + s, part);
    __threadfence();
    last = atomicAdd(L.cnt + i, 1u) == (unsigned int)(s1 - s0 - 1) ? 1 : 0;
  }
  last = __shfl_sync(0xffffffffu, last, 0);
  if (!last) return 0;
  __threadfence();
  double re = 0.0, im = 0.0;
  for (int32_t t = s0 + lane; t < s1; t += 32) {
    const double2 p = __ldcg(L.part + t);
    re += p.x;
    im += p.y;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    re += __shfl_xor_sync(0xffffffffu, re, o);
    im += __shfl_xor_sync(0xffffffffu, im, o);
  }
  if (lane == 0) L.cnt[i] = 0u;
  *y = make_double2(re, im);
  return 2;
}

// The reduction terms (v[0], v[1]) of split long row i, stored by the warp
// that completed it (one lane) in the row's first carry slot, whose partial
// sum that warp has consumed; the fence orders the store before the block's
// publication of its own partials.
__device__ __forceinline__ void te_split_row_publish(const TeLongRows& L, int64_t i, const double (&v)[2]) {
  __stcg(L.part + __ldg(L.row_seg + i), make_double2(v[0], v[1]));
  __threadfence();
}

// In the last block of a pass (after every block has published): add the
// split long rows' terms to this thread's values, rows ascending per thread
// (thread t takes rows t, t + blockDim.x, ...), a fixed order.
__device__ __forceinline__ void te_split_rows_add(double (&out)[2], const TeLongRows& L) {
  if (L.n_seg == L.n) return;  // no split rows
  for (int64_t i = threadIdx.x; i < L.n; i += blockDim.x) {
    const int32_t s0 = __ldg(L.row_seg + i), s1 = __ldg(L.row_seg + i + 1);
    if (s1 - s0 > 1) {
      const double2 p = __ldcg(L.part + s0);
      out[0] += p.x;
      out[1] += p.y;
    }
  }
}

