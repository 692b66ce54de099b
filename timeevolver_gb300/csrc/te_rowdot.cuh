// te_rowdot.cuh -- one CSR row times a complex vector, exactly 2 (real values)
// or 4 (complex values) FP64 FMAs per non-zero.
#pragma once
#include "te_internal.cuh"

template <bool REAL>
__device__ __forceinline__ double2 te_row_dot(const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
                                              const double* __restrict__ val, const double2* __restrict__ x,
                                              int32_t r) {
  const int32_t b = __ldg(row_ptr + r), e = __ldg(row_ptr + r + 1);
  double re = 0.0, im = 0.0;
  int32_t p = b;
  if (REAL) {
    for (; p + 4 <= e; p += 4) {
      int32_t c0 = __ldg(col + p), c1 = __ldg(col + p + 1), c2 = __ldg(col + p + 2), c3 = __ldg(col + p + 3);
      double a0 = __ldg(val + p), a1 = __ldg(val + p + 1), a2 = __ldg(val + p + 2), a3 = __ldg(val + p + 3);
      double2 x0 = __ldg(x + c0), x1 = __ldg(x + c1), x2 = __ldg(x + c2), x3 = __ldg(x + c3);
      re = fma(a0, x0.x, re);
      im = fma(a0, x0.y, im);
      re = fma(a1, x1.x, re);
      im = fma(a1, x1.y, im);
      re = fma(a2, x2.x, re);
      im = fma(a2, x2.y, im);
      re = fma(a3, x3.x, re);
      im = fma(a3, x3.y, im);
    }
    for (; p < e; ++p) {
      double a = __ldg(val + p);
      double2 xv = __ldg(x + __ldg(col + p));
      re = fma(a, xv.x, re);
      im = fma(a, xv.y, im);
    }
  } else {
    const double2* __restrict__ v2 = reinterpret_cast<const double2*>(val);
    for (; p + 2 <= e; p += 2) {
      int32_t c0 = __ldg(col + p), c1 = __ldg(col + p + 1);
      double2 a0 = __ldg(v2 + p), a1 = __ldg(v2 + p + 1);
      double2 x0 = __ldg(x + c0), x1 = __ldg(x + c1);
      re = fma(a0.x, x0.x, re);
      re = fma(-a0.y, x0.y, re);
      im = fma(a0.x, x0.y, im);
      im = fma(a0.y, x0.x, im);
      re = fma(a1.x, x1.x, re);
      re = fma(-a1.y, x1.y, re);
      im = fma(a1.x, x1.y, im);
      im = fma(a1.y, x1.x, im);
    }
    for (; p < e; ++p) {
      double2 a = __ldg(v2 + p);
      double2 xv = __ldg(x + __ldg(col + p));
      re = fma(a.x, xv.x, re);
      re = fma(-a.y, xv.y, re);
      im = fma(a.x, xv.y, im);
      im = fma(a.y, xv.x, im);
    }
  }
  return make_double2(re, im);
}
