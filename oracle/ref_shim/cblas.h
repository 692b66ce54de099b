/*
 * cblas.h stand-in for compiling the reference's core/*.cpp as the oracle's
 * second opinion (TEST INFRASTRUCTURE ONLY).
 *
 * Maps the CBLAS calls the reference makes (core/krylovTimeEvolver.cpp,
 * core/krylovObservables.cpp, core/matrixDataTypes.cpp) onto the ILP64
 * OpenBLAS that numpy ships, by its exported names (scipy_cblas_*64_).  The
 * enum values are the standard CBLAS ones.
 */
#pragma once

#include <cstdint>

typedef int64_t te_blasint;

enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };

extern "C" {
void scipy_cblas_zgemv64_(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE trans, te_blasint m, te_blasint n,
                          const void* alpha, const void* a, te_blasint lda, const void* x, te_blasint incx,
                          const void* beta, void* y, te_blasint incy);
void scipy_cblas_zdotc_sub64_(te_blasint n, const void* x, te_blasint incx, const void* y, te_blasint incy, void* ret);
void scipy_cblas_zcopy64_(te_blasint n, const void* x, te_blasint incx, void* y, te_blasint incy);
void scipy_cblas_zaxpy64_(te_blasint n, const void* alpha, const void* x, te_blasint incx, void* y, te_blasint incy);
void scipy_cblas_zscal64_(te_blasint n, const void* alpha, void* x, te_blasint incx);
void scipy_cblas_zdscal64_(te_blasint n, double alpha, void* x, te_blasint incx);
double scipy_cblas_dznrm264_(te_blasint n, const void* x, te_blasint incx);
}

#define cblas_zgemv scipy_cblas_zgemv64_
#define cblas_zdotc_sub scipy_cblas_zdotc_sub64_
#define cblas_zcopy scipy_cblas_zcopy64_
#define cblas_zaxpy scipy_cblas_zaxpy64_
#define cblas_zscal scipy_cblas_zscal64_
#define cblas_zdscal scipy_cblas_zdscal64_
#define cblas_dznrm2 scipy_cblas_dznrm264_
