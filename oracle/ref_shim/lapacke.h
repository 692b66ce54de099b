/*
 * lapacke.h stand-in for compiling the reference's core/*.cpp (TEST
 * INFRASTRUCTURE ONLY): LAPACKE_zhseqr, the one LAPACK call of the reference
 * (core/matrixDataTypes.h:135-156), from numpy's ILP64 OpenBLAS by its
 * exported name.  lapack_complex_double is defined by the reference's
 * mathHeader.h before it includes this file.
 */
#pragma once

#include <cstdint>

typedef int64_t lapack_int;
#define LAPACK_COL_MAJOR 102

extern "C" lapack_int scipy_LAPACKE_zhseqr64_(int matrix_layout, char job, char compz, lapack_int n, lapack_int ilo,
                                              lapack_int ihi, lapack_complex_double* h, lapack_int ldh,
                                              lapack_complex_double* w, lapack_complex_double* z, lapack_int ldz);
#define LAPACKE_zhseqr scipy_LAPACKE_zhseqr64_
