// matrixDataTypes.h -- TE::matrix, TE::vector and TE::smatrix of the GB300
// TimeEvolver: the public layout of core/matrixDataTypes.h:13-99 (COO storage
// with size_t indices, public fields), with the sparse product and the
// library preparation (initialize) done on the GPU through the C ABI of
// tegpu.h instead of MKL / Armadillo / OpenBLAS.
#pragma once

#include <complex>
#include <cstdlib>
#include <iostream>
#include <string>
#include <vector>

#include "tegpu.h"

namespace TE {

/** Dense matrix, col-major (core/matrixDataTypes.h:18-27). */
class matrix {
 public:
  size_t n, m;
  std::complex<double>* values;
  size_t numValues;
  matrix(size_t nn, size_t mm);
  matrix(size_t nn, size_t mm, std::complex<double>* vals);
  ~matrix();
};

/** Dense vector (core/matrixDataTypes.h:33-53). */
class vector {
 public:
  std::complex<double>* values;
  size_t length;
  vector(unsigned int n) {
    if (n == 0) {
      std::cerr << "Empty vectors are not supported." << std::endl;
      exit(1);
    }
    length = n;
    values = new std::complex<double>[length];
  }
  ~vector() { delete[] values; }
  operator std::complex<double>*() const { return NULL; }
};

/** Sparse matrix in COO storage (core/matrixDataTypes.h:59-99).  initialize()
 * uploads it to the GPU (CSR / SELL-32 with int32 indices); spMV runs there. */
class smatrix {
 public:
  std::complex<double>* values;
  size_t* columns;
  size_t* rowIndex;
  size_t numValues;
  size_t n, m;
  bool sym, hermitian;
  bool upperTri;
  bool initialized;

  double norm1();
  double normInf();

  smatrix();
  smatrix(std::complex<double>* val, size_t* col, size_t* row, size_t nbV, unsigned int nn, unsigned int mm);
  smatrix(const smatrix& old_obj);
  ~smatrix();

  int spMV(std::complex<double> alpha, std::complex<double>* in, std::complex<double>* out);
  int initialize();

  /** Device handle (uploads on first use); nullptr if the upload failed. */
  te_matrix device();

  static constexpr std::complex<double> one = std::complex<double>(1.0, 0.0);
  static constexpr std::complex<double> zero = std::complex<double>(0.0, 0.0);

 private:
  te_matrix dev_ = nullptr;
};

}  // namespace TE

/** Element-wise exp (core/matrixDataTypes.h:108-117). */
inline void expV(size_t len, std::complex<double>* x, std::complex<double>* y) {
  for (size_t i = 0; i < len; i++) y[i] = std::exp(x[i]);
}

/** Element-wise product (core/matrixDataTypes.h:122-130). */
inline void mulV(size_t len, std::complex<double>* a, std::complex<double>* b, std::complex<double>* y) {
  for (size_t i = 0; i < len; i++) y[i] = b[i] * a[i];
}
