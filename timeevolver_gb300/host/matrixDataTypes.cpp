// matrixDataTypes.cpp -- TE::matrix / TE::smatrix over the GPU library
// (reference behaviour: core/matrixDataTypes.cpp).
#include "matrixDataTypes.h"

#include <algorithm>
#include <cstring>

using namespace TE;

matrix::matrix(size_t nn, size_t mm) {
  n = nn;
  m = mm;
  numValues = n * m;
  values = (nn * mm > 0) ? new std::complex<double>[n * m]() : nullptr;
}

matrix::matrix(size_t nn, size_t mm, std::complex<double>* vals) : n(nn), m(mm) {
  numValues = n * m;
  values = new std::complex<double>[numValues];
  std::copy(vals, vals + numValues, values);
}

matrix::~matrix() {
  if (n * m > 0) delete[] values;
}

smatrix::smatrix() {
  sym = hermitian = upperTri = initialized = false;
  rowIndex = columns = nullptr;
  values = nullptr;
  m = n = 0;
  numValues = 0;
}

smatrix::smatrix(std::complex<double>* val, size_t* col, size_t* row, size_t nbV, unsigned int nn, unsigned int mm) {
  if (nn == 0 || mm == 0) {
    std::cerr << "Empty matrices are not supported." << std::endl;
    exit(1);
  }
  numValues = nbV;
  n = nn;
  m = mm;
  sym = hermitian = upperTri = false;
  columns = new size_t[nbV];
  rowIndex = new size_t[nbV];
  values = new std::complex<double>[nbV];
  initialized = false;
  std::copy(val, val + nbV, values);
  std::copy(col, col + nbV, columns);
  std::copy(row, row + nbV, rowIndex);
}

smatrix::smatrix(const smatrix& old_obj) {
  numValues = old_obj.numValues;
  n = old_obj.n;
  m = old_obj.m;
  sym = old_obj.sym;
  hermitian = old_obj.hermitian;
  upperTri = old_obj.upperTri;
  columns = new size_t[numValues];
  rowIndex = new size_t[numValues];
  values = new std::complex<double>[numValues];
  initialized = false;
  std::copy(old_obj.values, old_obj.values + numValues, values);
  std::copy(old_obj.columns, old_obj.columns + numValues, columns);
  std::copy(old_obj.rowIndex, old_obj.rowIndex + numValues, rowIndex);
}

smatrix::~smatrix() {
  if (dev_) te_matrix_destroy(dev_);
  if (n > 1 || m > 1) {
    delete[] rowIndex;
    delete[] values;
    delete[] columns;
  }
}

// maximum absolute column sum (core/matrixDataTypes.cpp:67-79)
double smatrix::norm1() {
  std::vector<double> colVal(n, 0.0);
  for (size_t i = 0; i != numValues; i++) colVal[columns[i]] += std::abs(values[i]);
  return colVal.empty() ? 0.0 : *std::max_element(colVal.begin(), colVal.end());
}

// maximum absolute row sum (core/matrixDataTypes.cpp:85-97)
double smatrix::normInf() {
  std::vector<double> rowVal(m, 0.0);
  for (size_t i = 0; i != numValues; i++) rowVal[rowIndex[i]] += std::abs(values[i]);
  return rowVal.empty() ? 0.0 : *std::max_element(rowVal.begin(), rowVal.end());
}

te_matrix smatrix::device() {
  if (!dev_) {
    int rc = te_matrix_create_coo((int64_t)m, (int64_t)n, (int64_t)numValues,
                                  reinterpret_cast<const uint64_t*>(rowIndex),
                                  reinterpret_cast<const uint64_t*>(columns),
                                  reinterpret_cast<const double*>(values), &dev_);
    if (rc != TE_OK) {
      std::cerr << "GPU sparse matrix upload failed: " << te_last_error() << std::endl;
      dev_ = nullptr;
    }
  }
  return dev_;
}

// out = alpha * this * in on the GPU (core/matrixDataTypes.cpp:169-190)
int smatrix::spMV(std::complex<double> alpha, std::complex<double>* in, std::complex<double>* out) {
  te_matrix A = device();
  if (!A) return -1;
  return te_matrix_spmv_host(A, alpha.real(), alpha.imag(), reinterpret_cast<const double*>(in),
                             reinterpret_cast<double*>(out));
}

// GPU preparation (core/matrixDataTypes.cpp:196-240): returns -1 when already
// initialised, 0 on success.
int smatrix::initialize() {
  if (initialized) return -1;
  if (!device()) return 1;
  initialized = true;
  return 0;
}
