// krylovObservables.h -- observables of the GB300 TimeEvolver (same API as
// core/krylovObservables.h:16-116).  During timeEvolve, sparse-matrix and
// vector observables are evaluated on the GPU (diagonal ones fused into the
// sampling pass); any other subclass of krylovBasicObservable is called on
// the host with the sampled state, exactly through its virtual expectation().
#pragma once

#include <complex>
#include <fstream>
#include <iostream>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "matrixDataTypes.h"

/** Raised by an observable to stop the evolution at the current sample. */
class requestStopException : public std::exception {
 public:
  virtual const char* what() const throw();
  requestStopException() = default;
};

using namespace TE;

enum obsType { VOID_TYPE_OBS, VECTOR_TYPE_OBS, SPARSE_MATRIX_TYPE_OBS, MATRIX_TYPE_OBS };

class krylovTimeEvolver;

class krylovBasicObservable {
 public:
  krylovBasicObservable(const std::string& name)
      : obs_name(name), dim(0), numSamples(0), sampleIndex(0), type(VOID_TYPE_OBS), expectationValues(nullptr) {}
  krylovBasicObservable(const std::string& name, std::vector<double> values);
  virtual ~krylovBasicObservable();
  virtual std::complex<double> expectation(std::complex<double>* vec, int len) = 0;
  obsType retType();
  std::string retName();
  double* retExpectationValues();
  size_t retNumSamples();
  virtual void initializeResultArray(size_t size);
  size_t resetResultArray();

  static constexpr std::complex<double> one = std::complex<double>(1.0, 0.0);
  static constexpr std::complex<double> zero = std::complex<double>(0.0, 0.0);

 protected:
  friend class krylovTimeEvolver;
  std::string obs_name;
  size_t dim;
  size_t numSamples;
  size_t sampleIndex;
  obsType type;
  double* expectationValues;
};

class krylovOutputObservable : public krylovBasicObservable {
 public:
  krylovOutputObservable(const std::string& name, std::vector<double> values);
  std::complex<double> expectation(std::complex<double>* vec, int len);
};

/** |<obs|state>|^2 (core/krylovObservables.cpp:216-236). */
class krylovVectorObservable : public krylovBasicObservable {
 public:
  krylovVectorObservable(const std::string& name, std::complex<double>* obs, size_t len);
  ~krylovVectorObservable() {}
  std::complex<double> expectation(std::complex<double>* vec, int len);
  const std::complex<double>* data() const { return obs.get(); }

 private:
  std::unique_ptr<std::complex<double>[]> obs;
};

/** Re <state|O|state> for a sparse O (core/krylovObservables.cpp:173-194). */
class krylovSpMatrixObservable : public krylovBasicObservable {
 public:
  krylovSpMatrixObservable(const std::string& name, std::unique_ptr<smatrix> obs);
  ~krylovSpMatrixObservable();
  std::complex<double> expectation(std::complex<double>* vec, int len);
  smatrix* matrixPtr() { return obs.get(); }

 private:
  std::unique_ptr<smatrix> obs;
  std::complex<double>* tmpBlasVec;
};

/** Re <state|O|state> for a dense O (core/krylovObservables.cpp:119-138); the
 * reference declares its constructor private, so it cannot be built there. */
class krylovMatrixObservable : public krylovBasicObservable {
  krylovMatrixObservable(const std::string& name, std::unique_ptr<matrix> obs);
  ~krylovMatrixObservable();
  std::complex<double> expectation(std::complex<double>* vec, int len);

 private:
  std::unique_ptr<matrix> obs;
  std::complex<double>* tmpBlasVec;
};
