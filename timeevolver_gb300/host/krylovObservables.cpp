// krylovObservables.cpp -- observables (reference: core/krylovObservables.cpp).
// The host-side expectation() bodies are used when a user calls them
// directly; during timeEvolve the GPU evaluates sparse and vector observables.
#include "krylovObservables.h"

std::string krylovBasicObservable::retName() { return obs_name; }
double* krylovBasicObservable::retExpectationValues() { return expectationValues; }
size_t krylovBasicObservable::retNumSamples() { return numSamples; }

void krylovBasicObservable::initializeResultArray(size_t size) {
  numSamples = size;
  expectationValues = new double[size]();
}

size_t krylovBasicObservable::resetResultArray() {
  sampleIndex = 0;
  return numSamples;
}

krylovBasicObservable::krylovBasicObservable(const std::string& name, std::vector<double> values)
    : obs_name(name), dim(0), numSamples(values.size()), sampleIndex(values.size()), type(VOID_TYPE_OBS),
      expectationValues(nullptr) {
  expectationValues = new double[numSamples];
  for (size_t i = 0; i != numSamples; i++) expectationValues[i] = values[i];
}

krylovBasicObservable::~krylovBasicObservable() {
  if (numSamples > 0) delete[] expectationValues;
}

obsType krylovBasicObservable::retType() { return type; }

krylovMatrixObservable::krylovMatrixObservable(const std::string& name, std::unique_ptr<matrix> obser)
    : krylovBasicObservable(name) {
  dim = obser->m;
  type = MATRIX_TYPE_OBS;
  tmpBlasVec = dim > 0 ? new std::complex<double>[dim] : nullptr;
  obs = std::move(obser);
}

krylovMatrixObservable::~krylovMatrixObservable() {
  if (dim > 0) delete[] tmpBlasVec;
}

std::complex<double> krylovMatrixObservable::expectation(std::complex<double>* vec, int len) {
  if (sampleIndex >= numSamples) {
    std::cerr << "Too many samples." << std::endl;
    exit(1);
  }
  if ((size_t)len != dim) {
    std::cerr << "Incompatible dimensions" << std::endl;
    exit(1);
  }
  std::complex<double> acc = 0;
  for (size_t r = 0; r < dim; ++r) {
    std::complex<double> s = 0;
    for (size_t c = 0; c < dim; ++c) s += obs->values[r + c * dim] * vec[c];
    acc += std::conj(vec[r]) * s;
  }
  expectationValues[sampleIndex++] = acc.real();
  return acc;
}

krylovSpMatrixObservable::krylovSpMatrixObservable(const std::string& name, std::unique_ptr<smatrix> obser)
    : krylovBasicObservable(name) {
  dim = obser->m;
  type = SPARSE_MATRIX_TYPE_OBS;
  obs = std::move(obser);
  obs->initialize();
  tmpBlasVec = new std::complex<double>[dim];
}

krylovSpMatrixObservable::~krylovSpMatrixObservable() {
  if (dim > 0) delete[] tmpBlasVec;
}

std::complex<double> krylovSpMatrixObservable::expectation(std::complex<double>* vec, int len) {
  if (sampleIndex >= numSamples) {
    std::cerr << "Too many samples." << std::endl;
    exit(1);
  }
  if ((size_t)len != dim) {
    std::cerr << "Incompatible dimensions" << std::endl;
    exit(1);
  }
  obs->spMV(one, vec, tmpBlasVec);
  std::complex<double> acc = 0;
  for (size_t i = 0; i < dim; ++i) acc += std::conj(vec[i]) * tmpBlasVec[i];
  expectationValues[sampleIndex++] = acc.real();
  return acc;
}

krylovVectorObservable::krylovVectorObservable(const std::string& name, std::complex<double>* obser, size_t len)
    : krylovBasicObservable(name) {
  dim = len;
  type = VECTOR_TYPE_OBS;
  obs = std::make_unique<std::complex<double>[]>(len);
  std::copy(obser, obser + len, obs.get());
}

std::complex<double> krylovVectorObservable::expectation(std::complex<double>* vec, int len) {
  if (sampleIndex >= numSamples) {
    std::cerr << "Too many samples." << std::endl;
    exit(1);
  }
  if ((size_t)len != dim) {
    std::cerr << "Incompatible dimensions" << std::endl;
    exit(1);
  }
  std::complex<double> acc = 0;
  for (size_t i = 0; i < dim; ++i) acc += std::conj(vec[i]) * obs[i];
  std::complex<double> ret(std::norm(acc), 0.0);
  expectationValues[sampleIndex++] = ret.real();
  return ret;
}

krylovOutputObservable::krylovOutputObservable(const std::string& name, std::vector<double> values)
    : krylovBasicObservable(name) {
  this->numSamples = values.size();
  initializeResultArray(numSamples);
  for (size_t i = 0; i != numSamples; i++) expectationValues[i] = values[i];
}

std::complex<double> krylovOutputObservable::expectation(std::complex<double>*, int) {
  throw std::runtime_error("krylovOutputObservable should not call `expectation` function.");
}

const char* requestStopException::what() const throw() {
  return "Observable requested termination of time evolution.";
}
