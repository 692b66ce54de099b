// krylovTimeEvolver.h -- the GB300 TimeEvolver's evolution class, with the
// constructors, timeEvolve() and krylovReturn of core/krylovTimeEvolver.h:32-68.
// The evolution runs on the GPU through the C ABI of tegpu.h; this class keeps
// the reference's ownership rules (Ham and observables move in and come back
// in krylovReturn), exit(1) on the conditions where the reference exits, and
// its status codes.
#pragma once

#include <complex>
#include <memory>
#include <vector>

#include "krylovLogger.h"
#include "krylovObservables.h"
#include "matrixDataTypes.h"
#include "version.h"

class krylovReturn {
 public:
  std::complex<double>* evolvedState;
  double err;
  double evolvedTime;
  size_t numSamples;
  size_t n_steps;
  size_t dim;
  size_t krylovDim;
  /* 0 ok, 1 lucky breakdown, 2 analytic error below the roundoff estimate,
     3 stopped by an observable, 10 roundoff may spoil the error, 11 tolerance
     unreachable due to roundoff, 20 quadrature inaccurate, 30 norm drift,
     100 multiple of these (core/krylovTimeEvolver.h:41-44) */
  int statusCode;
  std::vector<std::unique_ptr<krylovBasicObservable>> observableList;
  std::unique_ptr<smatrix> hamiltonianMatrix;

  krylovReturn(unsigned int Hsize, int status);
  ~krylovReturn();
};

class krylovTimeEvolver {
 public:
  krylovTimeEvolver(double t, std::complex<double>* v, double samplingStep,
                    std::vector<std::unique_ptr<krylovBasicObservable>> observables, std::unique_ptr<smatrix> Ham,
                    double expFactor, double tol, int mm, bool fastIntegration, bool progressBar);
  krylovTimeEvolver(double t, std::complex<double>* v, double samplingStep,
                    std::vector<std::unique_ptr<krylovBasicObservable>> observables, std::unique_ptr<smatrix> Ham);
  krylovReturn* timeEvolve();
  ~krylovTimeEvolver();

  bool fastIntegration, progressBar;
  std::complex<double> expFactor;
  double tol;
  size_t m;

  void changeLogLevel(krylovLogger::loggingLevel level);

 protected:
  double t;
  size_t Hsize;
  double samplingStep;
  int nbObservables;
  std::unique_ptr<smatrix> Ham;
  std::vector<std::unique_ptr<krylovBasicObservable>> obsVector;
  krylovLogger logger;
  size_t n_samples;
  std::vector<std::complex<double>> initial;
};
