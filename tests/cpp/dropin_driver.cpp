// Drop-in check: a program written against the reference's C++ API (basis,
// Hamiltonian, krylovSpMatrixObservable, krylovTimeEvolver, krylovReturn),
// compiled against the GB300 headers.  Prints one line per observable with
// its samples, then a line with the krylovReturn fields.
//
//   dropin_driver simple [csv_prefix]  two coupled oscillators (dim 201), t=10, tol 1e-6;
//                                     with csv_prefix the samples also go through saveResult
//   dropin_driver blackhole N0 Nm K maxT samplingStep
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "Basis.h"
#include "hamiltonian.h"
#include "krylovHelper.h"
#include "krylovObservables.h"
#include "krylovTimeEvolver.h"
#include "matrixDataTypes.h"

static double sym_break(int a, int b) {
  double c = std::fmod(std::sqrt(2.0) * std::pow(a, 3) + std::sqrt(7.0) * std::pow(b, 5), 1.0);
  return c < 0.5 ? c - 1.0 : c;
}

static void print_result(krylovReturn* res) {
  for (auto& o : res->observableList) {
    double* v = o->retExpectationValues();
    std::printf("%s", o->retName().c_str());
    for (size_t i = 0; i < o->retNumSamples(); ++i) std::printf(" %.17g", v[i]);
    std::printf("\n");
  }
  std::printf("RESULT status=%d steps=%zu samples=%zu krylov=%zu err=%.17g time=%.17g\n", res->statusCode,
              res->n_steps, res->numSamples, res->krylovDim, res->err, res->evolvedTime);
}

static int run(basicBasis& b, Hamiltonian& ham, std::vector<int> init, double t, double dt, double tol, bool full,
               const char* csv_prefix = nullptr) {
  std::unique_ptr<smatrix> H = ham.createHamiltonMatrix(&b);
  std::vector<std::unique_ptr<smatrix>> ops = ham.createNumberOperatorObservables(&b);
  std::vector<std::unique_ptr<krylovBasicObservable>> obs;
  for (size_t i = 0; i < ops.size(); ++i)  // named by mode index, as in the reference's example
    obs.push_back(std::make_unique<krylovSpMatrixObservable>(std::to_string(i), std::move(ops[i])));
  basisVector bv((unsigned)init.size());
  for (size_t i = 0; i < init.size(); ++i) bv.e[i] = init[i];
  std::vector<std::complex<double>> v(b.numberElements);
  v[b.hashTable.find(bv)->second] = 1.0;
  krylovReturn* res;
  if (full) {
    krylovTimeEvolver ev(t, v.data(), dt, std::move(obs), std::move(H), 1.0, tol, 40, false, false);
    ev.changeLogLevel(krylovLogger::ERROR);
    res = ev.timeEvolve();
  } else {
    krylovTimeEvolver ev(t, v.data(), dt, std::move(obs), std::move(H));
    ev.changeLogLevel(krylovLogger::ERROR);
    res = ev.timeEvolve();
  }
  print_result(res);
  if (csv_prefix) {
    parameter_list none;
    saveResult(res->observableList, none, csv_prefix);
  }
  delete res;
  return 0;
}

int main(int argc, char** argv) {
  if (argc >= 2 && std::strcmp(argv[1], "simple") == 0) {
    const int N0 = 200;
    basis b(N0, 2, 0, 0);
    Hamiltonian ham;
    ham.hamiltonOperator = {ham.createNumberOperator(0, 1.0), ham.createNumberOperator(1, 2.0),
                            ham.linInteraction(0, 1, 0, 0, false, 1.0), ham.linInteraction(0, 1, 0, 0, true, 1.0)};
    return run(b, ham, {N0, 0}, 10.0, 0.01, 1e-6, false,  // 5-argument constructor: tol 1e-6, m 40
               argc >= 3 ? argv[2] : nullptr);
  }
  if (argc >= 7 && std::strcmp(argv[1], "blackhole") == 0) {
    const int N0 = std::atoi(argv[2]), Nm = std::atoi(argv[3]), K = std::atoi(argv[4]);
    const double maxT = std::atof(argv[5]), dt = std::atof(argv[6]);
    const int C = 1;
    const double DeltaN = 12, C0 = 1, Cm = 1, sq = std::sqrt((double)N0);
    tensorBasis b(N0, 2, Nm, 2 * K, C);
    Hamiltonian ham;
    std::vector<opTerm>& h = ham.hamiltonOperator;
    for (int i = 2; i < K + 2; i++) h.push_back(ham.createNumberOperator(i, sq));
    for (int i = 2 + K; i < 2 * K + 2; i++) h.push_back(ham.createNumberOperator(i, sq));
    h.push_back(ham.linInteraction(0, 1, 0, 0, true, C0));
    h.push_back(ham.linInteraction(0, 1, 0, 0, false, C0));
    for (int i = 2; i < 2 + K; i++) h.push_back(ham.createFourPointA(0, 0, i, i, 0, 0, C, C, -sq / N0));
    for (int i = 2 + K; i < 2 + 2 * K; i++) h.push_back(ham.createFourPointA(0, 0, i, i, 0, 0, C, C, -sq / (N0 - DeltaN)));
    for (int m = 2; m <= 2 * K + 1; m++)
      for (int M = 2; M <= 2 * K + 1; M++) {
        double coeff = 0;
        if (m <= 1 + K && M > K + 1)
          coeff = sym_break(m, M) * Cm;
        else if (((m <= K + 1 && M <= 1 + K) || (m > 1 + K && M > 1 + K)) && m < M)
          coeff = sym_break(m, M) * Cm;
        if (coeff != 0) {
          opTerm a;
          a.coef = coeff;
          a.capacity = {C, C};
          a.mode = {m, M};
          a.operations = {-1, 1};
          h.push_back(a);
          opTerm bt = a;
          bt.mode = {M, m};
          h.push_back(bt);
        }
      }
    std::vector<int> init(2 + 2 * K, 0);
    init[0] = N0;
    for (int i = 0; i < std::min(K, Nm); ++i) init[2 + i] = 1;
    return run(b, ham, init, maxT, dt, 1e-8, true);
  }
  std::fprintf(stderr, "usage: dropin_driver simple | blackhole N0 Nm K maxT samplingStep\n");
  return 2;
}
