// hamiltonian.h -- operators built from creation/annihilation strings and their
// sparse matrices (public API of the reference's helper/hamiltonian.h:18-71).
#pragma once

#include <complex>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "Basis.h"
#include "matrixDataTypes.h"

using namespace TE;

/** One term: coef * op[n-1] ... op[1] op[0] (op[0] acts first); operations
 * +1 = creation, -1 = annihilation; capacity 0 = unbounded mode. */
struct opTerm {
  std::complex<double> coef;
  std::vector<int> operations;
  std::vector<int> mode;
  std::vector<int> capacity;
  void reset() {
    coef = std::complex<double>(0, 0);
    operations.clear();
    mode.clear();
    capacity.clear();
  }
};

class Hamiltonian {
 public:
  std::vector<opTerm> hamiltonOperator;

  Hamiltonian();

  std::string toString();
  std::unique_ptr<smatrix> createHamiltonMatrix(basicBasis* basis);
  std::vector<std::unique_ptr<smatrix>> createNumberOperatorObservables(basicBasis* basis);

  std::vector<opTerm> createKineticTerms(std::vector<int> modes, double gap);

  opTerm linInteraction(int a, int b, int ca, int cb, bool conjugate, double cof);
  opTerm createNumberOperator(int mode, double cof);
  opTerm createFourPointA(int a, int b, int c, int d, int ca, int cb, int cc, int cd, double cof);
  opTerm createFourPointB(int a, int b, int c, int d, int ca, int cb, int cc, int cd, double cof);
  opTerm createFourPointC(int a, int b, int c, int d, int ca, int cb, int cc, int cd, double cof);
  opTerm createSixPoint(int a, int b, int c, int d, int e, int f, int ca, int cb, int cc, int cd, int ce, int cf,
                        double cof);

  /** COO arrays of sum(op) in `basis` (rows ascending, columns ascending in a
   * row, per-column sums in term order, |v| < DBL_EPSILON dropped). */
  static void buildCOO(const std::vector<opTerm>& op, basicBasis* basis, std::vector<std::complex<double>>& values,
                       std::vector<size_t>& columns, std::vector<size_t>& rows);

 protected:
  std::unique_ptr<smatrix> createMatrix(std::vector<opTerm>& op, basicBasis* basis);
};
