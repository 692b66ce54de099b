// hamiltonian.cpp -- operator strings to sparse matrices
// (reference: helper/hamiltonian.cpp:11-456).
//
// createMatrix gives the reference's COO exactly: for every basis row, each
// term is applied operator by operator (op[0] first, sqrt(n+1) for a creation,
// sqrt(n) for an annihilation, zero past a capacity or below zero), the
// contributions are summed per target column in term order, columns are
// emitted ascending and sums with |v| < DBL_EPSILON are dropped.  Rows are
// independent, so blocks of rows are built on all host threads and
// concatenated in row order (the result does not depend on the thread count).
#include "hamiltonian.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <thread>

namespace {

opTerm make_term(double cof, std::vector<int> ops, std::vector<int> modes, std::vector<int> caps) {
  opTerm t;
  t.coef = std::complex<double>(cof, 0.0);
  t.operations = std::move(ops);
  t.mode = std::move(modes);
  t.capacity = std::move(caps);
  return t;
}

// Apply one term to a basis vector in place; returns false when the result is
// zero.  coef accumulates the square-root factors (complex * real, as the
// reference's coef *= sqrt(...)).
bool apply_term(const opTerm& t, int* occ, int K, std::complex<double>& coef) {
  bool alive = true;
  for (size_t i = 0; i < t.operations.size(); ++i) {
    const int md = t.mode[i];
    if (md < 0 || md >= K) {
      std::cerr << "creationOperator: mode does not exist in vector\n";
      exit(14);
    }
    const int n = occ[md];
    if (t.operations[i] == 1) {
      const int c = t.capacity[i];
      if (c != 0 && n + 1 > c) {
        alive = false;
      } else {
        coef = coef * std::sqrt(n + 1.0);
        occ[md] = n + 1;
      }
    } else if (t.operations[i] == -1) {
      if (n == 0) {
        alive = false;
      } else {
        coef = coef * std::sqrt((double)n);
        occ[md] = n - 1;
      }
    }
    if (!alive) return false;
  }
  return true;
}

}  // namespace

Hamiltonian::Hamiltonian() {}

std::vector<opTerm> Hamiltonian::createKineticTerms(std::vector<int> modes, double gap) {
  std::vector<opTerm> ret;
  for (int md : modes) ret.push_back(make_term(gap, {-1, 1}, {md, md}, {0, 0}));
  return ret;
}

opTerm Hamiltonian::linInteraction(int a, int b, int ca, int cb, bool conjugate, double cof) {
  if (!conjugate) return make_term(cof, {-1, 1}, {b, a}, {cb, ca});
  return make_term(cof, {-1, 1}, {a, b}, {ca, cb});
}

opTerm Hamiltonian::createNumberOperator(int mode, double cof) {
  return make_term(cof, {-1, 1}, {mode, mode}, {0, 0});
}

opTerm Hamiltonian::createFourPointA(int a, int b, int c, int d, int ca, int cb, int cc, int cd, double cof) {
  return make_term(cof, {-1, 1, -1, 1}, {d, c, b, a}, {cd, cc, cb, ca});
}

opTerm Hamiltonian::createFourPointB(int a, int b, int c, int d, int ca, int cb, int cc, int cd, double cof) {
  return make_term(cof, {-1, -1, 1, 1}, {d, c, b, a}, {cd, cc, cb, ca});
}

opTerm Hamiltonian::createFourPointC(int a, int b, int c, int d, int ca, int cb, int cc, int cd, double cof) {
  return make_term(cof, {1, 1, -1, -1}, {d, c, b, a}, {cd, cc, cb, ca});
}

opTerm Hamiltonian::createSixPoint(int a, int b, int c, int d, int e, int f, int ca, int cb, int cc, int cd, int ce,
                                   int cf, double cof) {
  return make_term(cof, {-1, 1, -1, 1, -1, 1}, {f, e, d, c, b, a}, {cf, ce, cd, cc, cb, ca});
}

std::string Hamiltonian::toString() {
  std::string ret;
  for (auto& t : hamiltonOperator) {
    ret += std::to_string(t.coef.real());
    for (size_t i = 0; i != t.capacity.size(); i++) {
      ret += (t.capacity[i] == 0) ? "a" : "b";
      ret += std::to_string(t.mode[i]);
      if (t.operations[i] == 1) ret += "d";
    }
    ret += "\n+";
  }
  return ret;
}

std::unique_ptr<smatrix> Hamiltonian::createHamiltonMatrix(basicBasis* basis) {
  return createMatrix(hamiltonOperator, basis);
}

std::vector<std::unique_ptr<smatrix>> Hamiltonian::createNumberOperatorObservables(basicBasis* basis) {
  std::vector<std::unique_ptr<smatrix>> out;
  for (int i = 0; i != basis->numberModes; i++) {
    std::vector<opTerm> ops{createNumberOperator(i, 1)};
    out.push_back(createMatrix(ops, basis));
  }
  return out;
}

void Hamiltonian::buildCOO(const std::vector<opTerm>& op, basicBasis* basis,
                           std::vector<std::complex<double>>& values, std::vector<size_t>& columns,
                           std::vector<size_t>& rows) {
  const int n = basis->numberElements;
  const int K = basis->numberModes;
  unsigned nt = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
  if (n < 4096) nt = 1;
  struct Part {
    std::vector<std::complex<double>> v;
    std::vector<size_t> c, r;
  };
  std::vector<Part> parts(nt);
  auto work = [&](unsigned tid) {
    const int r0 = (int)((int64_t)n * tid / nt), r1 = (int)((int64_t)n * (tid + 1) / nt);
    Part& P = parts[tid];
    std::vector<std::pair<int, std::complex<double>>> row;  // (column, value) in term order
    basisVector probe(K);
    for (int j = r0; j < r1; ++j) {
      row.clear();
      for (const opTerm& t : op) {
        for (int a = 0; a < K; ++a) probe.e[a] = basis->basisElements[j].e[a];
        std::complex<double> coef(1.0, 0.0);
        if (!apply_term(t, probe.e, K, coef)) continue;  // a zero contribution cannot change a sum
        coef = coef * t.coef;
        auto it = basis->hashTable.find(probe);
        if (it == basis->hashTable.end()) continue;
        const int col = it->second;
        bool merged = false;
        for (auto& e : row)
          if (e.first == col) {
            e.second += coef;
            merged = true;
            break;
          }
        if (!merged) row.emplace_back(col, coef);
      }
      std::stable_sort(row.begin(), row.end(), [](const auto& x, const auto& y) { return x.first < y.first; });
      for (auto& e : row) {
        if (std::abs(e.second) < DBL_EPSILON) continue;
        P.r.push_back((size_t)j);
        P.c.push_back((size_t)e.first);
        P.v.push_back(e.second);
      }
    }
  };
  if (nt == 1) {
    work(0);
  } else {
    std::vector<std::thread> th;
    for (unsigned i = 0; i < nt; ++i) th.emplace_back(work, i);
    for (auto& x : th) x.join();
  }
  size_t total = 0;
  for (auto& P : parts) total += P.v.size();
  values.clear();
  columns.clear();
  rows.clear();
  values.reserve(total);
  columns.reserve(total);
  rows.reserve(total);
  for (auto& P : parts) {
    values.insert(values.end(), P.v.begin(), P.v.end());
    columns.insert(columns.end(), P.c.begin(), P.c.end());
    rows.insert(rows.end(), P.r.begin(), P.r.end());
  }
}

std::unique_ptr<smatrix> Hamiltonian::createMatrix(std::vector<opTerm>& op, basicBasis* basis) {
  std::vector<std::complex<double>> v;
  std::vector<size_t> c, r;
  buildCOO(op, basis, v, c, r);
  const unsigned int N = (unsigned int)basis->numberElements;
  return std::make_unique<smatrix>(v.data(), c.data(), r.data(), v.size(), N, N);
}
