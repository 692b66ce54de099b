// Basis.h -- Fock bases of the GB300 TimeEvolver, with the public API of the
// reference's helper/Basis.h (basisVector, basisVectorHasher, basisState,
// basicBasis, basis, tensorBasis).  The order of the basis elements -- which
// fixes the layout of every state vector -- is the reference's
// (helper/Basis.cpp:64-91): modes K-1 down to 1 each append their non-zero
// occupations to every state found so far, mode 0 takes the remainder.
#pragma once

#include <complex>
#include <cstdint>
#include <iostream>
#include <unordered_map>
#include <vector>

/** Occupation numbers of the modes (helper/Basis.h:15-213). */
struct basisVector {
  int* e;
  size_t length;

  basisVector() : e(nullptr), length(0) {}
  basisVector(unsigned int le) {
    length = le;
    e = le ? new int[le]() : nullptr;
  }
  basisVector(int le, int pos) {
    if (le <= pos) {
      std::cerr << "basisvector too small" << std::endl;
      exit(12);
    }
    length = le > 0 ? (size_t)le : 0;
    e = le > 0 ? new int[le]() : nullptr;
    if (e) e[pos] = 1;
  }
  basisVector(const basisVector& o) : e(nullptr), length(o.length) {
    if (length) {
      e = new int[length];
      for (size_t i = 0; i < length; ++i) e[i] = o.e[i];
    }
  }
  ~basisVector() {
    if (length > 0) delete[] e;
  }
  void ones() {
    for (size_t i = 0; i < length; i++) e[i] = 1;
  }
  void zeros() {
    for (size_t i = 0; i < length; i++) e[i] = 0;
  }
  void zeros(int n) {
    if (n > 0) {
      if (length != 0) delete[] e;
      length = n;
      e = new int[n];
    }
    zeros();
  }
  void initInt(int* init, unsigned int le) {
    if (length == le)
      for (unsigned int i = 0; i != le; i++) e[i] = init[i];
  }
  int occuNumber() {
    int r = 0;
    for (size_t i = 0; i < length; i++) r += e[i];
    return r;
  }
  bool operator==(const basisVector& b) const {
    if (b.length != length) return false;
    for (size_t i = 0; i != length; i++)
      if (e[i] != b.e[i]) return false;
    return true;
  }
  basisVector& operator=(const basisVector& rhs) {
    if (this == &rhs) return *this;
    if (rhs.length != length) {
      if (length > 0) delete[] e;
      length = rhs.length;
      e = length ? new int[length] : nullptr;
    }
    for (size_t i = 0; i != length; i++) e[i] = rhs.e[i];
    return *this;
  }
};

/** Hash of an occupation vector (any good mix works: only lookups use it). */
struct basisVectorHasher {
  std::size_t operator()(const basisVector& b) const {
    uint64_t h = 1469598103934665603ull;
    for (size_t i = 0; i < b.length; ++i) {
      h ^= (uint64_t)(uint32_t)b.e[i] + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
      h *= 1099511628211ull;
    }
    return (std::size_t)h;
  }
};

/** A basis vector with a complex coefficient (helper/Basis.h:236-272). */
struct basisState {
 public:
  basisVector b;
  std::complex<double> coef;
  basisState(const basisState& rhs) {
    b = rhs.b;
    coef = rhs.coef;
  }
  basisState() {
    b = basisVector();
    coef = 0;
  }
  basisState(basisVector& rhs, std::complex<double>& c) {
    b = basisVector(rhs);
    coef = c;
  }
};

class basicBasis {
 public:
  int numberModes;
  int qudits;
  int numberElements;
  basisVector* basisElements;
  std::unordered_map<basisVector, int, basisVectorHasher> hashTable;

  virtual void createHashTable() = 0;
  basicBasis() {}
  virtual ~basicBasis() {}
};

/** N particles in K modes; the first nbQudits modes counted from the top
 * (K-1, K-2, ...) hold at most `capacity`; modes > 0 step by `quant`. */
class basis : public basicBasis {
 public:
  basis(int N, int K, int nbQudits, int capacity, int quant);
  basis(int N, int K, int nbQudits, int capacity);

  /** Binomial coefficient, 1 when k > n (helper/Basis.h:309-315). */
  int nchoosekSmart(int n, int k) {
    if (k > n) return 1;
    double r = 1.0;
    for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
    return (int)(r + 0.5);
  }

  basis& operator=(const basis& rhs) {
    if (numberElements > 0) delete[] basisElements;
    numberElements = rhs.numberElements;
    numberModes = rhs.numberModes;
    qudits = rhs.qudits;
    basisElements = new basisVector[numberElements];
    for (int i = 0; i != numberElements; i++) basisElements[i] = rhs.basisElements[i];
    return *this;
  }

  ~basis();
  void createHashTable();
};

/** Tensor product of basis(N1,K1,0,0) and basis(N2,K2,K2,C2), first index
 * major (helper/Basis.cpp:131-182). */
class tensorBasis : public basicBasis {
 public:
  tensorBasis(int N1, int K1, int N2, int K2, int C2);
  tensorBasis() {
    numberElements = 0;
    numberModes = 0;
    qudits = -1;
    basisElements = nullptr;
  }
  void createHashTable();
  ~tensorBasis() {
    if (numberElements != 0) delete[] basisElements;
  }
};
