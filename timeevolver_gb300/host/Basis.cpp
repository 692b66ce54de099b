// Basis.cpp -- basis enumeration in the reference's order
// (helper/Basis.cpp:37-121 and :131-182).
#include "Basis.h"

#include <algorithm>

basis::~basis() { delete[] basisElements; }

void basis::createHashTable() {
  hashTable.reserve((size_t)numberElements * 2);
  for (int i = 0; i != numberElements; i++) hashTable.insert(std::make_pair(basisElements[i], i));
}

basis::basis(int N, int K, int nbQudits, int capacity) : basis(N, K, nbQudits, capacity, 1) {}

basis::basis(int N, int K, int nbQudits, int capacity, int quant) {
  numberModes = K;
  // occupations of modes 1..K-1 as flat rows of K ints; mode 0 set at the end
  std::vector<int> states(K, 0);
  size_t count = 1;
  for (int k = K; k > 1; k--) {
    const size_t existing = count;
    for (size_t l = 0; l < existing; ++l) {
      int occ = 0;
      for (int i = 0; i < K; ++i) occ += states[l * K + i];
      int upper = (k > K - nbQudits) ? std::min(N - occ, capacity) : N - occ;
      std::vector<int> row(states.begin() + l * K, states.begin() + (l + 1) * K);
      for (int o = quant; o <= upper; o += quant) {
        row[k - 1] = o;
        states.insert(states.end(), row.begin(), row.end());
        ++count;
      }
    }
  }
  std::vector<size_t> keep;
  keep.reserve(count);
  for (size_t l = 0; l < count; ++l) {
    int occ = 0;
    for (int i = 0; i < K; ++i) occ += states[l * K + i];
    int missing = N - occ;
    if (K != nbQudits || missing <= capacity) {
      states[l * K] = missing;
      keep.push_back(l);
    }
  }
  numberElements = (int)keep.size();
  basisElements = new basisVector[numberElements];
  for (int i = 0; i < numberElements; ++i) {
    basisElements[i].zeros(K);
    basisElements[i].initInt(&states[keep[i] * K], K);
  }
  qudits = capacity;
  createHashTable();
}

tensorBasis::tensorBasis(int N1, int K1, int N2, int K2, int C2) {
  numberModes = K1 + K2;
  qudits = C2;
  basis b1(N1, K1, 0, 0);
  basis b2(N2, K2, K2, C2);
  const int l1 = b1.numberElements, l2 = b2.numberElements;
  numberElements = l1 * l2;
  if (l2 == 0) {
    // as the reference: the elements of the first factor, numberElements stays 0
    basisElements = new basisVector[l1];
    for (int i = 0; i != l1; i++) basisElements[i] = b1.basisElements[i];
    return;
  }
  basisElements = new basisVector[(size_t)l1 * l2];
  std::vector<int> tmp(K1 + K2);
  for (int i = 0; i != l1; i++)
    for (int j = 0; j != l2; j++) {
      for (int a = 0; a < K1; ++a) tmp[a] = b1.basisElements[i].e[a];
      for (int a = 0; a < K2; ++a) tmp[K1 + a] = b2.basisElements[j].e[a];
      basisElements[i * l2 + j].zeros(K1 + K2);
      basisElements[i * l2 + j].initInt(tmp.data(), K1 + K2);
    }
  createHashTable();
}

void tensorBasis::createHashTable() {
  hashTable.reserve((size_t)numberElements * 2);
  for (int i = 0; i != numberElements; i++) hashTable.insert(std::make_pair(basisElements[i], i));
}
