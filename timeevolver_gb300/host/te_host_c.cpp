// te_host_c.cpp -- C entry points (include/te_model.h) over the C++ basis and
// Hamiltonian helpers.
#include <memory>
#include <vector>

#include "Basis.h"
#include "hamiltonian.h"
#include "te_model.h"

struct te_basis_s {
  std::unique_ptr<basicBasis> b;
};

struct te_operator_s {
  std::vector<opTerm> terms;
  std::vector<std::complex<double>> v;
  std::vector<size_t> c, r;
};

extern "C" int te_basis_create(int N, int K, int nb_qudits, int capacity, int quant, te_basis* out) {
  if (!out || N < 0 || K < 1 || quant < 1) return -1;
  te_basis h = new te_basis_s();
  h->b.reset(new basis(N, K, nb_qudits, capacity, quant));
  *out = h;
  return 0;
}

extern "C" int te_tensor_basis_create(int N1, int K1, int N2, int K2, int C2, te_basis* out) {
  if (!out || N1 < 0 || K1 < 1 || N2 < 0 || K2 < 1) return -1;
  te_basis h = new te_basis_s();
  h->b.reset(new tensorBasis(N1, K1, N2, K2, C2));
  *out = h;
  return 0;
}

extern "C" int te_basis_destroy(te_basis b) {
  delete b;
  return 0;
}

extern "C" int te_basis_shape(te_basis b, int64_t* n_elements, int* n_modes) {
  if (!b) return -1;
  if (n_elements) *n_elements = b->b->numberElements;
  if (n_modes) *n_modes = b->b->numberModes;
  return 0;
}

extern "C" int te_basis_elements(te_basis b, int32_t* out) {
  if (!b || !out) return -1;
  const int K = b->b->numberModes;
  for (int i = 0; i < b->b->numberElements; ++i)
    for (int a = 0; a < K; ++a) out[(int64_t)i * K + a] = b->b->basisElements[i].e[a];
  return 0;
}

extern "C" int64_t te_basis_index(te_basis b, const int32_t* occupations) {
  if (!b || !occupations) return -1;
  basisVector v(b->b->numberModes);
  for (int a = 0; a < b->b->numberModes; ++a) v.e[a] = occupations[a];
  auto it = b->b->hashTable.find(v);
  return it == b->b->hashTable.end() ? -1 : it->second;
}

extern "C" int te_operator_create(te_operator* out) {
  if (!out) return -1;
  *out = new te_operator_s();
  return 0;
}

extern "C" int te_operator_destroy(te_operator op) {
  delete op;
  return 0;
}

extern "C" int te_operator_add_term(te_operator op, double coef_re, double coef_im, int n_ops, const int32_t* ops,
                                    const int32_t* modes, const int32_t* capacities) {
  if (!op || n_ops < 0 || (n_ops > 0 && (!ops || !modes || !capacities))) return -1;
  opTerm t;
  t.coef = std::complex<double>(coef_re, coef_im);
  for (int i = 0; i < n_ops; ++i) {
    if (ops[i] != 1 && ops[i] != -1) return -1;
    t.operations.push_back(ops[i]);
    t.mode.push_back(modes[i]);
    t.capacity.push_back(capacities[i]);
  }
  op->terms.push_back(t);
  return 0;
}

extern "C" int te_operator_build(te_operator op, te_basis b, int64_t* nnz) {
  if (!op || !b) return -1;
  for (auto& t : op->terms)
    for (int md : t.mode)
      if (md < 0 || md >= b->b->numberModes) return -1;
  Hamiltonian::buildCOO(op->terms, b->b.get(), op->v, op->c, op->r);
  if (nnz) *nnz = (int64_t)op->v.size();
  return 0;
}

extern "C" int te_operator_coo(te_operator op, uint64_t* rows, uint64_t* cols, double* values) {
  if (!op) return -1;
  for (size_t i = 0; i < op->v.size(); ++i) {
    if (rows) rows[i] = op->r[i];
    if (cols) cols[i] = op->c[i];
    if (values) {
      values[2 * i] = op->v[i].real();
      values[2 * i + 1] = op->v[i].imag();
    }
  }
  return 0;
}
