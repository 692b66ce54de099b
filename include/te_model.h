/*
 * te_model.h -- C entry points of the model helpers in libtimeevolver.so
 * (the C++ basis / Hamiltonian classes of timeevolver_gb300/host), for
 * callers that cannot use C++ (Python ctypes, other FFIs).
 *
 * Reference interfaces replaced (paths inside the TimeEvolver project):
 *   basis(N, K, nbQudits, capacity[, quant])   helper/Basis.h:300-301, Basis.cpp:26-121
 *   tensorBasis(N1, K1, N2, K2, C2)            helper/Basis.h:346, Basis.cpp:131-182
 *   basicBasis::hashTable lookups              helper/Basis.h:284
 *   Hamiltonian opTerm list + createMatrix     helper/hamiltonian.h:18-71, hamiltonian.cpp:318-402
 * Returns 0 on success, a negative code on invalid input.
 */
#ifndef TE_MODEL_H
#define TE_MODEL_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct te_basis_s* te_basis;
typedef struct te_operator_s* te_operator;

int te_basis_create(int N, int K, int nb_qudits, int capacity, int quant, te_basis* out);
int te_tensor_basis_create(int N1, int K1, int N2, int K2, int C2, te_basis* out);
int te_basis_destroy(te_basis b);
/* number of elements and modes */
int te_basis_shape(te_basis b, int64_t* n_elements, int* n_modes);
/* occupation numbers, row-major n_elements x n_modes */
int te_basis_elements(te_basis b, int32_t* out);
/* index of an occupation vector, -1 when absent */
int64_t te_basis_index(te_basis b, const int32_t* occupations);

int te_operator_create(te_operator* out);
int te_operator_destroy(te_operator op);
/* append one opTerm: coef * ops[n-1]...ops[0] (ops[0] acts first),
 * +1 creation / -1 annihilation, capacity 0 = unbounded */
int te_operator_add_term(te_operator op, double coef_re, double coef_im, int n_ops, const int32_t* ops,
                         const int32_t* modes, const int32_t* capacities);
/* build the sparse matrix in basis b; *nnz receives the entry count */
int te_operator_build(te_operator op, te_basis b, int64_t* nnz);
/* copy the built COO (rows, columns as uint64; complex values interleaved) */
int te_operator_coo(te_operator op, uint64_t* rows, uint64_t* cols, double* values);

#ifdef __cplusplus
}
#endif
#endif
