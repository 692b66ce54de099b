"""C++ basis / Hamiltonian helpers (libtimeevolver.so) against the oracle's
numpy restatement: identical basis order and bit-identical COO arrays (CPU)."""
import numpy as np
import pytest

from oracle import models as om


@pytest.fixture(scope="module")
def tm():
    import timeevolver_gb300 as te
    te.build()
    from timeevolver_gb300 import models
    return models


@pytest.mark.parametrize("N,K,nq,cap,quant", [(2, 3, 0, 0, 1), (8, 8, 0, 0, 1), (6, 5, 2, 2, 1), (7, 4, 0, 0, 2),
                                              (2, 8, 8, 1, 1), (3, 1, 0, 0, 1)])
def test_basis_order(tm, N, K, nq, cap, quant):
    B = tm.Basis(N, K, nq, cap, quant)
    ref = om.basis(N, K, nq, cap, quant)
    assert np.array_equal(B.elements(), ref)
    for i in [0, len(ref) // 2, len(ref) - 1]:
        assert B.index(ref[i]) == i


def test_tensor_basis(tm):
    B = tm.Basis.tensor(20, 2, 2, 8, 1)
    assert np.array_equal(B.elements(), om.tensor_basis(20, 2, 2, 8, 1))


def test_bose_hubbard_matrix_bitwise(tm):
    for L, N, J, U in [(6, 6, 1.0, 2.0), (8, 8, 1.0, 2.0), (5, 7, [0.9, 1.1, 1.0, 0.8], 3.0)]:
        B, (r, c, v) = tm.bose_hubbard(L, N, J, U)
        _, (r2, c2, v2) = om.bose_hubbard(L, N, J, U)
        assert np.array_equal(r, r2) and np.array_equal(c, c2)
        assert np.array_equal(v.view(np.float64), v2.view(np.float64))


def test_black_hole_terms(tm):
    B = tm.Basis.tensor(20, 2, 2, 8, 1)
    terms = om.black_hole_terms(20, 2, 12.0, 4)
    r, c, v = tm.operator_matrix(terms, B)
    r2, c2, v2 = om.create_matrix(terms, om.tensor_basis(20, 2, 2, 8, 1))
    assert np.array_equal(r, r2) and np.array_equal(c, c2) and np.array_equal(v, v2)


def test_number_operators(tm):
    B = tm.Basis(4, 3)
    obs = tm.number_operator_observables(B)
    ref = om.number_operator_observables(om.basis(4, 3))
    for (r, c, v), (r2, c2, v2) in zip(obs, ref):
        assert np.array_equal(r, r2) and np.array_equal(c, c2) and np.array_equal(v, v2)
