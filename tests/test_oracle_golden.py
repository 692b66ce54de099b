"""The oracle against the reference's own golden outputs (CPU only).

Goldens: output/ResultBlackHole_N20_*.h5 (test/testBlackHole.cpp),
output/ResultBlackHole_N1_*.h5 (test/testBlackHoleLB.cpp) and
output/SimpleExampleOutputOccupationNumber*.csv (test/testSimpleExample.cpp),
extracted by tests/golden/make_golden.py.  The reference compares at 1e-8
absolute (testBlackHole.cpp:39-44); the CSV golden is rounded to 6 digits.
"""
import os

import numpy as np
import pytest

from oracle import models

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _vec(n, i):
    v = np.zeros(n, dtype=np.complex128)
    v[i] = 1.0
    return v


def test_black_hole_n20(oracle_lib):
    states, H, i0 = models.black_hole(N0=20, Nm=2, K=4)
    assert len(states) == 588
    obs = [("sparse", o) for o in models.number_operator_observables(states)]
    r = oracle_lib.evolve(H, _vec(len(states), i0), 10.0, 0.01, obs, tol=1e-8, m=40)
    gold = np.load(os.path.join(GOLD, "blackhole_N20.npy"))
    assert r["num_samples"] == 1001
    assert np.max(np.abs(r["samples"] - gold)) < 1e-8
    assert r["err"] <= 1e-8


def test_black_hole_lucky_breakdown(oracle_lib):
    states, H, i0 = models.black_hole(N0=1, Nm=1, K=1)
    assert len(states) == 4
    obs = [("sparse", o) for o in models.number_operator_observables(states)]
    r = oracle_lib.evolve(H, _vec(4, i0), 1000.0, 1.0, obs, tol=1e-8, m=40)
    gold = np.load(os.path.join(GOLD, "blackhole_N1_LB.npy"))
    assert r["status"] == 1 and r["krylov_dim"] == 4 and r["n_steps"] == 1
    assert np.max(np.abs(r["samples"] - gold)) < 1e-8


def test_simple_example_six_digits(oracle_lib):
    states, H, i0 = models.simple_example()
    obs = [("sparse", o) for o in models.number_operator_observables(states)]
    r = oracle_lib.evolve(H, _vec(len(states), i0), 10.0, 0.01, obs, tol=1e-6, m=40)
    gold = np.load(os.path.join(GOLD, "simple_example.npy"))
    rounded = np.vectorize(lambda x: float("%g" % x))(r["samples"])
    assert np.array_equal(rounded, gold)


def test_basis_order_and_sizes():
    # helper/Basis.cpp:64-91: mode K-1 is filled first, the write index never resets
    b = models.basis(2, 3)
    assert b.tolist() == [[2, 0, 0], [1, 0, 1], [0, 0, 2], [1, 1, 0], [0, 2, 0], [0, 1, 1]]
    assert len(models.basis(8, 8)) == 6435
    assert len(models.tensor_basis(20, 2, 2, 8, 1)) == 588
    q = models.basis(2, 4, 4, 1)  # all modes capped at 1
    assert (q.sum(axis=1) == 2).all() and q.max() == 1 and len(q) == 6


def test_bose_hubbard_nnz_formula():
    # offdiag = 2(L-1) C(N+L-2, L-1), diag = dim - C(L, N) (rows with all n_i <= 1 vanish)
    from math import comb
    for L, N in [(6, 6), (8, 8)]:
        states, (row, col, val) = models.bose_hubbard(L, N, 1.0, 2.0)
        dim = comb(N + L - 1, N)
        assert len(states) == dim
        off = np.sum(row != col)
        assert off == 2 * (L - 1) * comb(N + L - 2, L - 1)
        assert np.sum(row == col) == dim - comb(L, N)
        # Hermitian
        A = np.zeros((dim, dim), dtype=complex) if dim < 3000 else None
        if A is not None:
            A[row, col] = val
            assert np.allclose(A, A.conj().T)


def test_spmv_and_norm1(oracle_lib):
    states, H = models.bose_hubbard(5, 4, 1.0, 2.0)
    n = len(states)
    rng = np.random.default_rng(3)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    A = np.zeros((n, n), dtype=complex)
    np.add.at(A, (H[0], H[1]), H[2])
    y = oracle_lib.spmv(H, x, alpha=-0.5j)
    assert np.allclose(y, -0.5j * (A @ x), rtol=0, atol=1e-12)
    assert abs(oracle_lib.norm1(H, n) - np.abs(A).sum(axis=0).max()) < 1e-12


def test_quadrature_rule(oracle_lib):
    for kind, p, a, b, exact in [(0, 3.0, 0.0, 1.0, 0.25), (1, 2.0, 0.0, 1.0, np.sin(2.0) / 2),
                                 (2, 1.0, 0.0, 2.0, np.e ** 2 - 1), (0, 39.0, 0.0, 1.0, 1 / 40)]:
        val, err, l1, levels = oracle_lib.ts_test(kind, p, a, b, 1e-3)
        assert abs(val - exact) < 1e-6 * abs(exact)
        assert err <= 1e-3 * l1 and levels >= 2


def test_lanczos_and_eigen(oracle_lib):
    states, H = models.bose_hubbard(6, 4, 1.0, 2.0)
    n = len(states)
    rng = np.random.default_rng(0)
    v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    v /= np.linalg.norm(v)
    L = oracle_lib.lanczos(H, v, 20, 1e-12)
    V, Hm = L["V"], L["H"]
    # orthonormal basis and the Krylov relation A V = V H_k + h v_m e_m^T
    assert np.allclose(V.conj().T @ V, np.eye(20), atol=1e-8)
    lam, Z = oracle_lib.krylov_eig(Hm)
    assert np.allclose(Z @ np.diag(lam) @ Z.conj().T, Hm, atol=1e-10)
    assert np.allclose(lam.real, 0.0, atol=1e-12)


def test_stop_request_semantics(oracle_lib):
    states, H = models.bose_hubbard(4, 4, 1.0, 2.0)
    n = len(states)
    v = np.zeros(n, dtype=np.complex128)
    v[0] = 1
    obs = [("sparse", o) for o in models.number_operator_observables(states)] + [("stop", 5)]
    r = oracle_lib.evolve(H, v, 2.0, 0.1, obs, tol=1e-8, m=20)
    assert r["status"] == 3 and r["num_samples"] == 5
    r0 = oracle_lib.evolve(H, v, 2.0, 0.1, obs[:-1] + [("stop", 0)], tol=1e-8, m=20)
    assert r0["status"] == 0 and r0["num_samples"] == 0 and r0["n_steps"] == 0
