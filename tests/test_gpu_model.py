"""Operator matrices built on the GPU (te_model_create_device) against the host
builder (the reference's Basis/createMatrix restated in C++; needs a GB300):
same basis order, same entries bit for bit, same 1-norm, same evolutions."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _csr_of_coo(n, coo):
    row, col, val = coo
    rp = np.zeros(n + 1, dtype=np.int64)
    np.add.at(rp, np.asarray(row, dtype=np.int64) + 1, 1)
    return np.cumsum(rp), np.asarray(col, dtype=np.int64), np.asarray(val, dtype=np.complex128)


@pytest.mark.parametrize("L,N", [(4, 4), (6, 6), (8, 8), (10, 10), (7, 3), (3, 9)])
def test_bose_hubbard_device_equals_host(te_gpu, L, N):
    from timeevolver_gb300 import models
    B, coo = models.bose_hubbard(L, N, 1.0, 2.0)
    Hd, dim = models.bose_hubbard_device(L, N, 1.0, 2.0)
    assert dim == B.size
    rp, ci, val = Hd.to_csr()
    rp0, ci0, val0 = _csr_of_coo(dim, coo)
    assert np.array_equal(rp, rp0) and np.array_equal(ci, ci0)
    assert np.array_equal(val, val0)  # bit for bit
    Hh = te_gpu.Matrix.from_coo(dim, coo)
    assert Hd.info()["norm1"] == Hh.info()["norm1"]  # the reference's 1-norm, bit for bit
    assert Hd.info()["real"]


def test_general_terms_and_quant(te_gpu):
    """Per-bond couplings, a chemical potential, a complex hopping phase and a
    basis of pairs (quant = 2)."""
    from timeevolver_gb300 import models
    L, N = 5, 8
    terms = models.bose_hubbard_terms(L, [0.9, 1.1, 1.0, 0.8], 1.5, mu=0.3)
    terms.append(models.lin_interaction(0, 2, 0, 0, False, 0.25j))
    terms.append(models.lin_interaction(0, 2, 0, 0, True, -0.25j))
    for quant in (1, 2):
        B = models.Basis(N, L, 0, 0, quant)
        coo = models.operator_matrix(terms, B)
        Hd, dim = te_gpu.Matrix.from_terms_device(N, L, terms, quant=quant)
        assert dim == B.size
        rp, ci, val = Hd.to_csr()
        rp0, ci0, val0 = _csr_of_coo(dim, coo)
        assert np.array_equal(rp, rp0) and np.array_equal(ci, ci0)
        assert np.max(np.abs(val - val0)) <= 1e-15 * np.max(np.abs(val0))
        H = np.zeros((dim, dim), dtype=complex)
        np.add.at(H, (rp_rows(rp), ci), val)
        assert np.max(np.abs(H - H.conj().T)) < 1e-14  # Hermitian term list


def rp_rows(rp):
    return np.repeat(np.arange(len(rp) - 1), np.diff(rp))


def test_state_index(te_gpu):
    from timeevolver_gb300 import models
    L, N = 6, 6
    B = models.Basis(N, L, 0, 0)
    el = B.elements()
    rng = np.random.default_rng(3)
    for i in rng.integers(0, B.size, size=40):
        assert te_gpu.state_index_device(N, el[i]) == i
    assert te_gpu.state_index_device(N, [N - 1] + [0] * (L - 1)) == -1  # wrong particle number


def test_device_built_evolution(te_gpu):
    """The same evolution from the device- and the host-built matrices."""
    from timeevolver_gb300 import models
    L = N = 8
    B, coo = models.bose_hubbard(L, N, 1.0, 2.0)
    Hd, dim = models.bose_hubbard_device(L, N, 1.0, 2.0)
    v = np.zeros(dim, dtype=np.complex128)
    v[te_gpu.state_index_device(N, [N] + [0] * (L - 1))] = 1.0
    n0 = models.operator_matrix([models.number_operator(0, 1.0)], B)
    a = te_gpu.evolve(Hd, v, 5.0, 0.5, [("sparse", n0)], tol=1e-8, m=40)
    b = te_gpu.evolve(coo, v, 5.0, 0.5, [("sparse", n0)], tol=1e-8, m=40)
    assert a["n_steps"] == b["n_steps"] and a["status"] == b["status"]
    assert np.array_equal(a["samples"], b["samples"]) and np.array_equal(a["state"], b["state"])


def _device_equals_host(te_gpu, desc, host_basis, terms):
    from timeevolver_gb300 import models
    coo = models.operator_matrix(terms, host_basis)
    Hd, dim = te_gpu.Matrix.from_terms_device_basis(desc, terms)
    assert dim == host_basis.size
    rp, ci, val = Hd.to_csr()
    rp0, ci0, val0 = _csr_of_coo(dim, coo)
    assert np.array_equal(rp, rp0) and np.array_equal(ci, ci0)
    assert np.array_equal(val, val0)  # bit for bit
    assert Hd.info()["norm1"] == te_gpu.Matrix.from_coo(dim, coo).info()["norm1"]
    el = host_basis.elements()
    rng = np.random.default_rng(7)
    for i in rng.integers(0, dim, size=25):
        assert te_gpu.basis_index_device(desc, el[i]) == i
    return Hd, dim, coo


@pytest.mark.parametrize("N,K,nq,cap,quant", [(6, 5, 2, 2, 1), (8, 4, 4, 3, 1), (5, 5, 5, 1, 1), (7, 6, 3, 1, 1),
                                              (9, 5, 2, 4, 2), (10, 3, 3, 4, 2)])
def test_qudit_basis_device_equals_host(te_gpu, N, K, nq, cap, quant):
    """basis(N, K, nbQudits, capacity, quant) on the GPU: the last nbQudits
    modes capped, and with every mode a qudit the states whose mode 0 would
    exceed the capacity dropped; hopping terms with capacities on the
    creation operators, on-site terms.  Entries, 1-norm and indices equal the
    host builder's."""
    from timeevolver_gb300 import models
    terms = []
    for b in range(K - 1):
        terms.append((complex(-0.7 - 0.1 * b), [-1, 1], [b + 1, b], [0, cap if b >= K - nq else 0]))
        terms.append((complex(-0.7 - 0.1 * b), [-1, 1], [b, b + 1], [0, cap if b + 1 >= K - nq else 0]))
    for i in range(K):
        terms.append(models.four_point_a(i, i, i, i, 0, 0, 0, 0, 0.8))
        terms.append(models.number_operator(i, 0.3 * i - 0.8))
    B = models.Basis(N, K, nq, cap, quant)
    _device_equals_host(te_gpu, te_gpu.basis_desc(N, K, nq, cap, quant), B, terms)
    # states outside the capacity are not basis states
    occ = [0] * K
    occ[K - 1] = cap + 1
    occ[0] = N - cap - 1
    if occ[0] >= 0:
        assert te_gpu.basis_index_device(te_gpu.basis_desc(N, K, nq, cap, quant), occ) == -1


def test_tensor_basis_black_hole_device_golden(te_gpu, oracle_lib):
    """The black-hole model of the reference's example on tensorBasis(20, 2,
    2, 8, 1) (dim 588, 74 terms) built on the GPU: the matrix equals the host
    builder's bit for bit, and its evolution reproduces the reference's golden
    trajectories (output/ResultBlackHole_N20_...h5)."""
    import os
    from oracle import models as omodels
    from timeevolver_gb300 import models
    terms = omodels.black_hole_terms(20, 2, 12.0, 4)
    assert len(terms) > 64
    B = models.Basis.tensor(20, 2, 2, 8, 1)
    desc = te_gpu.basis_desc(0, 0, tensor=(20, 2, 2, 8, 1))
    Hd, dim, coo = _device_equals_host(te_gpu, desc, B, terms)
    assert dim == 588
    init = [20, 0, 1, 1] + [0] * 6
    v = np.zeros(dim, dtype=np.complex128)
    v[te_gpu.basis_index_device(desc, init)] = 1.0
    obs = [("sparse", o) for o in models.number_operator_observables(B)]
    r = te_gpu.evolve(Hd, v, 10.0, 0.01, obs, tol=1e-8, m=40)
    gold = np.load(os.path.join(os.path.dirname(__file__), "golden", "blackhole_N20.npy"))
    assert r["num_samples"] == 1001 and r["err"] <= 1e-8
    assert np.max(np.abs(r["samples"] - gold)) < 1e-8
    # an empty second set is rejected, as are inconsistent descriptors
    with pytest.raises(te_gpu.TeError):
        te_gpu.Matrix.from_terms_device_basis(te_gpu.basis_desc(0, 0, tensor=(2, 2, 5, 2, 1)), terms[:4])
    with pytest.raises(te_gpu.TeError):
        te_gpu.Matrix.from_terms_device_basis(te_gpu.basis_desc(4, 3, 4, 1, 1), terms[:2])
