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
