"""The load-imbalanced synthetic workload (needs a GB300): the device
generator against its plain-Python restatement, and evolutions of the
generated complex Hermitian matrix against the CPU oracle.

Evolution tolerances follow test_gpu_parity: the free-running three-term
recurrence agrees with the oracle to the Krylov truncation error (final
states within 2 tol, observables within 4 tol ||O||); the reorthogonalising
mode, which is insensitive to rounding, to 1e-11.
"""
import numpy as np
import pytest

import synth_zipf

pytestmark = pytest.mark.gpu

N_SMALL = 4096
SEED = 7


@pytest.fixture(scope="module")
def zipf_small(te_gpu):
    H, est = te_gpu.Matrix.zipf(N_SMALL, 1.5, 2, 256, SEED, 20)
    return H, est


@pytest.fixture(scope="module")
def restated():
    return synth_zipf.generate(N_SMALL, 1.5, 2, 256, SEED, 20)


def test_generator_matches_restatement(zipf_small, restated):
    H, est = zipf_small
    rp, ci, val = H.to_csr()
    rp0, ci0, val0, est0 = restated
    assert np.array_equal(rp.astype(np.int64), rp0)
    assert np.array_equal(ci.astype(np.int64), ci0)
    assert abs(est - est0) <= 1e-10 * est0
    assert np.max(np.abs(val - val0)) <= 1e-12 * np.max(np.abs(val0))
    info = H.info()
    assert not info["real"] and info["nnz"] == len(ci0)


def test_generated_matrix_is_hermitian(zipf_small):
    import scipy.sparse as sp
    H, _ = zipf_small
    rp, ci, val = H.to_csr()
    A = sp.csr_matrix((val, ci, rp), shape=(N_SMALL, N_SMALL))
    assert abs(A - A.getH()).max() == 0.0
    # columns ascend within every row
    for r in range(0, N_SMALL, 97):
        assert np.all(np.diff(ci[rp[r]:rp[r + 1]]) > 0)


def test_norm1_fixed_point_matches_column_sums(zipf_small):
    H, _ = zipf_small
    rp, ci, val = H.to_csr()
    colsum = np.zeros(N_SMALL)
    np.add.at(colsum, ci, np.abs(val))
    assert abs(H.info()["norm1"] - colsum.max()) <= 1e-11 * colsum.max()


def test_device_csr_upload_roundtrip(te_gpu, zipf_small):
    torch = pytest.importorskip("torch")
    H, _ = zipf_small
    rp, ci, val = H.to_csr()
    M = te_gpu.Matrix.from_device_csr(N_SMALL, torch.tensor(rp, device="cuda"), torch.tensor(ci, device="cuda"),
                                      torch.tensor(val, device="cuda"))
    rp2, ci2, val2 = M.to_csr()
    assert np.array_equal(rp, rp2) and np.array_equal(ci, ci2) and np.array_equal(val, val2)
    x = np.random.default_rng(3).standard_normal(N_SMALL) + 0j
    assert np.allclose(M.spmv(x), H.spmv(x), rtol=0, atol=1e-13)


def test_spmv_matches_scipy(zipf_small):
    import scipy.sparse as sp
    H, _ = zipf_small
    rp, ci, val = H.to_csr()
    A = sp.csr_matrix((val, ci, rp), shape=(N_SMALL, N_SMALL))
    rng = np.random.default_rng(5)
    x = rng.standard_normal(N_SMALL) + 1j * rng.standard_normal(N_SMALL)
    y = H.spmv(x, alpha=-1j)
    assert np.max(np.abs(y - (-1j) * (A @ x))) <= 1e-13 * np.max(np.abs(y))


def _state(n, seed):
    rng = np.random.default_rng(seed)
    v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    return v / np.linalg.norm(v)


def _diag_observable(n, seed):
    d = np.random.default_rng(seed).uniform(-1.0, 1.0, n)
    return (np.arange(n), np.arange(n), d.astype(np.complex128)), np.max(np.abs(d))


@pytest.mark.parametrize("reorth", [False, True])
def test_evolution_matches_oracle(te_gpu, oracle_lib, zipf_small, reorth):
    H, _ = zipf_small
    coo = H.to_coo()
    v = _state(N_SMALL, 11)
    O, o_norm = _diag_observable(N_SMALL, 12)
    t, ss, tol = 8.0, 1.0, 1e-8
    gpu = te_gpu.evolve(H, v, t, ss, [("sparse", O)], tol=tol, m=40, reorth=reorth)
    ref = oracle_lib.evolve(coo, v, t, ss, [("sparse", O)], tol=tol, m=40, reorth=reorth)
    assert gpu["status"] == ref["status"]
    assert gpu["n_steps"] == ref["n_steps"]
    assert gpu["num_samples"] == ref["num_samples"] == 9
    assert gpu["err"] <= tol and ref["err"] <= tol
    if reorth:
        assert np.max(np.abs(gpu["samples"] - ref["samples"])) < 1e-11
        assert np.linalg.norm(gpu["state"] - ref["state"]) < 1e-11
    else:
        assert np.max(np.abs(gpu["samples"] - ref["samples"])) <= 4 * tol * o_norm
        assert np.linalg.norm(gpu["state"] - ref["state"]) <= 2 * tol


def test_time_reversal_large(te_gpu):
    """exp(+iHt) exp(-iHt) v = v on a 2e6-dimensional generated matrix."""
    n = 2_000_000
    H, _ = te_gpu.Matrix.zipf(n, 1.5, 2, 256, 1, 30)
    v = _state(n, 1)
    t, tol = 20.0, 1e-8
    fwd = te_gpu.evolve(H, v, t, t, [], tol=tol, m=40)
    assert fwd["err"] <= tol
    back = te_gpu.evolve(H, fwd["state"], t, t, [], exp_factor=-1.0, tol=tol, m=40)
    assert back["err"] <= tol
    assert abs(np.linalg.norm(fwd["state"]) - 1.0) < 1e-12
    assert np.linalg.norm(back["state"] - v) <= 2 * tol
