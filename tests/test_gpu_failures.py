"""Failure paths of the evolution (needs a GB300), each made on purpose
without faulting the GPU:

* a grid-barrier wait of the persistent Lanczos kernel that runs out (every
  barrier waits for one arrival more than the grid has, with a short poll
  limit): the run returns TE_ERR_DEVICE_TIMEOUT and the same evolver then
  runs correctly;
* NaN or Inf in H, rejected at upload; a NaN in v, rejected as not normalized;
* a tolerance no step size can meet (Krylov dimension 2, tol 1e-12): 20
  halvings, then TE_ERR_NO_STEP where the reference exits
  (krylovTimeEvolver.cpp:198-209);
* a tanh-sinh rule capped at level 2, so that the quadrature misses its
  accuracy: code 20 on the same steps as the oracle with the same cap
  (krylovTimeEvolver.cpp:584-618);
* exp(-ixT) for arguments beyond the Chebyshev-Bessel series, through the
  tridiagonal QR eigensolve: its eigenvalues against scipy's, the evolution
  against the oracle and the exact exponential; with the QR capped at one
  sweep it reports TE_ERR_EIGEN (the LAPACK failure of zhseqr,
  matrixDataTypes.h:135-156).
"""
import numpy as np
import pytest

from oracle import models

pytestmark = pytest.mark.gpu

TE_ERR_INVALID_ARG, TE_ERR_NOT_NORMALIZED, TE_ERR_NO_STEP, TE_ERR_EIGEN, TE_ERR_DEVICE_TIMEOUT = -1, -4, -5, -6, -10


def _fock(states, occ):
    v = np.zeros(len(states), dtype=np.complex128)
    v[models.index_of(states, occ)] = 1.0
    return v


def _run(te, ev):
    """time_evolve, returning (result, None) or (None, error code)."""
    try:
        return ev.time_evolve(trace=True), None
    except te.TeError as e:
        return None, e.code


def test_barrier_timeout_returns_error_and_evolver_recovers(te_gpu, oracle_lib):
    states, H = models.bose_hubbard(8, 8, 1.0, 2.0)
    v = _fock(states, [8] + [0] * 7)
    M = te_gpu.Matrix.from_coo(len(states), H)
    ev = te_gpu.Evolver(M, v, 2.0, 0.5, [], tol=1e-8, m=40)
    ev.set_option(te_gpu.OPT_FUSED_LANCZOS, 2)  # the persistent kernel, whose barriers are under test
    ev.set_option(te_gpu.OPT_BARRIER_SPIN_LIMIT, 1 << 14)  # ~10 ms of polling per wait
    ev.set_option(te_gpu.OPT_BARRIER_EXTRA_ARRIVALS, 1)
    import time
    t0 = time.perf_counter()
    out, code = _run(te_gpu, ev)
    assert out is None and code == TE_ERR_DEVICE_TIMEOUT
    assert time.perf_counter() - t0 < 5.0
    assert "barrier" in te_gpu.lib().te_last_error().decode()
    # the context is intact: the same evolver, reset, runs to the oracle's result
    ev.set_option(te_gpu.OPT_BARRIER_EXTRA_ARRIVALS, 0)
    ev.reset(v)
    out, code = _run(te_gpu, ev)
    assert code is None
    ref = oracle_lib.evolve(H, v, 2.0, 0.5, [], tol=1e-8, m=40)
    assert out["n_steps"] == ref["n_steps"] and out["status"] == ref["status"]
    assert np.linalg.norm(out["state"] - ref["state"]) < 2e-8
    ev.close()
    # invalid option values are refused
    ev2 = te_gpu.Evolver(M, v, 2.0, 0.5, [], tol=1e-8, m=40)
    for opt, val in [(te_gpu.OPT_BARRIER_SPIN_LIMIT, 0), (te_gpu.OPT_BARRIER_EXTRA_ARRIVALS, 2),
                     (te_gpu.OPT_TS_MAX_LEVEL, 1), (te_gpu.OPT_TS_MAX_LEVEL, 9), (te_gpu.OPT_QR_SWEEP_LIMIT, -1)]:
        with pytest.raises(te_gpu.TeError) as e:
            ev2.set_option(opt, val)
        assert e.value.code == TE_ERR_INVALID_ARG
    ev2.close()


@pytest.mark.parametrize("bad", [np.nan, np.inf, -np.inf])
@pytest.mark.parametrize("path", ["host", "device"])
def test_nonfinite_matrix_rejected(te_gpu, bad, path):
    states, H = models.bose_hubbard(6 if path == "host" else 10, 6 if path == "host" else 10, 1.0, 2.0)
    row, col, val = H
    val = val.copy()
    val[len(val) // 3] = bad
    assert (path == "device") == (len(val) >= 1 << 18)  # the row-sorted COO of >= 2^18 entries converts on the GPU
    with pytest.raises(te_gpu.TeError) as e:
        te_gpu.Matrix(len(states), row, col, val)
    assert e.value.code == TE_ERR_INVALID_ARG
    assert "not finite" in str(e.value)


def test_nonfinite_csr_rejected(te_gpu):
    import torch
    rp = torch.tensor([0, 1, 2], dtype=torch.int32, device="cuda")
    ci = torch.tensor([0, 1], dtype=torch.int32, device="cuda")
    vals = torch.tensor([1.0, float("nan")], dtype=torch.float64, device="cuda")
    with pytest.raises(te_gpu.TeError) as e:
        te_gpu.Matrix.from_device_csr(2, rp, ci, vals)
    assert e.value.code == TE_ERR_INVALID_ARG
    with pytest.raises(te_gpu.TeError) as e:
        te_gpu.Matrix.from_csr(2, [0, 1, 2], [0, 1], np.array([1.0, np.inf], dtype=np.complex128))
    assert e.value.code == TE_ERR_INVALID_ARG


def test_nan_start_vector_rejected(te_gpu):
    states, H = models.bose_hubbard(5, 5, 1.0, 2.0)
    M = te_gpu.Matrix.from_coo(len(states), H)
    v = _fock(states, [5, 0, 0, 0, 0])
    v[3] = np.nan
    with pytest.raises(te_gpu.TeError) as e:
        te_gpu.Evolver(M, v, 1.0, 0.5, [], tol=1e-8, m=20)
    assert e.value.code == TE_ERR_NOT_NORMALIZED


def test_normalisation_check_large_vector(te_gpu):
    """The start vector's normalisation check (krylovTimeEvolver.cpp:45-48) on a
    vector long enough for the multi-threaded sum (2^21 values and more): a
    norm 2 tol away from 1 is rejected, one tol/2 away is accepted, as is a
    NaN anywhere; the same for te_evolver_reset."""
    n = 1 << 20  # 2^21 doubles
    rows = np.arange(n, dtype=np.int64)
    M = te_gpu.Matrix.from_coo(n, (rows, rows, np.ones(n, dtype=np.complex128)))
    rng = np.random.default_rng(11)
    v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    v /= np.linalg.norm(v)
    tol = 1e-8
    ev = te_gpu.Evolver(M, v * (1.0 + 0.5 * tol), 0.1, 0.1, [], tol=tol, m=10)
    try:
        with pytest.raises(te_gpu.TeError) as e:
            ev.reset(v * (1.0 + 2.0 * tol))
        assert e.value.code == TE_ERR_NOT_NORMALIZED
        bad = v.copy()
        bad[n - 3] = np.nan
        with pytest.raises(te_gpu.TeError) as e:
            ev.reset(bad)
        assert e.value.code == TE_ERR_NOT_NORMALIZED
    finally:
        ev.close()
    with pytest.raises(te_gpu.TeError) as e:
        te_gpu.Evolver(M, v * (1.0 + 2.0 * tol), 0.1, 0.1, [], tol=tol, m=10)
    assert e.value.code == TE_ERR_NOT_NORMALIZED
    M.close()


def test_unreachable_tolerance_no_step(te_gpu, oracle_lib):
    """Krylov dimension 2 at tol 1e-12: each halving lowers the error per unit
    time by only 2, so 20 halvings cannot meet the tolerance rate."""
    states, H = models.bose_hubbard(6, 6, 1.0, 2.0)
    v = _fock(states, [6, 0, 0, 0, 0, 0])
    with pytest.raises(RuntimeError, match="code -3"):
        oracle_lib.evolve(H, v, 1.0, 0.5, [], tol=1e-12, m=2)
    M = te_gpu.Matrix.from_coo(len(states), H)
    ev = te_gpu.Evolver(M, v, 1.0, 0.5, [], tol=1e-12, m=2)
    out, code = _run(te_gpu, ev)
    assert out is None and code == TE_ERR_NO_STEP
    assert "no small enough time step" in te_gpu.lib().te_last_error().decode()
    ev.close()


def test_quadrature_failure_status_20(te_gpu, oracle_lib):
    states, H = models.bose_hubbard(8, 8, 1.0, 2.0)
    v = _fock(states, [8] + [0] * 7)
    obs = [("sparse", o) for o in models.number_operator_observables(states)[:2]]
    oracle_lib.set_ts_max_level(2)
    try:
        ref = oracle_lib.evolve(H, v, 2.0, 0.5, obs, tol=1e-8, m=40, trace=True)
    finally:
        oracle_lib.set_ts_max_level(8)
    assert ref["status"] == 20 and ref["nb_err_int"] >= 1
    M = te_gpu.Matrix.from_coo(len(states), H)
    ev = te_gpu.Evolver(M, v, 2.0, 0.5, [("sparse", te_gpu.Matrix.from_coo(len(states), o)) for _, o in obs],
                        tol=1e-8, m=40)
    ev.set_option(te_gpu.OPT_TS_MAX_LEVEL, 2)
    out, code = _run(te_gpu, ev)
    assert code is None
    assert out["status"] == ref["status"] and out["nb_err_int"] == ref["nb_err_int"]
    assert out["n_steps"] == ref["n_steps"]
    assert [s["code"] for s in out["trace"]] == [s["code"] for s in ref["trace"]]
    for a, b in zip(out["trace"], ref["trace"]):
        assert abs(a["t_step"] - b["t_step"]) <= 1e-12 * b["t_step"]
    # free-running three-term recurrence: observables within the bound 4 tol ||O||
    assert np.max(np.abs(out["samples"] - ref["samples"])) < 4 * 1e-8 * 8.0
    ev.close()


def _detuned_chain(n=41, detuning=1000.0, split=20):
    """Hopping 1 along a chain of n sites, on-site energy `detuning` from site
    `split` on.  Lanczos from site 0 reproduces the chain as T; the amplitude
    that reaches the last Krylov vector is ~detuning^-(n - split), so the error
    bound stays negligible and the first step doubles to the whole interval,
    where x * ||T|| is far beyond the Chebyshev-Bessel series."""
    rows, cols, vals = [], [], []
    for i in range(n):
        if i > 0:
            rows.append(i), cols.append(i - 1), vals.append(1.0)
        if i >= split:
            rows.append(i), cols.append(i), vals.append(detuning)
        if i < n - 1:
            rows.append(i), cols.append(i + 1), vals.append(1.0)
    H = (np.array(rows, dtype=np.int64), np.array(cols, dtype=np.int64), np.array(vals, dtype=np.complex128))
    dense = np.zeros((n, n))
    for r, c, x in zip(*H):
        dense[r, c] = x.real
    return H, dense


def test_eigen_fallback_matches_scipy_and_oracle(te_gpu, oracle_lib):
    import scipy.linalg as sl
    H, dense = _detuned_chain()
    n = dense.shape[0]
    v = np.zeros(n, dtype=np.complex128)
    v[0] = 1.0
    e0 = v.copy()
    t, tol = 100.0, 1e-6
    M = te_gpu.Matrix.from_coo(n, H)
    ev = te_gpu.Evolver(M, v, t, 10.0, [("vector", e0)], tol=tol, m=40)
    out, code = _run(te_gpu, ev)
    assert code is None
    km = ev.krylov_matrix()
    assert km["eig_used"], "the step should have evaluated exp(-ixT) through the eigen-decomposition"
    lam_ref = sl.eigh_tridiagonal(km["diag"], km["offdiag"], eigvals_only=True)
    scale = np.max(np.abs(lam_ref))
    assert np.max(np.abs(np.sort(km["eigenvalues"]) - lam_ref)) <= 1e-12 * scale
    # T is the chain itself (up to the signs of the off-diagonal)
    assert np.max(np.abs(km["diag"] - np.diag(dense)[:40])) <= 1e-12 * scale
    assert np.max(np.abs(np.abs(km["offdiag"]) - 1.0)) <= 1e-12
    ref = oracle_lib.evolve(H, v, t, 10.0, [("vector", e0)], tol=tol, m=40, trace=True)
    assert out["n_steps"] == ref["n_steps"] == 1 and out["status"] == ref["status"]
    assert out["num_samples"] == ref["num_samples"] == 11
    assert np.max(np.abs(out["samples"] - ref["samples"])) < 1e-9
    assert np.linalg.norm(out["state"] - ref["state"]) < 2 * tol
    exact = sl.expm(-1j * t * dense) @ v
    assert np.linalg.norm(out["state"] - exact) < tol
    ev.close()


def test_eigen_failure_surfaces(te_gpu):
    H, dense = _detuned_chain()
    n = dense.shape[0]
    v = np.zeros(n, dtype=np.complex128)
    v[0] = 1.0
    M = te_gpu.Matrix.from_coo(n, H)
    ev = te_gpu.Evolver(M, v, 100.0, 10.0, [], tol=1e-6, m=40)
    ev.set_option(te_gpu.OPT_QR_SWEEP_LIMIT, 1)
    out, code = _run(te_gpu, ev)
    assert out is None and code == TE_ERR_EIGEN
    assert "eigensolver" in te_gpu.lib().te_last_error().decode()
    # with the default limit the same evolver runs through
    ev.set_option(te_gpu.OPT_QR_SWEEP_LIMIT, 0)
    ev.reset(v)
    out, code = _run(te_gpu, ev)
    assert code is None and out["n_steps"] == 1
    ev.close()
