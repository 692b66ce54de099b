"""CUDA path against the oracle and the reference goldens (needs a GB300).

Tolerances.  Sparse products agree to 1e-13 relative.  A free-running
evolution uses the reference's three-term Lanczos recurrence without
reorthogonalisation; once the Krylov basis loses orthogonality its last
coefficients amplify rounding, so two correct FP64 runs (CPU oracle, GPU)
agree only to the Krylov truncation error, which the a-posteriori bound
controls: both final states lie within tol of the exact state, hence within
2*tol of each other, and a sampled observable O differs by at most
4*tol*||O||.  The tests assert these bounds, the same step count, status and
sample count, an error bound <= tol, and the 1e-9 absolute observable
agreement wherever the recurrence stays stable (small Krylov spaces, the
goldens).
"""
import os

import numpy as np
import pytest

from oracle import models

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
OBS_TOL = 1e-9


def _fock(states, occ):
    v = np.zeros(len(states), dtype=np.complex128)
    v[models.index_of(states, occ)] = 1.0
    return v


def _random_state(n, seed):
    rng = np.random.default_rng(seed)
    v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    return v / np.linalg.norm(v)


def _random_hermitian(n, per_row, seed):
    rng = np.random.default_rng(seed)
    rows = np.repeat(np.arange(n), per_row)
    cols = rng.integers(0, n, size=n * per_row)
    vals = rng.standard_normal(n * per_row) + 1j * rng.standard_normal(n * per_row)
    A = {}
    for r, c, v in zip(rows, cols, vals):
        A[(r, c)] = A.get((r, c), 0) + v / 2
        A[(c, r)] = A.get((c, r), 0) + np.conj(v) / 2
    keys = sorted(A)
    row = np.array([k[0] for k in keys], dtype=np.int64)
    col = np.array([k[1] for k in keys], dtype=np.int64)
    val = np.array([A[k] for k in keys], dtype=np.complex128)
    return row, col, val


def _compare(gpu, ref, tol, obs_norm=None, strict=True):
    """strict: observables to 1e-9 absolute; otherwise to 4 tol ||O||."""
    assert gpu["status"] == ref["status"], (gpu["status"], ref["status"])
    assert gpu["num_samples"] == ref["num_samples"]
    assert gpu["n_steps"] == ref["n_steps"], (gpu["n_steps"], ref["n_steps"])
    assert gpu["krylov_dim"] == ref["krylov_dim"]
    d_obs = np.max(np.abs(gpu["samples"] - ref["samples"])) if gpu["samples"].size else 0.0
    bound = OBS_TOL if strict else max(OBS_TOL, 4 * tol * obs_norm)
    assert d_obs < bound, (d_obs, bound)
    assert np.linalg.norm(gpu["state"] - ref["state"]) < 2 * tol
    assert gpu["err"] <= tol and ref["err"] <= tol
    assert abs(gpu["evolved_time"] - ref["evolved_time"]) < 1e-12 * max(1.0, ref["evolved_time"])
    return d_obs


def test_spmv_real_and_complex(te_gpu, oracle_lib):
    states, H = models.bose_hubbard(7, 6, 1.0, 2.0)
    n = len(states)
    x = _random_state(n, 1)
    for coo, alpha in [(H, -0.75j), (_random_hermitian(3000, 9, 2), 0.3 - 1.1j)]:
        nn = int(coo[0].max()) + 1 if coo is not H else n
        xx = x if coo is H else _random_state(nn, 4)
        M = te_gpu.Matrix.from_coo(nn, coo)
        info = M.info()
        assert info["real"] == (coo is H)
        y = M.spmv(xx, alpha)
        ref = oracle_lib.spmv(coo, xx, alpha)
        assert np.linalg.norm(y - ref) <= 1e-13 * np.linalg.norm(ref)
        assert abs(info["norm1"] - oracle_lib.norm1(coo, nn)) <= 1e-12 * info["norm1"]


def test_bose_hubbard_l8_matches_oracle(te_gpu, oracle_lib):
    """Plain method, small: L=8 N=8 (dim 6435), t=10, tol 1e-8, m=40, <n_i> every 0.1."""
    states, H = models.bose_hubbard(8, 8, 1.0, 2.0)
    v = _fock(states, [8] + [0] * 7)
    obs = [("sparse", o) for o in models.number_operator_observables(states)]
    gpu = te_gpu.evolve(H, v, 10.0, 0.1, obs, tol=1e-8, m=40, trace=True)
    ref = oracle_lib.evolve(H, v, 10.0, 0.1, obs, tol=1e-8, m=40, trace=True)
    _compare(gpu, ref, 1e-8, obs_norm=8.0, strict=False)
    for a, b in zip(gpu["trace"], ref["trace"]):
        assert abs(a["t_step"] - b["t_step"]) <= 1e-12 * b["t_step"]
        assert a["code"] == b["code"]
    assert gpu["launches"] > 0


def test_bose_hubbard_l12_matches_oracle(te_gpu, oracle_lib):
    """Plain method, large: L=12 N=12 U=3 (dim 1352078), random complex v
    (seed 0), tol 1e-8, m=40, <n_0> every 0.5; the first Krylov steps (t=1)."""
    states, H = models.bose_hubbard(12, 12, 1.0, 3.0)
    n = len(states)
    v = _random_state(n, 0)
    obs = [("sparse", models.create_matrix([models.number_operator(0, 1.0)], states))]
    gpu = te_gpu.evolve(H, v, 1.0, 0.5, obs, tol=1e-8, m=40, trace=True)
    ref = oracle_lib.evolve(H, v, 1.0, 0.5, obs, tol=1e-8, m=40, trace=True)
    _compare(gpu, ref, 1e-8, obs_norm=12.0, strict=True)
    for a, b in zip(gpu["trace"], ref["trace"]):
        assert abs(a["t_step"] - b["t_step"]) <= 1e-12 * b["t_step"]


def test_golden_black_hole_n20(te_gpu):
    states, H, i0 = models.black_hole(N0=20, Nm=2, K=4)
    v = np.zeros(len(states), dtype=np.complex128)
    v[i0] = 1
    obs = [("sparse", o) for o in models.number_operator_observables(states)]
    r = te_gpu.evolve(H, v, 10.0, 0.01, obs, tol=1e-8, m=40)
    gold = np.load(os.path.join(GOLD, "blackhole_N20.npy"))
    assert r["num_samples"] == 1001
    assert np.max(np.abs(r["samples"] - gold)) < 1e-8
    assert r["err"] <= 1e-8


def test_golden_lucky_breakdown(te_gpu, oracle_lib):
    states, H, i0 = models.black_hole(N0=1, Nm=1, K=1)
    v = np.zeros(4, dtype=np.complex128)
    v[i0] = 1
    obs = [("sparse", o) for o in models.number_operator_observables(states)]
    r = te_gpu.evolve(H, v, 1000.0, 1.0, obs, tol=1e-8, m=40)
    gold = np.load(os.path.join(GOLD, "blackhole_N1_LB.npy"))
    assert r["status"] == 1 and r["krylov_dim"] == 4 and r["n_steps"] == 1
    assert np.max(np.abs(r["samples"] - gold)) < 1e-8
    ref = oracle_lib.evolve(H, v, 1000.0, 1.0, obs, tol=1e-8, m=40)
    _compare(r, ref, 1e-8)


def test_golden_simple_example(te_gpu, oracle_lib):
    states, H, i0 = models.simple_example()
    v = np.zeros(len(states), dtype=np.complex128)
    v[i0] = 1
    obs = [("sparse", o) for o in models.number_operator_observables(states)]
    r = te_gpu.evolve(H, v, 10.0, 0.01, obs, tol=1e-6, m=40)
    gold = np.load(os.path.join(GOLD, "simple_example.npy"))
    assert np.max(np.abs(r["samples"] - gold)) <= 6e-4  # 6 significant digits of values up to 200
    ref = oracle_lib.evolve(H, v, 10.0, 0.01, obs, tol=1e-6, m=40)
    _compare(r, ref, 1e-6)


def test_complex_matrix_random_state(te_gpu, oracle_lib):
    H = _random_hermitian(2000, 6, 7)
    n = 2000
    v = _random_state(n, 8)
    o = np.zeros(n, dtype=np.complex128)
    o[:10] = 0.3
    diag = (np.arange(n, dtype=np.int64), np.arange(n, dtype=np.int64), np.linspace(0, 1, n).astype(complex))
    obs = [("sparse", diag), ("vector", o)]
    gpu = te_gpu.evolve(H, v, 2.0, 0.25, obs, exp_factor=0.7, tol=1e-9, m=30)
    ref = oracle_lib.evolve(H, v, 2.0, 0.25, obs, exp_factor=0.7, tol=1e-9, m=30)
    _compare(gpu, ref, 1e-9)


def test_fast_integration(te_gpu, oracle_lib):
    states, H = models.bose_hubbard(6, 6, 1.0, 3.0)
    v = _random_state(len(states), 0)
    obs = [("sparse", models.create_matrix([models.number_operator(0, 1.0)], states))]
    gpu = te_gpu.evolve(H, v, 3.0, 0.5, obs, tol=1e-8, m=40, fast_integration=True)
    ref = oracle_lib.evolve(H, v, 3.0, 0.5, obs, tol=1e-8, m=40, fast_integration=True)
    _compare(gpu, ref, 1e-8)


def test_general_sparse_and_callback_observables(te_gpu, oracle_lib):
    states, H = models.bose_hubbard(5, 5, 1.0, 2.0)
    n = len(states)
    v = _fock(states, [5, 0, 0, 0, 0])
    hop = models.create_matrix([models.lin_interaction(0, 1, 0, 0, False, 1.0),
                                models.lin_interaction(0, 1, 0, 0, True, 1.0)], states)
    seen = []

    def cb(state):
        seen.append(np.vdot(state, state).real)
        return float(np.abs(state[0]) ** 2)

    gpu = te_gpu.evolve(H, v, 1.0, 0.1, [("sparse", hop), ("callback", cb)], tol=1e-8, m=20)
    ref = oracle_lib.evolve(H, v, 1.0, 0.1, [("sparse", hop)], tol=1e-8, m=20)
    assert np.max(np.abs(gpu["samples"][0] - ref["samples"][0])) < OBS_TOL
    assert len(seen) == 11 and np.allclose(seen, 1.0, atol=1e-8)
    i0 = models.index_of(states, [5, 0, 0, 0, 0])
    assert abs(gpu["samples"][1][0] - 1.0) < 1e-12


def test_stop_request(te_gpu, oracle_lib):
    states, H = models.bose_hubbard(4, 4, 1.0, 2.0)
    n = len(states)
    v = np.zeros(n, dtype=np.complex128)
    v[0] = 1
    calls = []

    def stopper(state):
        calls.append(1)
        if len(calls) == 6:
            raise te_gpu.StopEvolution()
        return 0.0

    obs = [("sparse", o) for o in models.number_operator_observables(states)]
    gpu = te_gpu.evolve(H, v, 2.0, 0.1, obs + [("callback", stopper)], tol=1e-8, m=20)
    ref = oracle_lib.evolve(H, v, 2.0, 0.1, obs + [("stop", 5)], tol=1e-8, m=20)
    assert gpu["status"] == ref["status"] == 3
    assert gpu["num_samples"] == ref["num_samples"] == 5
    assert abs(gpu["evolved_time"] - ref["evolved_time"]) < 1e-12
    assert np.max(np.abs(gpu["samples"][:4, :5] - ref["samples"][:, :5])) < OBS_TOL


def test_invalid_inputs(te_gpu):
    states, H = models.bose_hubbard(3, 3, 1.0, 2.0)
    n = len(states)
    M = te_gpu.Matrix.from_coo(n, H)
    with pytest.raises(te_gpu.TeError) as e:
        te_gpu.Evolver(M, np.ones(n, dtype=complex), 1.0, 0.1)
    assert e.value.code == -4


def test_reorthogonalised_mode_strict_parity(te_gpu, oracle_lib):
    """Classical Gram-Schmidt with one reorthogonalisation pass on both sides:
    the basis stays orthonormal, rounding no longer amplifies, and the
    observables agree to 1e-9 absolute on the case where the three-term
    recurrence cannot (L=8, t=10)."""
    states, H = models.bose_hubbard(8, 8, 1.0, 2.0)
    v = _fock(states, [8] + [0] * 7)
    obs = [("sparse", o) for o in models.number_operator_observables(states)]
    gpu = te_gpu.evolve(H, v, 10.0, 0.1, obs, tol=1e-8, m=40, reorth=True, trace=True)
    ref = oracle_lib.evolve(H, v, 10.0, 0.1, obs, tol=1e-8, m=40, reorth=True, trace=True)
    d_obs = _compare(gpu, ref, 1e-8, strict=True)
    assert d_obs < 1e-11, d_obs
    for a, b in zip(gpu["trace"], ref["trace"]):
        assert abs(a["h"] - b["h"]) <= 1e-7 * b["h"]
    # and the stable basis reproduces the three-term result within the error bound
    plain = oracle_lib.evolve(H, v, 10.0, 0.1, obs, tol=1e-8, m=40)
    assert np.max(np.abs(gpu["samples"] - plain["samples"])) < 4 * 1e-8 * 8.0


def test_reorthogonalised_mode_l12(te_gpu, oracle_lib):
    states, H = models.bose_hubbard(12, 12, 1.0, 3.0)
    v = _random_state(len(states), 0)
    obs = [("sparse", models.create_matrix([models.number_operator(0, 1.0)], states))]
    gpu = te_gpu.evolve(H, v, 0.5, 0.25, obs, tol=1e-8, m=40, reorth=True)
    ref = oracle_lib.evolve(H, v, 0.5, 0.25, obs, tol=1e-8, m=40, reorth=True)
    _compare(gpu, ref, 1e-8, strict=True)


@pytest.mark.parametrize("lanes", [1, 2, 4])
def test_spmv_lanes_variants(te_gpu, oracle_lib, lanes):
    """Every lanes-per-row variant of the SpMV passes against the oracle: the
    product to 1e-13 and a full L=8 evolution within the parity bounds."""
    states, H = models.bose_hubbard(8, 8, 1.0, 2.0)
    n = len(states)
    M = te_gpu.Matrix.from_coo(n, H)
    M.set_spmv_lanes(lanes)
    assert M.spmv_lanes(tune=False) == lanes
    x = _random_state(n, 7)
    ref = oracle_lib.spmv(H, x, -1j)
    assert np.linalg.norm(M.spmv(x, -1j) - ref) <= 1e-13 * np.linalg.norm(ref)
    v = _fock(states, [8] + [0] * 7)
    obs = [("sparse", o) for o in models.number_operator_observables(states)]
    O = [("sparse", te_gpu.Matrix.from_coo(n, o)) for _, o in obs]
    ev = te_gpu.Evolver(M, v, 10.0, 0.1, O, tol=1e-8, m=40)
    gpu = ev.time_evolve()
    ev.close()
    assert M.spmv_lanes(tune=False) == lanes  # a pinned choice is kept by the evolver
    ref = oracle_lib.evolve(H, v, 10.0, 0.1, obs, tol=1e-8, m=40)
    _compare(gpu, ref, 1e-8, obs_norm=8.0, strict=False)


def test_spmv_lanes_tuning(te_gpu):
    """The lanes per row of the FP64 passes follow the matrix's shape: 2 for
    L=10 (2 887 chunks, fewer than the resident warps), 1 for L=11 (11 011
    chunks), for a complex and a real matrix, and the same for every copy of
    a matrix (the choice changes the rounding of the row sums)."""
    states, H = models.bose_hubbard(10, 10, 1.0, 2.0)
    row, col, val = (np.asarray(a) for a in H)
    phase = np.where(row < col, np.exp(0.3j), np.where(row > col, np.exp(-0.3j), 1.0))
    Hc = (row, col, np.asarray(val, dtype=np.complex128) * phase)  # Hermitian, complex hopping
    M = te_gpu.Matrix.from_coo(len(states), Hc)
    assert not M.info()["real"]
    assert M.spmv_lanes(tune=True) == 2
    assert M.spmv_lanes(tune=True) == 2  # chosen once
    for _ in range(2):
        assert te_gpu.Matrix.from_coo(len(states), H).spmv_lanes(tune=True) == 2
    states11, H11 = models.bose_hubbard(11, 11, 1.0, 2.0)
    assert te_gpu.Matrix.from_coo(len(states11), H11).spmv_lanes(tune=True) == 1
    # the autotuner proper times the variants, once
    Mt = te_gpu.Matrix.from_coo(len(states), H)
    Mt.set_spmv_lanes(-1)
    k = Mt.spmv_lanes(tune=True)
    assert k in (1, 2, 4) and Mt.spmv_lanes(tune=True) == k


@pytest.mark.parametrize("L,t,sampling", [(8, 10.0, 0.1), (11, 2.0, 0.5)])
def test_fused_and_per_iteration_lanczos_agree(te_gpu, oracle_lib, L, t, sampling):
    """The persistent Lanczos kernel and the per-iteration passes: same step
    sequence and status, states within the Krylov truncation error, and both
    within the bounds against the oracle."""
    states, H = models.bose_hubbard(L, L, 1.0, 2.0)
    n = len(states)
    v = _fock(states, [L] + [0] * (L - 1))
    O = models.create_matrix([models.number_operator(0, 1.0)], states)
    M = te_gpu.Matrix.from_coo(n, H)
    Om = te_gpu.Matrix.from_coo(n, O)
    out = {}
    for fused in (2, 0):  # always fused / never fused
        ev = te_gpu.Evolver(M, v, t, sampling, [("sparse", Om)], tol=1e-8, m=40)
        ev.set_option(te_gpu.OPT_FUSED_LANCZOS, fused)
        out[fused] = ev.time_evolve()
        ev.close()
    a, b = out[2], out[0]
    assert a["n_steps"] == b["n_steps"] and a["status"] == b["status"] and a["num_samples"] == b["num_samples"]
    assert np.linalg.norm(a["state"] - b["state"]) < 2e-8
    ref = oracle_lib.evolve(H, v, t, sampling, [("sparse", O)], tol=1e-8, m=40)
    for r in (a, b):
        _compare(r, ref, 1e-8, obs_norm=float(L), strict=False)


def test_dense_observable(te_gpu, oracle_lib):
    """A dense Hermitian observable on the GPU (te_evolver_add_dense_observable)
    against the oracle with the same matrix as a full COO."""
    states, H = models.bose_hubbard(5, 5, 1.0, 2.0)
    n = len(states)
    rng = np.random.default_rng(9)
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    D = (A + A.conj().T) / (2 * np.sqrt(n))
    rr, cc = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    coo = (rr.ravel(), cc.ravel(), D.ravel())
    v = _fock(states, [5, 0, 0, 0, 0])
    ev = te_gpu.Evolver(te_gpu.Matrix.from_coo(n, H), v, 2.0, 0.25, [("dense", D)], tol=1e-8, m=30)
    gpu = ev.time_evolve()
    ev.close()
    ref = oracle_lib.evolve(H, v, 2.0, 0.25, [("sparse", coo)], tol=1e-8, m=30)
    d_norm = np.max(np.abs(np.linalg.eigvalsh(D)))
    _compare(gpu, ref, 1e-8, obs_norm=d_norm, strict=False)
    # the value at t = 0 is exact
    assert abs(gpu["samples"][0][0] - np.real(v.conj() @ D @ v)) < 1e-13


@pytest.mark.parametrize("fused_obs", [True, False])
def test_device_stop_condition(te_gpu, oracle_lib, fused_obs):
    """A device-side stop condition stops where an observable raising the stop
    request at the same sample does (the oracle's stop at that index): status 3,
    the samples before it, the time and error of the step start."""
    states, H = models.bose_hubbard(4, 4, 1.0, 2.0)
    n = len(states)
    v = _fock(states, [4, 0, 0, 0])
    obs = [("sparse", o) for o in models.number_operator_observables(states)]
    full = oracle_lib.evolve(H, v, 2.0, 0.1, obs, tol=1e-8, m=20)
    n0 = full["samples"][0]
    k = int(np.argmax(n0 <= 3.6))  # first sample with <n_0> <= 3.6 (it falls from 4 to 3.46)
    assert 0 < k < len(n0) - 1
    ref = oracle_lib.evolve(H, v, 2.0, 0.1, obs + [("stop", k)], tol=1e-8, m=20)
    M = te_gpu.Matrix.from_coo(n, H)
    O = [("sparse", te_gpu.Matrix.from_coo(n, o)) for _, o in obs]
    if not fused_obs:  # a general (non-diagonal) observable routes samples through the per-sample path
        O.append(("sparse", te_gpu.Matrix.from_coo(n, H)))
    ev = te_gpu.Evolver(M, v, 2.0, 0.1, O, tol=1e-8, m=20)
    ev.add_stop_condition(0, 3.6, -1)
    gpu = ev.time_evolve()
    ev.close()
    assert gpu["status"] == ref["status"] == 3
    assert gpu["num_samples"] == ref["num_samples"] == k
    assert abs(gpu["evolved_time"] - ref["evolved_time"]) < 1e-12
    assert abs(gpu["err"] - ref["err"]) < 1e-12
    assert np.max(np.abs(gpu["samples"][:4, :k] - ref["samples"][:, :k])) < OBS_TOL
