"""Fixed-point SpMV of the three-term Lanczos passes (te_fixed.cuh; needs a
GB300).  The SpMV runs in integer arithmetic on values
quantised at 2^-61 of the largest row 1-norm and of max|u|, with one rounding
to double per row; the evolution must meet the same bounds against the oracle
as the FP64 path (same steps, status and samples; states within 2 tol).
"""
import numpy as np
import pytest

from oracle import models

pytestmark = pytest.mark.gpu


def _fock(states, occ):
    v = np.zeros(len(states), dtype=np.complex128)
    v[models.index_of(states, occ)] = 1.0
    return v


def _run(te_gpu, M, v, t, dt, obs, fixed, m=40, tol=1e-8):
    obs = [(k, te_gpu.Matrix.from_coo(len(v), d) if k == "sparse" and isinstance(d, tuple) else d) for k, d in obs]
    ev = te_gpu.Evolver(M, v, t, dt, obs, tol=tol, m=m)
    ev.set_option(te_gpu.OPT_FIXED_SPMV, fixed)
    r = ev.time_evolve()
    ev.close()
    return r


def _bounds(gpu, ref, tol, obs_norm, same_steps=True):
    """same_steps=False: the error-controlled guarantees only (an adaptive
    step whose error estimate lands within rounding of the tolerance may be
    accepted on one machine and halved on the other)."""
    assert gpu["status"] == ref["status"]
    assert gpu["num_samples"] == ref["num_samples"]
    assert abs(gpu["evolved_time"] - ref["evolved_time"]) < 1e-12 * max(1.0, ref["evolved_time"])
    if same_steps:
        assert gpu["n_steps"] == ref["n_steps"]
        assert gpu["krylov_dim"] == ref["krylov_dim"]
    assert np.linalg.norm(gpu["state"] - ref["state"]) < 2 * tol
    assert np.max(np.abs(gpu["samples"] - ref["samples"])) < max(1e-9, 4 * tol * obs_norm)
    assert gpu["err"] <= tol


@pytest.mark.parametrize("L,U,t,same_steps", [(10, 2.0, 5.0, True), (10, 40.0, 2.0, False)])
def test_fixed_spmv_bose_hubbard(te_gpu, oracle_lib, L, U, t, same_steps):
    """BH L=10 N=10 (dim 92378, 2887 chunks): the fixed-point passes run (two
    more launches per Krylov step: the encoding of u_0), agree with the FP64
    passes (same steps) and with the oracle.  U = 40 puts the hopping 10^3
    below the largest row 1-norm; there the GPU (fixed-point and FP64 alike)
    takes 35 steps and the oracle 36, so that case is held to the
    error-controlled bounds."""
    states, H = models.bose_hubbard(L, L, 1.0, U)
    n = len(states)
    v = _fock(states, [L] + [0] * (L - 1))
    O = models.create_matrix([models.number_operator(0, 1.0)], states)
    M, Om = te_gpu.Matrix.from_coo(n, H), te_gpu.Matrix.from_coo(n, O)
    assert M.fixed_layout()["state"] == 0
    a = _run(te_gpu, M, v, t, 0.5, [("sparse", Om)], 1)
    b = _run(te_gpu, M, v, t, 0.5, [("sparse", Om)], 0)
    fl = M.fixed_layout()
    assert fl["state"] == 2 and 0 < fl["n_values"] <= 4096  # few distinct values: dictionary
    assert a["launches"] == b["launches"] + 2 * a["n_steps"]
    assert a["n_steps"] == b["n_steps"] and a["status"] == b["status"]
    assert np.linalg.norm(a["state"] - b["state"]) < 2e-8
    ref = oracle_lib.evolve(H, v, t, 0.5, [("sparse", O)], tol=1e-8, m=40)
    for r in (a, b):
        _bounds(r, ref, 1e-8, float(L), same_steps)


def test_fixed_spmv_first_krylov_space(te_gpu, oracle_lib):
    """One Krylov step of a random start vector: the Krylov coefficients come
    from 40 fixed-point SpMVs; the step size and error agree with the oracle's
    to 1e-12 and the samples to 1e-9 (no loss of orthogonality yet)."""
    states, H = models.bose_hubbard(10, 10, 1.0, 3.0)
    n = len(states)
    rng = np.random.default_rng(4)
    v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    v[:: 7] *= 1e-9  # components nine decades below the rest
    v /= np.linalg.norm(v)
    O = models.create_matrix([models.number_operator(0, 1.0)], states)
    M = te_gpu.Matrix.from_coo(n, H)
    ev = te_gpu.Evolver(M, v, 0.2, 0.1, [("sparse", te_gpu.Matrix.from_coo(n, O))], tol=1e-8, m=40)
    gpu = ev.time_evolve(trace=True)
    ev.close()
    ref = oracle_lib.evolve(H, v, 0.2, 0.1, [("sparse", O)], tol=1e-8, m=40, trace=True)
    _bounds(gpu, ref, 1e-8, 10.0)
    assert np.max(np.abs(gpu["samples"] - ref["samples"])) < 1e-9
    for x, y in zip(gpu["trace"], ref["trace"]):
        assert abs(x["t_step"] - y["t_step"]) <= 1e-12 * y["t_step"]
        # estimates near the rounding level (1e-17 vs 5e-15) are noise: floor 1e-4 tol
        assert abs(x["err_step"] - y["err_step"]) <= 1e-6 * y["err_step"] + 1e-12


def _hub_matrix(n, hubs, hub_len, seed):
    rng = np.random.default_rng(seed)
    r = np.repeat(np.arange(n), 4)
    c = rng.integers(0, n, size=4 * n)
    hr = np.repeat(np.array(hubs), hub_len)
    hc = np.concatenate([rng.choice(n, size=hub_len, replace=False) for _ in hubs])
    row = np.concatenate([r, hr])
    col = np.concatenate([c, hc])
    val = rng.standard_normal(len(row))
    # symmetrise: H = (A + A^T) / 2, duplicates summed by the CSR build
    row, col, val = np.concatenate([row, col]), np.concatenate([col, row]), np.concatenate([val, val]) / 2
    key = row * n + col
    order = np.argsort(key, kind="stable")
    key, val = key[order], val[order]
    uk, start = np.unique(key, return_index=True)
    sval = np.add.reduceat(val, start)
    return uk // n, uk % n, sval.astype(np.complex128)


def test_fixed_spmv_long_rows(te_gpu, oracle_lib):
    """Real matrix of 70000 rows (2188 chunks) with 3 hub rows of 3000
    entries: the hubs stay FP64 (warp per row) next to the fixed-point chunks."""
    n = 70000
    row, col, val = _hub_matrix(n, [5, n // 3, n - 2], 3000, 12)
    M = te_gpu.Matrix(n, row, col, val)
    assert M.layout()["long_rows"] == 3 and M.info()["real"]
    rng = np.random.default_rng(6)
    v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    v /= np.linalg.norm(v)
    d = (np.arange(n), np.arange(n), rng.uniform(-1, 1, n).astype(np.complex128))
    a = _run(te_gpu, M, v, 1.0, 0.25, [("sparse", d)], 1, m=30)
    b = _run(te_gpu, M, v, 1.0, 0.25, [("sparse", d)], 0, m=30)
    assert M.fixed_layout()["state"] == 1  # Gaussian values: limbs per slot
    assert a["launches"] == b["launches"] + 2 * a["n_steps"]
    ref = oracle_lib.evolve((row, col, val), v, 1.0, 0.25, [("sparse", d)], tol=1e-8, m=30)
    for r in (a, b):
        _bounds(r, ref, 1e-8, 1.0)


def test_fixed_spmv_complex(te_gpu, oracle_lib):
    """A complex Hermitian matrix of 70000 rows (2188 chunks, Gaussian values):
    the complex fixed-point SpMV (four limb products per entry) against the
    FP64 passes and the oracle."""
    rng = np.random.default_rng(8)
    n = 70000
    r = np.repeat(np.arange(n), 3)
    c = rng.integers(0, n, size=3 * n)
    z = rng.standard_normal(3 * n) + 1j * rng.standard_normal(3 * n)
    row, col, val = np.concatenate([r, c]), np.concatenate([c, r]), np.concatenate([z, z.conj()]) / 2
    key = row * n + col
    order = np.argsort(key, kind="stable")
    uk, start = np.unique(key[order], return_index=True)
    row, col, val = uk // n, uk % n, np.add.reduceat(val[order], start)
    M = te_gpu.Matrix(n, row, col, val)
    assert not M.info()["real"]
    v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    v /= np.linalg.norm(v)
    d = (np.arange(n), np.arange(n), rng.uniform(-1, 1, n).astype(np.complex128))
    a = _run(te_gpu, M, v, 1.0, 0.25, [("sparse", d)], 1, m=30)
    b = _run(te_gpu, M, v, 1.0, 0.25, [("sparse", d)], 0, m=30)
    assert M.fixed_layout()["state"] == 1
    assert a["launches"] == b["launches"] + 2 * a["n_steps"]
    assert a["n_steps"] == b["n_steps"] and a["status"] == b["status"]
    ref = oracle_lib.evolve((row, col, val), v, 1.0, 0.25, [("sparse", d)], tol=1e-8, m=30)
    for res in (a, b):
        _bounds(res, ref, 1e-8, 1.0)


def test_fixed_spmv_dictionary_matches_limbs(te_gpu):
    """The same BH matrix through the value dictionary and through per-slot
    limbs (the dictionary ruled out by a value set too large for it: the
    diagonal perturbed by up to 1e-13 of its largest entry, tens of thousands
    of distinct doubles): the evolutions agree to the perturbation."""
    states, H = models.bose_hubbard(10, 10, 1.0, 2.0)
    n = len(states)
    row, col, val = H
    row, col, val = np.asarray(row), np.asarray(col), np.asarray(val, dtype=np.complex128)
    rng = np.random.default_rng(2)
    pert = val.copy()
    diag = row == col
    pert[diag] += rng.uniform(-1, 1, diag.sum()) * 1e-13 * np.abs(val[diag]).max()
    v = _fock(states, [10] + [0] * 9)
    Md, Ml = te_gpu.Matrix(n, row, col, val), te_gpu.Matrix(n, row, col, pert)
    a = _run(te_gpu, Md, v, 1.0, 0.5, [], 1)
    b = _run(te_gpu, Ml, v, 1.0, 0.5, [], 1)
    assert Md.fixed_layout()["state"] == 2 and Ml.fixed_layout()["state"] == 1
    assert a["n_steps"] == b["n_steps"]
    assert np.linalg.norm(a["state"] - b["state"]) < 1e-10  # ||dH|| t <= 9e-12


def _random_hermitian_70k(seed, complex_values):
    rng = np.random.default_rng(seed)
    n = 70000
    r = np.repeat(np.arange(n), 3)
    c = rng.integers(0, n, size=3 * n)
    z = rng.standard_normal(3 * n) + (1j * rng.standard_normal(3 * n) if complex_values else 0)
    row, col, val = np.concatenate([r, c]), np.concatenate([c, r]), np.concatenate([z, np.conj(z)]) / 2
    key = row * n + col
    order = np.argsort(key, kind="stable")
    uk, start = np.unique(key[order], return_index=True)
    return n, (uk // n, uk % n, np.add.reduceat(np.asarray(val, np.complex128)[order], start))


@pytest.mark.parametrize("complex_values,blocks", [(False, 3), (True, 2), (True, 8)])
def test_fixed_spmv_column_blocks(te_gpu, oracle_lib, complex_values, blocks):
    """Column blocks of the fixed-point SpMV (forced on a 70000-row matrix;
    automatic for fixed-point vectors above 96 MB): the block passes add exact
    int64 row sums, so the products equal the unblocked ones; the evolutions
    agree with the unblocked path and stay within the bounds of the oracle."""
    n, coo = _random_hermitian_70k(21, complex_values)
    rng = np.random.default_rng(5)
    v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    v /= np.linalg.norm(v)
    d = (np.arange(n), np.arange(n), rng.uniform(-1, 1, n).astype(np.complex128))
    Mb = te_gpu.Matrix(n, *coo)
    Mb.set_fixed_blocks(blocks)
    a = _run(te_gpu, Mb, v, 1.0, 0.25, [("sparse", d)], 1, m=30)
    assert Mb.fixed_layout()["state"] == 3 and Mb.fixed_layout()["n_values"] == blocks
    Mu = te_gpu.Matrix(n, *coo)
    Mu.set_fixed_blocks(1)
    b = _run(te_gpu, Mu, v, 1.0, 0.25, [("sparse", d)], 1, m=30)
    assert Mu.fixed_layout()["state"] == 1
    assert a["n_steps"] == b["n_steps"] and a["status"] == b["status"]
    assert a["launches"] > b["launches"]  # the block passes
    assert np.linalg.norm(a["state"] - b["state"]) < 1e-9
    ref = oracle_lib.evolve(coo, v, 1.0, 0.25, [("sparse", d)], tol=1e-8, m=30)
    _bounds(a, ref, 1e-8, 1.0)


def test_fixed_spmv_without_memory_runs_fp64(te_gpu):
    """An evolution that cannot get device memory for the fixed-point vectors
    runs the FP64 passes instead of failing: the result equals, bit for bit,
    the run with TE_OPT_FIXED_SPMV = 0 on the same matrix.  The library's
    cached buffers are released and the device is filled up to 24 MB (the
    fixed-point copies of the basis need 59 MB) just for that run."""
    import torch
    states, H = models.bose_hubbard(10, 10, 1.0, 2.0)
    n = len(states)
    v = _fock(states, [10] + [0] * 9)
    O = models.create_matrix([models.number_operator(0, 1.0)], states)
    M, Om = te_gpu.Matrix.from_coo(n, H), te_gpu.Matrix.from_coo(n, O)
    _run(te_gpu, M, v, 1.0, 0.5, [("sparse", Om)], 1)  # loads every kernel of both paths
    ref = _run(te_gpu, M, v, 1.0, 0.5, [("sparse", Om)], 0)
    M2 = te_gpu.Matrix.from_coo(n, H)
    ev = te_gpu.Evolver(M2, v, 1.0, 0.5, [("sparse", Om)], tol=1e-8, m=40)
    ev.set_option(te_gpu.OPT_FIXED_SPMV, 0)
    # the evolver's own buffers, allocated on its first run, and the FP64
    # reference on this matrix: the FP64 passes use the lanes per row tuned
    # for it, which another copy of the matrix may tune differently
    ref2 = ev.time_evolve()
    ev.reset(v)
    ev.set_option(te_gpu.OPT_FIXED_SPMV, 1)
    torch.cuda.synchronize()
    # the library keeps released buffers for reuse (among them the fixed-point
    # copies of the earlier runs): free them, so that no memory is left to have
    te_gpu.release_buffers()
    blocker = None
    for spare in (24, 32, 48):
        try:
            blocker = torch.empty(torch.cuda.mem_get_info()[0] - (spare << 20), dtype=torch.uint8, device="cuda")
            break
        except RuntimeError:
            torch.cuda.empty_cache()
    assert blocker is not None
    try:
        r = ev.time_evolve()
    finally:
        del blocker
        torch.cuda.empty_cache()
        ev.close()
    assert r["n_steps"] == ref["n_steps"] and r["status"] == ref["status"]
    assert np.linalg.norm(ref2["state"] - ref["state"]) < 1e-12
    assert np.array_equal(r["state"], ref2["state"])
    assert np.array_equal(r["samples"], ref2["samples"])
