"""The oracle's restatement against the reference itself (CPU only).

oracle/ref_recipe.py compiles the reference's own core/*.cpp (unmodified, with
stand-ins only for CBLAS/LAPACKE, Boost.Math quadrature and Boost.Log) into
oracle/_ref/libteref.so where the reference tree is present; these tests are
skipped elsewhere.  They check that build against the reference's goldens
(so the stand-ins reproduce the reference's outputs), then the restatement
in oracle/te_oracle.cpp against it on the small and large Bose-Hubbard
workloads.

Tolerances: the goldens at the reference's own 1e-8 (testBlackHole.cpp:39-44)
and 6 digits (the CSV).  Restatement against reference: the same status,
step count and sample count; both error bounds <= tol; states
within 2 tol and observables within 4 tol ||O|| (two FP64 runs of the
three-term recurrence agree to the Krylov truncation error once the basis
loses orthogonality), and to 1e-9 where the recurrence stays stable.
"""
import os

import numpy as np
import pytest

import oracle
from oracle import models

GOLD = os.path.join(os.path.dirname(__file__), "golden")

pytestmark = pytest.mark.skipif(not oracle.ref_available(), reason="oracle/_ref not built (reference tree absent)")


def _vec(n, i):
    v = np.zeros(n, dtype=np.complex128)
    v[i] = 1.0
    return v


def _same_run(a, b, tol, obs_bound):
    assert a["status"] == b["status"], (a["status"], b["status"])
    assert a["n_steps"] == b["n_steps"], (a["n_steps"], b["n_steps"])
    assert a["num_samples"] == b["num_samples"]
    assert a["krylov_dim"] == b["krylov_dim"]
    assert abs(a["evolved_time"] - b["evolved_time"]) <= 1e-12 * max(1.0, b["evolved_time"])
    assert a["err"] <= tol and b["err"] <= tol
    d_obs = float(np.max(np.abs(a["samples"] - b["samples"]))) if a["samples"].size else 0.0
    d_state = float(np.linalg.norm(a["state"] - b["state"]))
    assert d_obs < obs_bound, d_obs
    assert d_state < 2 * tol, d_state
    return d_obs, d_state


def test_reference_build_reproduces_black_hole_golden():
    states, H, i0 = models.black_hole(N0=20, Nm=2, K=4)
    obs = [("sparse", o) for o in models.number_operator_observables(states)]
    r = oracle.ref_evolve(H, _vec(len(states), i0), 10.0, 0.01, obs, tol=1e-8, m=40)
    gold = np.load(os.path.join(GOLD, "blackhole_N20.npy"))
    assert r["num_samples"] == 1001
    assert np.max(np.abs(r["samples"] - gold)) < 1e-8
    assert r["err"] <= 1e-8


def test_reference_build_reproduces_lucky_breakdown_golden():
    states, H, i0 = models.black_hole(N0=1, Nm=1, K=1)
    obs = [("sparse", o) for o in models.number_operator_observables(states)]
    r = oracle.ref_evolve(H, _vec(4, i0), 1000.0, 1.0, obs, tol=1e-8, m=40)
    gold = np.load(os.path.join(GOLD, "blackhole_N1_LB.npy"))
    assert r["status"] == 1 and r["krylov_dim"] == 4 and r["n_steps"] == 1
    assert np.max(np.abs(r["samples"] - gold)) < 1e-8


def test_reference_build_reproduces_simple_example_golden():
    states, H, i0 = models.simple_example()
    obs = [("sparse", o) for o in models.number_operator_observables(states)]
    r = oracle.ref_evolve(H, _vec(len(states), i0), 10.0, 0.01, obs, tol=1e-6, m=40)
    gold = np.load(os.path.join(GOLD, "simple_example.npy"))
    rounded = np.vectorize(lambda x: float("%g" % x))(r["samples"])
    assert np.array_equal(rounded, gold)


@pytest.mark.parametrize("fast", [False, True])
def test_restatement_matches_reference_small(oracle_lib, fast):
    """Bose-Hubbard L=8 N=8 (dim 6435), all bosons on site 0, t=10, tol 1e-8,
    m=40, <n_i> every 0.1 (both integration methods)."""
    states, H = models.bose_hubbard(8, 8, 1.0, 2.0)
    v = _vec(len(states), models.index_of(states, [8] + [0] * 7))
    obs = [("sparse", o) for o in models.number_operator_observables(states)]
    ref = oracle.ref_evolve(H, v, 10.0, 0.1, obs, tol=1e-8, m=40, fast_integration=fast)
    port = oracle_lib.evolve(H, v, 10.0, 0.1, obs, tol=1e-8, m=40, fast_integration=fast)
    _same_run(port, ref, 1e-8, 4 * 1e-8 * 8.0)


def test_restatement_matches_reference_vector_observable(oracle_lib):
    rng = np.random.default_rng(3)
    states, H = models.bose_hubbard(6, 5, 0.7, 1.3)
    n = len(states)
    v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    v /= np.linalg.norm(v)
    o = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    o /= np.linalg.norm(o)
    ref = oracle.ref_evolve(H, v, 3.0, 0.25, [("vector", o)], exp_factor=0.8, tol=1e-9, m=24)
    port = oracle_lib.evolve(H, v, 3.0, 0.25, [("vector", o)], exp_factor=0.8, tol=1e-9, m=24)
    _same_run(port, ref, 1e-9, 1e-9)


def test_restatement_matches_reference_large():
    """Bose-Hubbard L=12 N=12 U=3 (dim 1352078), complex Gaussian v
    (default_rng(0)), tol 1e-8, m=40, <n_0> every 0.5, to t=1."""
    states, H = models.bose_hubbard(12, 12, 1.0, 3.0)
    n = len(states)
    rng = np.random.default_rng(0)
    v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    v /= np.linalg.norm(v)
    obs = [("sparse", models.create_matrix([models.number_operator(0, 1.0)], states))]
    ref = oracle.ref_evolve(H, v, 1.0, 0.5, obs, tol=1e-8, m=40)
    port = oracle.evolve(H, v, 1.0, 0.5, obs, tol=1e-8, m=40, n_threads=os.cpu_count())
    d_obs, _ = _same_run(port, ref, 1e-8, 1e-9)
    assert ref["n_steps"] >= 4
