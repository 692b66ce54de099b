"""Batched evolutions (te_batch_*) against the single-evolution path and the
oracle (needs a GB300)."""
import numpy as np
import pytest

from oracle import models

pytestmark = pytest.mark.gpu


def _instances(te, seed, count):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        L = int(rng.integers(3, 8))
        N = L if i % 5 else 1  # every fifth instance: one boson -> small Krylov space, lucky breakdown
        J = float(rng.uniform(0.5, 1.5))
        U = float(rng.uniform(0.0, 4.0))
        t = float(rng.uniform(1.0, 4.0))
        states, H = models.bose_hubbard(L, N, J, U)
        v = np.zeros(len(states), dtype=np.complex128)
        v[models.index_of(states, [N] + [0] * (L - 1))] = 1.0
        n0 = models.create_matrix([models.number_operator(0, 1.0)], states)
        out.append(dict(coo=H, n0=n0, v=v, t=t, sampling_step=t / 4.0, tol=1e-8, m=32, n=len(states)))
    return out


def test_batch_matches_single_and_oracle(te_gpu, oracle_lib):
    specs = _instances(te_gpu, 3, 24)
    inst = []
    for s in specs:
        inst.append(dict(H=te_gpu.Matrix.from_coo(s["n"], s["coo"]), v=s["v"], t=s["t"],
                         sampling_step=s["sampling_step"], tol=s["tol"], m=s["m"],
                         observables=[te_gpu.Matrix.from_coo(s["n"], s["n0"])]))
    batch = te_gpu.Batch(inst)
    res = batch.run()
    assert batch.launch_count() > 0
    for i, s in enumerate(specs):
        single = te_gpu.evolve(s["coo"], s["v"], s["t"], s["sampling_step"], [("sparse", s["n0"])], tol=s["tol"],
                               m=s["m"])
        ref = oracle_lib.evolve(s["coo"], s["v"], s["t"], s["sampling_step"], [("sparse", s["n0"])], tol=s["tol"],
                                m=s["m"])
        r = res[i]
        for other in (single, ref):
            assert r["status"] == other["status"], (i, r["status"], other["status"])
            assert r["n_steps"] == other["n_steps"], (i, r["n_steps"], other["n_steps"])
            assert r["num_samples"] == other["num_samples"]
            assert r["krylov_dim"] == other["krylov_dim"]
            assert abs(r["evolved_time"] - other["evolved_time"]) < 1e-12 * max(1.0, s["t"])
        samples = batch.samples(i)
        N = int(max(1, s["v"].size and 1))
        bound = max(1e-9, 4 * s["tol"] * 8.0)
        assert np.max(np.abs(samples - single["samples"])) < bound
        assert np.max(np.abs(samples - ref["samples"])) < bound
        st = batch.state(i)
        assert np.linalg.norm(st - ref["state"]) < 2 * s["tol"]
        assert np.linalg.norm(st - single["state"]) < 2 * s["tol"]
    batch.close()


def test_batch_rerun_is_deterministic(te_gpu):
    specs = _instances(te_gpu, 5, 8)
    inst = [dict(H=te_gpu.Matrix.from_coo(s["n"], s["coo"]), v=s["v"], t=s["t"], sampling_step=s["sampling_step"],
                 tol=s["tol"], m=s["m"], observables=[te_gpu.Matrix.from_coo(s["n"], s["n0"])]) for s in specs]
    batch = te_gpu.Batch(inst)
    r1 = batch.run()
    s1 = [batch.samples(i) for i in range(len(specs))]
    r2 = batch.run()
    s2 = [batch.samples(i) for i in range(len(specs))]
    assert r1 == r2
    for a, b in zip(s1, s2):
        assert np.array_equal(a, b)
