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


def _batch(te, specs, persistent):
    inst = [dict(H=te.Matrix.from_coo(s["n"], s["coo"]), v=s["v"], t=s["t"], sampling_step=s["sampling_step"],
                 tol=s["tol"], m=s["m"], observables=[te.Matrix.from_coo(s["n"], s["n0"])]) for s in specs]
    return te.Batch(inst, persistent=persistent)


def test_persistent_launch_equals_graph_path(te_gpu, oracle_lib):
    """The whole batch in one persistent cooperative launch runs the graph
    path's passes over the same logical schedule: results, samples and final
    states equal bit for bit, with one kernel launch per run (after the two of
    the reset), and a second run repeats the first."""
    specs = _instances(te_gpu, 3, 24)
    graph = _batch(te_gpu, specs, False)
    rg = graph.run()
    pers = _batch(te_gpu, specs, True)
    for rep in range(2):
        rp = pers.run()
        assert pers.launch_count() == 3
        assert pers.global_steps() == graph.global_steps() > 0
        assert rp == rg
        for i in range(len(specs)):
            assert np.array_equal(pers.samples(i), graph.samples(i)), i
            assert np.array_equal(pers.state(i), graph.state(i)), i
    s = specs[7]
    ref = oracle_lib.evolve(s["coo"], s["v"], s["t"], s["sampling_step"], [("sparse", s["n0"])], tol=s["tol"],
                            m=s["m"])
    assert np.linalg.norm(pers.state(7) - ref["state"]) < 2 * s["tol"]
    graph.close()
    pers.close()


def test_persistent_barrier_timeout_then_recovers(te_gpu):
    """A grid barrier that waits for one block more than the grid has gives up
    after the spin limit: te_batch_run returns TE_ERR_DEVICE_TIMEOUT (no hang,
    the context stays usable), and the same batch then runs normally."""
    specs = _instances(te_gpu, 5, 6)
    ref = _batch(te_gpu, specs, False)
    rr = ref.run()
    b = _batch(te_gpu, specs, True)
    b.set_option(te_gpu.BATCH_OPT_BARRIER_SPIN_LIMIT, 2000)
    b.set_option(te_gpu.BATCH_OPT_BARRIER_EXTRA_ARRIVALS, 1)
    with pytest.raises(te_gpu.TeError) as e:
        b.run()
    assert e.value.code == -10  # TE_ERR_DEVICE_TIMEOUT
    b.set_option(te_gpu.BATCH_OPT_BARRIER_EXTRA_ARRIVALS, 0)
    b.set_option(te_gpu.BATCH_OPT_BARRIER_SPIN_LIMIT, 1 << 22)
    assert b.run() == rr
    for i in range(len(specs)):
        assert np.array_equal(b.samples(i), ref.samples(i))
    with pytest.raises(te_gpu.TeError):
        b.set_option(te_gpu.BATCH_OPT_PERSISTENT, 2)
    ref.close()
    b.close()
