"""The benchmarked workloads, whole, against the oracle (needs a GB300).

* The headline solve: Bose-Hubbard L=12 N=12 J=1 U=3 (dim 1352078), complex
  Gaussian v (numpy default_rng(0), real then imaginary parts), t=10,
  tol 1e-8, m=40, <n_0> every 0.5 -- the full 48-step run, on the default
  fixed-point SpMV and on the FP64 SpMV (TE_OPT_FIXED_SPMV 0).
* The batched workload: instances drawn by the benchmark's own generator
  (L 6..10, N=L, m=32, t up to 20), batched, against the oracle and against
  the single-evolution path.
* The load-imbalanced Zipf matrix at dim 1e6 (complex, fixed-point SpMV,
  automatic form) against the oracle; at dim 8e6, where the fixed-point form
  is split into column blocks automatically, against the FP64 SpMV.

Tolerances (reference algorithm: krylovTimeEvolver.cpp:261-512, status logic
:446-504): both runs are within tol of the exact state, so final states agree
within 2 tol and a sampled observable within 4 tol ||O||; step sizes follow
from the error integral of each step and agree to 1e-12 relative; the
returned error bound is <= tol.
"""
import os
import sys

import numpy as np
import pytest

from oracle import models

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

TOL = 1e-8


def _state(n, seed):
    rng = np.random.default_rng(seed)
    v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    return v / np.linalg.norm(v)


# --------------------------------------------------------------- headline

@pytest.fixture(scope="module")
def headline(oracle_lib):
    states, H = models.bose_hubbard(12, 12, 1.0, 3.0)
    n = len(states)
    v = _state(n, 0)
    O = models.create_matrix([models.number_operator(0, 1.0)], states)
    ref = oracle_lib.evolve(H, v, 10.0, 0.5, [("sparse", O)], tol=TOL, m=40, trace=True,
                            n_threads=os.cpu_count())
    return n, H, O, v, ref


@pytest.mark.parametrize("spmv", ["fixed", "fp64"])
def test_headline_solve_matches_oracle(te_gpu, headline, spmv):
    n, H, O, v, ref = headline
    opt = {te_gpu.OPT_FIXED_SPMV: 1 if spmv == "fixed" else 0}
    M = te_gpu.Matrix.from_coo(n, H)
    gpu = te_gpu.evolve(M, v, 10.0, 0.5, [("sparse", O)], tol=TOL, m=40, trace=True, options=opt)
    layout = M.fixed_layout()
    assert (layout["state"] > 0) == (spmv == "fixed")
    assert ref["n_steps"] == 48 and ref["status"] == 10
    assert gpu["n_steps"] == 48 and gpu["status"] == 10
    assert gpu["num_samples"] == ref["num_samples"] == 21
    assert gpu["krylov_dim"] == ref["krylov_dim"] == 40
    assert gpu["nb_err_roundoff"] == ref["nb_err_roundoff"] and gpu["nb_err_int"] == ref["nb_err_int"]
    assert len(gpu["trace"]) == len(ref["trace"]) == 48
    d_step = max(abs(a["t_step"] - b["t_step"]) / b["t_step"] for a, b in zip(gpu["trace"], ref["trace"]))
    assert d_step <= 1e-12, d_step
    assert [a["code"] for a in gpu["trace"]] == [b["code"] for b in ref["trace"]]
    d_state = float(np.linalg.norm(gpu["state"] - ref["state"]))
    d_obs = float(np.max(np.abs(gpu["samples"] - ref["samples"])))
    assert d_state < 2 * TOL, d_state
    assert d_obs < 4 * TOL * 12.0, d_obs
    assert gpu["err"] <= TOL and ref["err"] <= TOL
    assert abs(gpu["evolved_time"] - ref["evolved_time"]) < 1e-12 * 10.0
    print("headline %s: 48 steps, status 10; max rel d t_step %.2e, |d state| %.2e, max |d <n_0>| %.2e, "
          "err gpu %.3e oracle %.3e" % (spmv, d_step, d_state, d_obs, gpu["err"], ref["err"]))


# ---------------------------------------------------------------- batched

@pytest.fixture(scope="module")
def batched_specs():
    import bench
    specs = bench.batched_instances()[:24]
    assert {s["L"] for s in specs} == {6, 7, 8, 9, 10}
    return specs


def test_batched_instances_match_oracle(te_gpu, oracle_lib, batched_specs):
    specs = batched_specs
    mats = [(te_gpu.Matrix.from_coo(s["n"], s["coo"]), te_gpu.Matrix.from_coo(s["n"], s["n0"])) for s in specs]
    batch = te_gpu.Batch([dict(H=H, v=s["v"], t=s["t"], sampling_step=s["t"], tol=TOL, m=32, observables=[O])
                          for s, (H, O) in zip(specs, mats)])
    res = batch.run()
    worst_state = worst_obs = 0.0
    fixed_diff = []
    for i, (s, (H, O)) in enumerate(zip(specs, mats)):
        ref = oracle_lib.evolve(s["coo"], s["v"], s["t"], s["t"], [("sparse", s["n0"])], tol=TOL, m=32,
                                n_threads=os.cpu_count())
        r = res[i]
        assert r["status"] == ref["status"], (i, r["status"], ref["status"])
        assert r["n_steps"] == ref["n_steps"], (i, s["L"], r["n_steps"], ref["n_steps"])
        assert r["num_samples"] == ref["num_samples"] == 2
        assert r["err"] <= TOL
        st = batch.state(i)
        d_state = float(np.linalg.norm(st - ref["state"]))
        d_obs = float(np.max(np.abs(batch.samples(i) - ref["samples"])))
        assert d_state < 2 * TOL, (i, d_state)
        assert d_obs < 4 * TOL * s["L"], (i, d_obs)
        worst_state, worst_obs = max(worst_state, d_state), max(worst_obs, d_obs)
        # the single-evolution path with the FP64 SpMV takes the batch's step sequence
        fp64 = te_gpu.evolve(H, s["v"], s["t"], s["t"], [("sparse", s["n0"])], tol=TOL, m=32,
                             options={te_gpu.OPT_FIXED_SPMV: 0})
        assert fp64["n_steps"] == r["n_steps"] and fp64["status"] == r["status"], i
        assert np.linalg.norm(fp64["state"] - st) < 2 * TOL
        # its default (fixed-point SpMV for the larger chains) stays within the bound of the oracle
        single = te_gpu.evolve(H, s["v"], s["t"], s["t"], [("sparse", s["n0"])], tol=TOL, m=32)
        assert np.linalg.norm(single["state"] - ref["state"]) < 2 * TOL
        assert single["err"] <= TOL
        if single["n_steps"] != ref["n_steps"]:
            assert abs(single["n_steps"] - ref["n_steps"]) <= 1
            fixed_diff.append(i)
    batch.close()
    print("batched: 24 instances (L 6..10); max |d state| %.2e, max |d <n_0>| %.2e; default single path with "
          "another step count on %s" % (worst_state, worst_obs, fixed_diff))


def test_batched_persistent_launch_equals_graph_path(te_gpu, batched_specs):
    """The benchmark's own instances (L 6..10, m=32) in one persistent launch
    and through the per-step graph: same results, samples and states bit for
    bit (the persistent kernel rereads what its blocks rewrite between grid
    barriers through L2, so no SM uses a stale copy)."""
    specs = batched_specs
    mats = [(te_gpu.Matrix.from_coo(s["n"], s["coo"]), te_gpu.Matrix.from_coo(s["n"], s["n0"])) for s in specs]
    inst = [dict(H=H, v=s["v"], t=s["t"], sampling_step=s["t"], tol=TOL, m=32, observables=[O])
            for s, (H, O) in zip(specs, mats)]
    graph, pers = te_gpu.Batch(inst), te_gpu.Batch(inst, persistent=True)
    rg = graph.run()
    for _ in range(2):
        rp = pers.run()
        bad = [i for i in range(len(specs)) if rp[i] != rg[i] or not np.array_equal(pers.samples(i), graph.samples(i))
               or not np.array_equal(pers.state(i), graph.state(i))]
        assert not bad, bad
    assert pers.global_steps() == graph.global_steps()
    graph.close()
    pers.close()


# ------------------------------------------------------------------- Zipf

def test_zipf_1e6_matches_oracle(te_gpu, oracle_lib):
    n = 1_000_000
    H, _ = te_gpu.Matrix.zipf(n, 1.5, 2, 256, 1, 30)
    coo = H.to_coo()
    v = _state(n, 1)
    t = 10.0
    gpu = te_gpu.evolve(H, v, t, t, [], tol=TOL, m=40, trace=True)
    layout = H.fixed_layout()
    assert layout["state"] == 1  # complex limbs, one block (the vector fits L2)
    ref = oracle_lib.evolve(coo, v, t, t, [], tol=TOL, m=40, trace=True, n_threads=os.cpu_count())
    assert gpu["status"] == ref["status"] and gpu["n_steps"] == ref["n_steps"]
    d_step = max(abs(a["t_step"] - b["t_step"]) / b["t_step"] for a, b in zip(gpu["trace"], ref["trace"]))
    assert d_step <= 1e-12, d_step
    d_state = float(np.linalg.norm(gpu["state"] - ref["state"]))
    assert d_state < 2 * TOL, d_state
    assert gpu["err"] <= TOL and ref["err"] <= TOL
    print("zipf 1e6: %d steps, status %d, |d state| %.2e, max rel d t_step %.2e"
          % (gpu["n_steps"], gpu["status"], d_state, d_step))


def test_zipf_column_blocks_match_fp64(te_gpu):
    n = 8_000_000
    H, _ = te_gpu.Matrix.zipf(n, 1.5, 2, 256, 3, 30)
    v = _state(n, 5)
    t = 20.0
    blk = te_gpu.evolve(H, v, t, t, [], tol=TOL, m=40, trace=True)
    layout = H.fixed_layout()
    assert layout["state"] == 3 and layout["n_values"] >= 2  # automatic column blocks
    fp = te_gpu.evolve(H, v, t, t, [], tol=TOL, m=40, trace=True, options={te_gpu.OPT_FIXED_SPMV: 0})
    assert blk["status"] == fp["status"] and blk["n_steps"] == fp["n_steps"]
    d_step = max(abs(a["t_step"] - b["t_step"]) / b["t_step"] for a, b in zip(blk["trace"], fp["trace"]))
    assert d_step <= 1e-12, d_step
    d_state = float(np.linalg.norm(blk["state"] - fp["state"]))
    assert d_state < 2 * TOL, d_state
    assert blk["err"] <= TOL and fp["err"] <= TOL
    print("zipf 8e6: %d column blocks, %d steps, |d state| %.2e" % (layout["n_values"], blk["n_steps"], d_state))
