"""The multi-process (replica) host logic of bench.py on the CPU: two gloo ranks
on 127.0.0.1 exercise the barrier, the max-over-ranks timing, the replica
throughput and the rank-0-only output, as a GPU run with one rank per GPU
uses them (there with NCCL)."""
import json
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    ws, r, local = bench.dist_info()
    dist = bench.init_dist(ws, local, backend="gloo")
    bench.barrier(dist)
    # a per-rank "timed region": rank 1 is the slow one
    ms = 100.0 + 50.0 * r
    worst = bench.max_over_ranks(dist, ms)
    value = bench.replica_seconds_per_solve(worst, 5, ws)
    bench.barrier(dist)
    if r == 0:  # one JSON line, from rank 0 only
        with open(os.path.join(out_dir, "line.json"), "w") as f:
            f.write(json.dumps({"value": value, "max_ms": worst, "n_gpus": ws}) + "\n")
    with open(os.path.join(out_dir, "rank%d.txt" % r), "w") as f:
        f.write("%g\n" % worst)
    dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_gloo_ranks(tmp_path):
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    line = json.loads((tmp_path / "line.json").read_text())
    assert line["n_gpus"] == 2
    assert line["max_ms"] == 150.0  # the slowest rank sets the time
    assert abs(line["value"] - 150.0 / 1000.0 / 5 / 2) < 1e-15  # 2 replicas x 5 solves in 150 ms
    for r in range(world):
        assert float((tmp_path / ("rank%d.txt" % r)).read_text()) == 150.0
    assert sorted(p.name for p in tmp_path.iterdir()) == ["line.json", "rank0.txt", "rank1.txt"]


def test_reference_arm_other_ranks_do_nothing(monkeypatch, capsys):
    """--impl reference under torchrun: ranks other than 0 return at once."""
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")

    class Args:
        steps, warmup, gpus = 1, 0, 2

    bench.run_reference(Args())
    assert capsys.readouterr().out == ""
