"""The multi-GPU path of bench.py is replicas only: every rank runs the same
workload, the job time is the maximum over ranks and the value counts the
units of all ranks.  Exercised here on CPU with world_size-2 gloo ranks."""
import os
import socket
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local_ms = 10.0 * (rank + 1) + 5.0  # rank 0: 15 ms, rank 1: 25 ms
    job_ms = bench.max_over_ranks(local_ms, world, torch, torch.device("cpu"))
    value = bench.replica_rate(1e9, job_ms, world)
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(f"{job_ms} {value}\n")


def test_max_over_ranks_and_replica_rate_gloo(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    for r in range(world):
        job_ms, value = map(float, (tmp_path / f"rank{r}.txt").read_text().split())
        assert job_ms == 25.0
        # 2 ranks x 1e9 units in 25 ms = 80 G units/s
        assert value == pytest.approx(80.0)


def test_single_rank_is_identity():
    sys.path.insert(0, REPO)
    import bench
    assert bench.max_over_ranks(12.5, 1, None, None) == 12.5
    assert bench.replica_rate(2e9, 1000.0, 1) == pytest.approx(2.0)


def test_reference_arm_other_ranks_do_nothing(capsys):
    sys.path.insert(0, REPO)
    import bench

    class A:
        n, steps, warmup = 1024, 1, 0
    assert bench.run_reference(A(), 1, 2) == 0
    assert capsys.readouterr().out == ""
