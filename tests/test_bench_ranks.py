"""bench.py with N > 1 ranks (CPU, gloo, world size 2): the replicas' whole-job
throughput uses the slowest rank's time on every rank, and the reference arm
runs on rank 0 only."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)

    def max_over_ranks(x: float) -> float:
        t = torch.tensor([x], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    # rank r took (1 + r) seconds for its 5 steps
    out[rank] = bench.replica_rate(5, 1.0 + rank, world, max_over_ranks)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_rate_uses_the_slowest_rank():
    world = 2
    out = mp.Manager().dict()
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    # 2 ranks x 5 steps over the slowest rank's 2 s
    assert out[0] == out[1] == pytest.approx(5.0)


def test_reference_arm_runs_on_rank_zero_only(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class A:
        steps, warmup = 1, 0

    bench.run_reference(A(), rank=1, world=2)
    assert capsys.readouterr().out == ""
