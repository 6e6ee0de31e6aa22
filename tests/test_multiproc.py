"""The bench's multi-rank bookkeeping on CPU processes (gloo, world size 2).

On several GPUs every rank solves its own replica of the workload and the job's time is
the slowest rank's (all-reduce MAX over ranks); the whole-job throughput counts every
rank's solves. The same helpers run here over gloo with two CPU processes.
"""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(100.0 + 50.0 * rank, world)  # rank 1 is the slow one
        q.put((rank, ms, bench.replica_throughput(5, ms, world)))
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=10) for _ in range(2))
    for rank, ms, value in out:
        assert ms == 150.0                     # both ranks report the slower rank's time
        assert abs(value - 2 * 5 / 0.150) < 1e-9  # 10 solves in 0.15 s


def test_single_rank_is_untouched():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5, 1) == 12.5
    assert bench.replica_throughput(4, 500.0, 1) == 8.0
