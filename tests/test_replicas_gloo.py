"""Multi-GPU runs are independent replicas (one simulation does not shard without a
halo exchange): bench.py reduces each rank's timed region to the whole-job figure
with two collectives -- the slowest rank's time and the units summed over ranks.
Checked here on CPU with two gloo ranks."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q) -> None:
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    secs, value = bench.job_throughput(dist, seconds=1.0 + rank, units=100.0 * (rank + 1), device="cpu")
    q.put((rank, secs, value))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_reduce_to_the_job_throughput():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, secs, value in out:
        assert secs == 2.0                      # the slowest rank's time, on every rank
        assert value == pytest.approx(300.0 / 2.0)  # all ranks' units over that time


def test_single_process_needs_no_collective():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_throughput(None, 2.0, 50.0) == (2.0, 25.0)
