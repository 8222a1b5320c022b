"""bench.py's multi-rank path on the CPU: two gloo ranks on 127.0.0.1, each
timing a replica; the job time is the slowest rank's and the value counts
the cells of every rank."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    dist.barrier()
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, dist)
    q.put((rank, ms, bench.whole_job_value(1000, 3, ms, world)))
    dist.destroy_process_group()


def test_two_ranks_take_the_slowest_time_and_sum_the_work():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, value in out:
        assert ms == 15.0
        assert abs(value - 1000 * 3 / 15e-3 / 1e6 * 2) < 1e-9
