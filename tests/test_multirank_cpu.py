"""The benchmark's multi-rank bookkeeping (replicas, one grid per rank) with
two gloo ranks on the CPU: the job's time is the slowest rank's, and the job's
rate counts every rank's cells."""
import os

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.max_over_ranks(1.0 + rank, world)          # rank 1 is the slow one
    rate = bench.job_rate(100, 10, world, t)
    q.put((rank, t, rate, bench.dist_env()[:2]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_take_the_slowest_time_and_sum_the_work():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, rate, env in out:
        assert t == 2.0 and rate == 100 * 10 * 2 / 2.0 and env == (rank, 2)


def test_one_rank_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5 and bench.job_rate(8, 2, 1, 4.0) == 4.0
