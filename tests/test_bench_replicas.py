"""bench.py's replicas-only N>1 host logic on two gloo ranks (CPU): the job
time is the slowest rank's, the throughput counts every rank's work."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 100.0 + 50.0 * rank                      # rank 1 is the slow one
    m = bench.max_over_ranks(ms, dist, "cpu")
    v = bench.job_throughput(world, 1_000_000, m)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, m, v))


def test_max_over_ranks_and_job_throughput_gloo():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 1000)
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, m, v in out:
        assert m == 150.0
        assert v == pytest.approx(2 * 1_000_000 / 0.150)


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5) == 12.5
    assert bench.job_throughput(1, 10, 1000.0) == 10.0
