"""Instance sharding over GPUs (pticm.sharding) on the CPU: the partition
covers every instance once and balances the ranks' cost, and the per-instance
results of two gloo ranks merge into the full set on every rank.  No GPU: the
per-instance work of a rank is stood in by a host computation on its share."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "pt-icm_gb300")


def _costs(count=256):
    sys.path.insert(0, PKG)
    from pticm import instances as I
    from pticm import sharding as S
    insts = I.batch_mix(count)
    return insts, [S.instance_cost(x.n, x.m, 64) for x in insts]


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_partition_covers_every_instance_once_and_balances(world):
    from pticm import sharding as S
    _, costs = _costs()
    shares = S.partition(costs, world)
    assert len(shares) == world
    flat = sorted(i for s in shares for i in s)
    assert flat == list(range(len(costs)))
    loads = S.share_loads(costs, shares)
    # longest-processing-time-first: within 4/3 of the lower bound of the optimum
    bound = max(sum(costs) / world, max(costs))
    assert max(loads) <= 4.0 / 3.0 * bound + 1e-6
    assert S.partition(costs, world) == shares   # deterministic


def test_partition_edge_cases():
    from pticm import sharding as S
    assert S.partition([], 3) == [[], [], []]
    assert S.partition([5.0], 2) == [[0], []]
    assert S.partition([1.0, 1.0, 1.0, 1.0], 2) == [[0, 2], [1, 3]]
    with pytest.raises(ValueError):
        S.partition([1.0], 0)


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, PKG)
    from pticm import sharding as S
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    insts, costs = _costs(64)
    share = S.partition(costs, world)[rank]
    local = {i: float(np.abs(insts[i].w).sum()) for i in share}   # this rank's "results"
    merged = S.gather_results(local, world, dist)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, share, merged))


def test_two_gloo_ranks_gather_every_instance():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29700 + (os.getpid() % 1000)
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    insts, _ = _costs(64)
    want = {i: float(np.abs(x.w).sum()) for i, x in enumerate(insts)}
    (r0, s0, m0), (r1, s1, m1) = out
    assert set(s0).isdisjoint(s1) and sorted(s0 + s1) == list(range(64))
    assert m0 == want and m1 == want


def test_gather_refuses_an_instance_on_two_ranks():
    from pticm import sharding as S

    class FakeDist:
        @staticmethod
        def all_gather_object(parts, local):
            parts[0] = {1: 0.0}
            parts[1] = {1: 0.0}

    with pytest.raises(ValueError):
        S.gather_results({1: 0.0}, 2, FakeDist)
