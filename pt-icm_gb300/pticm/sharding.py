"""Instance sharding over several GPUs (replicas only: no data-path collective).

A batch of independent instances (the batched workload, the folder mode, the
pilot runs of the learned ladder) splits over N GPUs by instance: each rank
builds a pticm.Batch of its own share and runs it alone; nothing crosses
GPUs while the PT steps run.  At the end the per-instance results are
gathered on rank 0 with one object gather over the process group (gloo or
NCCL), outside the timed data path.

The reference has no instance-level parallelism (one problem per process,
src/main.cc:15-209); its replica partition over MPI ranks
(src/solver.cc:22-30, src/initialization.cc:128-136) gives each rank a
contiguous block of replicas of one instance.  Here the unit is a whole
instance, and the shares are balanced by cost: the instances are taken in
order of decreasing cost and each goes to the rank with the least cost so
far (longest-processing-time-first), so the slowest rank, which sets the
job's time, carries at most 4/3 of the optimum.
"""
from __future__ import annotations

import heapq


def instance_cost(n: int, m: int, replicas: int) -> float:
    """Work of one PT step of an instance: its replicas' site visits and
    adjacency entries (2 + 6 * degree bytes per visit in the sweep)."""
    return float(replicas) * (2.0 * n + 12.0 * m)


def partition(costs, world: int):
    """Shares of `world` ranks: a list per rank of instance indices, in
    increasing index order.  Deterministic (ties by index, then rank)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    heap = [(0.0, r) for r in range(world)]
    shares = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        shares[r].append(i)
        heapq.heappush(heap, (load + float(costs[i]), r))
    return [sorted(s) for s in shares]


def share_loads(costs, shares):
    return [sum(float(costs[i]) for i in s) for s in shares]


def gather_results(local: dict, world: int, dist=None):
    """Per-instance results of every rank merged on every rank: `local` maps
    instance index -> result on this rank; the merged dict holds every
    instance once (ranks must hold disjoint indices)."""
    if dist is None or world == 1:
        return dict(local)
    parts = [None] * world
    dist.all_gather_object(parts, local)
    merged = {}
    for p in parts:
        for k, v in p.items():
            if k in merged:
                raise ValueError(f"instance {k} was run on two ranks")
            merged[k] = v
    return merged


def run_shard(problems, indices, *, nt, seed, steps, icm=True, exchange=1, beta=None, autotune_steps=20):
    """This rank's share of a batch: a pticm.Batch of problems[indices] on the
    current GPU, run for `steps` PT steps; returns {index: (best energy,
    accepted flips)} and the batch (for timing and statistics)."""
    import numpy as np
    import pticm
    if not indices:
        return {}, None
    mine = [problems[i] for i in indices]
    bat = pticm.Batch(mine, nt=nt, seed=seed, icm=icm, exchange=exchange)
    bat.set_ladders(pticm.beta_linspace(0.5, 3.0, nt) if beta is None else np.asarray(beta, np.float64))
    bat.init_states(seed + 1)
    if autotune_steps:
        bat.autotune(autotune_steps)
    bat.run(steps)
    best, flips = bat.best()
    return {i: (float(best[k]), int(flips[k])) for k, i in enumerate(indices)}, bat
