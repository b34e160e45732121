"""Throughput benchmark of the GB300 PT-ICM engine.

Workload (the configuration the spin-flip metric is quoted on): random
sparse MaxCut graph N=2000, M=19990 uniform distinct pairs, w=+1 (seed 2);
64 temperatures linear in beta for T=0.5..15; two replicas per temperature
(R=128); ICM on; one sweep per PT step.  One bench step = one persistent
engine launch of 1000 PT steps; 40 steps = the workload's 40000 PT steps.

metric  spin-flip attempts/s = R * N * sweeps * PT steps / device time
value   engine launches timed with CUDA events on the engine's own stream,
        inputs resident; L2 is flushed (256 MB write) between steps
e2e     the same metric through the C ABI from host buffers per step:
        problem upload, ladder, initial states from pinned host memory,
        the run, and the best state/energy/statistics read back
roofline  the sweep's algorithmic bytes 2N + 12M per replica-sweep
        (1 B spin read + 1 B write per site, 4 B column + 1 B coupling +
        1 B neighbour spin per adjacency entry) per launch / launch time,
        against the measured HBM copy bandwidth
cpu_baseline  the C oracle port of the reference (oracle/pticm_oracle.c)
        on one host core, on a bounded sample of the same workload

--impl reference times that CPU port on all host cores instead.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "pt-icm_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

PT_PER_STEP = 1000
METRIC = "spin-flip attempts/s"
WORKLOAD = ("random MaxCut N=2000 M=19990 w=+1 (seed 2), Nt=64 x 2 chains (R=128), "
            "T 0.5..15 linear in beta, ICM on, 1 sweep per PT step, 1000 PT steps per bench step")
C1_WORKLOAD = ("+-J toroidal lattice L=20 (N=400, M=800, seed 1), Nt=32 x 2 chains (R=64), "
               "T 0.5..3.0 linear in beta, ICM on, 1 sweep per PT step, 1000 PT steps per bench step")

# The single-instance workloads: graph, ladder, the reference arm's PT steps
# per process per bench step, and the ncu summary that holds the traffic.
SPECS = {
    "c2": dict(graph="c2", fname="c2", n=2000, m=19990, nt=64, T0=0.5, T1=15.0, workload=WORKLOAD, ref_pts=20,
               profile="pt_engine_c2_bench.md"),
    "c1": dict(graph="c1", fname="c1.gset", n=400, m=800, nt=32, T0=0.5, T1=3.0, workload=C1_WORKLOAD, ref_pts=200,
               profile="pt_engine_c1_bench.md"),
}
# PT steps the CPU legs run untimed before the timed window (the oracle's
# cost per step settles after a few hundred steps from the random start)
CPU_WARM_PTS = 300


def _graph(spec):
    from pticm import instances
    return getattr(instances, spec["graph"])()


def _profiled_traffic(summary):
    """DRAM bytes per engine launch from a committed ncu summary."""
    try:
        with open(os.path.join(ROOT, "profiles", summary)) as f:
            for line in f:
                if line.startswith("| traffic_bytes_per_launch |"):
                    return int(line.split("|")[2].strip())
    except (OSError, ValueError):
        pass
    return None


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------ replicas-only N>1
def max_over_ranks(value, dist=None, device="cpu"):
    """The largest of every rank's value (the job ends with its slowest
    rank); the value itself on one rank."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(world, units_per_rank, max_ms):
    """Whole-job throughput of `world` independent replicas that each did
    units_per_rank units, the job taking the slowest rank's time."""
    return world * units_per_rank / (max_ms / 1000.0)


def phase_split(ctx, steps, pt_per_call):
    """Where a PT step's time goes, after the timed region: the step time
    with phases left out (sweep only; sweep and exchange; all), then the
    in-kernel clock64 timers (pticm_set_profiling) over `steps` steps, us per
    PT step (mean and max over blocks) and, for the ICM phases, per pair."""
    out = {"masked_us_per_step": {}}
    for mask, name in ((1, "sweep"), (3, "sweep+exchange"), (7, "all")):
        ctx.run(pt_per_call, mask)
        out["masked_us_per_step"][name] = ctx.stats()[0].last_run_ms * 1e3 / pt_per_call
    ctx.set_profiling(True)
    ctx.run(steps)
    mean, mx = ctx.profile()
    ctx.set_profiling(False)
    pairs = max(mean["icm_pairs"], 1.0)
    out["steps"] = steps
    out["icm_pairs_per_block"] = mean["icm_pairs"] / steps
    out["us_per_step"] = {k: [round(mean[k] * 1e3 / steps, 3), round(mx[k] * 1e3 / steps, 3)]
                          for k in mean if k != "icm_pairs" and not k.startswith("x_")}
    out["us_per_icm_pair"] = {k: round(mean[k] * 1e3 / pairs, 3) for k in mean
                              if k.startswith(("icm", "uf")) and k != "icm_pairs"}
    return out


# ---------------------------------------------------------------- CPU legs
def _cpu_sample(args):
    """One oracle solve (worker): CPU_WARM_PTS + warm PT steps untimed, then
    `timed` PT steps timed inside the oracle's main loop."""
    seed, warm, timed, path, nt, T0, T1 = args
    from oracle import pyoracle as O
    O.build()
    p = O.Problem.load(path, seed)
    sec, _ = O.solve_timed(p, seed=seed, Nt=nt, pts=CPU_WARM_PTS + warm + timed, timed_from=CPU_WARM_PTS + warm,
                           icm=True, T0=T0, T1=T1)
    return sec


def _write_graph_tmp(spec):
    import tempfile
    d = tempfile.mkdtemp(prefix="pticm_bench_")
    return _graph(spec).write_gset(os.path.join(d, spec["fname"]))   # c2: no extension, 1-based like Gset


def cpu_baseline(spec, pts=300):
    """Oracle port on one core, timed over `pts` PT steps after CPU_WARM_PTS."""
    path = _write_graph_tmp(spec)
    sec = _cpu_sample((1, 0, pts, path, spec["nt"], spec["T0"], spec["T1"]))
    attempts = 2 * spec["nt"] * spec["n"] * pts
    return {"value": attempts / sec, "unit": METRIC, "cores": 1, "kind": "port",
            "sample": f"PT steps {CPU_WARM_PTS}..{CPU_WARM_PTS + pts} of the workload (ICM on; the first "
                      f"{CPU_WARM_PTS} untimed), one process, {sec:.2f} s timed"}


def run_reference(args, spec):
    """The reference algorithm's CPU implementation (the C oracle port) on
    every host core: one single-rank process per core, each running
    CPU_WARM_PTS + warmup*ref_pts PT steps untimed and then steps*ref_pts
    timed PT steps (its main loop timed inside the process; problem build
    and initialisation outside).  A bench step is ref_pts PT steps of every
    process; the job takes the slowest process's time."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from oracle import pyoracle as O
    O.build()
    path = _write_graph_tmp(spec)
    cores = os.cpu_count() or 1
    pts = args.ref_pts or spec["ref_pts"]
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        secs = pool.map(_cpu_sample, [(1000 + i, args.warmup * pts, args.steps * pts, path, spec["nt"], spec["T0"],
                                       spec["T1"]) for i in range(cores)])
    total = max(secs)
    attempts = args.steps * cores * 2 * spec["nt"] * spec["n"] * pts
    value = attempts / total
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "attempts/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000 * total / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": spec["workload"].replace("1000 PT steps per bench step",
                                                            f"{pts} PT steps per process per bench step"),
                       "parallelism": f"{cores} independent single-rank processes",
                       "untimed_pt_steps_per_process": CPU_WARM_PTS + args.warmup * pts},
            "cpu_baseline": {"value": value, "unit": "attempts/s", "cores": cores, "kind": "port",
                             "sample": f"{cores} processes x {args.steps * pts} timed PT steps after "
                                       f"{CPU_WARM_PTS + args.warmup * pts} untimed ones"},
            "e2e": {"value": value, "unit": "attempts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------- GPU leg
def run_gpu(args, spec):
    import numpy as np
    import torch
    import pticm
    N_SPINS, M_EDGES, NT, T0, T1 = spec["n"], spec["m"], spec["nt"], spec["T0"], spec["T1"]

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    inst = _graph(spec)
    prob = pticm.Problem.from_instance(inst)
    info = prob.info()
    beta = pticm.beta_linspace(T0, T1, NT)
    ctx = pticm.Context(prob, nt=NT, seed=1 + rank, icm=True)
    ctx.set_ladder(beta)
    ctx.init_states(1 + rank)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    attempts_per_step = 2 * NT * N_SPINS * PT_PER_STEP

    for _ in range(args.warmup):
        ctx.run(PT_PER_STEP)
    mism = ctx.verify()
    if mism:
        raise RuntimeError(f"verify found {mism} mismatches after warm-up")

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    dev_ms = []
    barrier()
    wall0 = time.perf_counter()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            ctx.run(PT_PER_STEP)
            st, _, _ = ctx.stats()
            dev_ms.append(st.last_run_ms)
    barrier()
    wall = time.perf_counter() - wall0
    total_ms = max_over_ranks(sum(dev_ms), dist, "cuda")
    value = job_throughput(world, attempts_per_step * args.steps, total_ms)
    mism = ctx.verify()
    if args.phases and rank == 0:
        print(json.dumps({"phase_split": phase_split(ctx, 2000, PT_PER_STEP)}), file=sys.stderr, flush=True)

    # end-to-end through the C ABI from host buffers, per step.  The input
    # states are the warmed-up replicas, each given to the replica that
    # starts at its temperature, so that the timed steps do the same
    # (equilibrium) work as the device-timed ones.
    s_now, _, _, slot_now = ctx.replicas()
    by_slot = np.empty_like(s_now)
    by_slot[slot_now] = s_now
    states_host = torch.empty((2 * NT, N_SPINS), dtype=torch.uint8).pin_memory()
    states_host.copy_(torch.from_numpy(by_slot))
    src = np.ascontiguousarray(inst.src, np.int32)
    dst = np.ascontiguousarray(inst.dst, np.int32)
    w = np.ascontiguousarray(inst.w, np.float64)
    h2d = src.nbytes + dst.nbytes + w.nbytes + beta.nbytes + states_host.numel()
    d2h = 0
    e2e_times = []
    for i in range(args.e2e_steps + 1):
        barrier()
        t0 = time.perf_counter()
        p2 = pticm.Problem.from_coo(inst.n, src, dst, w)
        c2 = pticm.Context(p2, nt=NT, seed=100 + i, icm=True)
        c2.set_ladder(beta)
        c2.set_states(states_host.numpy())
        c2.run(PT_PER_STEP)
        E, sweep, best, rep = c2.best()
        st2, att, suc = c2.stats()
        d2h = best.nbytes + 8 + 8 + att.nbytes + suc.nbytes + 64
        del c2, p2
        barrier()
        if i > 0:
            e2e_times.append(time.perf_counter() - t0)
    e2e_value = world * attempts_per_step / statistics.median(e2e_times)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0
    peak, peak_kind = _peaks()
    bytes_per_launch = (2 * N_SPINS + 12 * M_EDGES) * 2 * NT * PT_PER_STEP
    launch_s = (sum(dev_ms) / len(dev_ms)) / 1000.0
    achieved = bytes_per_launch / launch_s / 1e9
    smem_peak = pticm.smem_copy_rate(2000)
    lay = ctx.layout()
    line = {
        "metric": METRIC, "value": value, "unit": "attempts/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int8 spins, int32 fields/energies",
        "data": "synthetic",
        "config": {"workload": spec["workload"], "l2": "flushed between steps (256 MB write)",
                   "replicas_per_gpu": 2 * NT, "ncolors": info.ncolors, "icm_pairs": ctx.ladder()[2],
                   "layout": {"replicas_per_block": lay.replicas_per_block, "blocks": lay.blocks,
                              "threads": lay.threads, "block_team": lay.block_team},
                   "parallelism": "replicas only" if world > 1 else "1 GPU",
                   "wall_s": wall, "verify_mismatches_after": mism},
        "e2e": {"value": e2e_value, "unit": "attempts/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h),
                "what": "problem upload + ladder + initial states (the warmed-up replicas) from pinned host "
                        "memory + 1000 PT steps + best state/statistics read back, per step"},
        "gpu_launches": args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": _profiled_traffic(spec["profile"]),
                     "note": f"algorithmic bytes 2N+12M per replica-sweep; peak {peak_kind} HBM copy; "
                             "data is shared-memory resident; traffic = ncu DRAM bytes per launch "
                             f"(profiles/{spec['profile']})"},
        "roofline_smem": {"achieved": achieved, "peak": smem_peak, "unit": "GB/s", "frac": achieved / smem_peak,
                          "note": "the same algorithmic bytes against the shared-memory copy rate measured in "
                                  "this run (pticm_smem_copy_rate: one block per SM, read + written bytes), the "
                                  "tier the replicas and the staged adjacency live in"},
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(spec, args.cpu_pts)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


BATCH_COUNT, BATCH_NT, BATCH_PT_PER_STEP = 1024, 32, 100
BATCH_WORKLOAD = ("1024 uneven instances in one persistent launch: 512 +-J toroidal lattices L in {10,20,32,50}, "
                  "512 random +-1 graphs N log-uniform 200..5000, mean degree U[3,20] (seeds 1000+i); "
                  "Nt=32 x 2 chains (R=64) each, T 0.5..3.0 linear in beta, ICM on, groups autotuned, "
                  "100 PT steps of every instance per bench step")


def run_gpu_batched(args):
    """The batched workload: spin-flip attempts/s over all instances."""
    import numpy as np
    import torch
    import pticm
    from pticm import instances as I

    from pticm import sharding as SH

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    t_gen = time.perf_counter()
    all_insts = I.batch_mix(args.batch_count)
    # N GPUs: the instances are split by cost (pticm.sharding), each rank runs
    # its share as a batch of its own; nothing crosses GPUs while it runs
    costs = [SH.instance_cost(x.n, x.m, 2 * BATCH_NT) for x in all_insts]
    share = SH.partition(costs, world)[rank]
    insts = [all_insts[i] for i in share]
    probs = [pticm.Problem.from_instance(x) for x in insts]
    t_gen = time.perf_counter() - t_gen
    total_sites = sum(x.n for x in all_insts) * 2 * BATCH_NT
    beta = pticm.beta_linspace(0.5, 3.0, BATCH_NT)
    bat = pticm.Batch(probs, nt=BATCH_NT, seed=1, icm=True, exchange=1)
    bat.set_ladders(beta)
    bat.init_states(2)
    t_tune = time.perf_counter()
    bat.autotune(20)
    t_tune = time.perf_counter() - t_tune
    sites = sum(x.n for x in insts) * 2 * BATCH_NT
    bytes_per_sweep = sum(2 * x.n + 12 * x.m for x in insts) * 2 * BATCH_NT
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        bat.run(BATCH_PT_PER_STEP)
    if bat.verify():
        raise RuntimeError("verify found mismatches after warm-up")
    dev_ms = []
    launches0 = bat.info().launches

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    barrier()
    wall0 = time.perf_counter()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            bat.run(BATCH_PT_PER_STEP)
            dev_ms.append(bat.info().last_run_ms)
    barrier()
    launches = bat.info().launches - launches0
    wall = time.perf_counter() - wall0
    info = bat.info()
    total_ms = max_over_ranks(sum(dev_ms), dist, "cuda")
    value = total_sites * BATCH_PT_PER_STEP * args.steps / (total_ms / 1000.0)
    mism = bat.verify()
    g, t_us, staged, teams = bat.groups()
    # end to end: problems from host edge lists, ladders, states, the run and
    # the per-instance best energies back, per step
    e2e_t = []
    h2d = sum(x.src.nbytes + x.dst.nbytes + x.w.nbytes for x in insts) + beta.nbytes * len(insts)
    # problems are built on all host cores (the C ABI releases the GIL and
    # problem construction is thread-safe)
    import concurrent.futures as cf
    pool = cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 1)
    for i in range(args.e2e_steps):
        barrier()
        t0 = time.perf_counter()
        ps = list(pool.map(lambda x: pticm.Problem.from_coo(x.n, x.src, x.dst, x.w), insts))
        b2 = pticm.Batch(ps, nt=BATCH_NT, seed=50 + i, icm=True, exchange=1)
        b2.set_ladders(beta)
        b2.init_states(60 + i)
        b2.run(BATCH_PT_PER_STEP)
        best, flips = b2.best()
        del b2, ps
        barrier()
        e2e_t.append(max_over_ranks(time.perf_counter() - t0, dist, "cuda"))
    # the per-instance results of every rank, gathered after the timed runs
    results = SH.gather_results({i: (float(e), int(f)) for i, e, f in zip(share, *bat.best())}, world, dist)
    if rank != 0:
        dist.destroy_process_group()
        return 0
    if len(results) != len(all_insts):
        raise RuntimeError("sharded run lost instances")
    peak, peak_kind = _peaks()
    launch_s = sum(dev_ms) / 1000.0 / args.steps   # this rank's launches and its share's bytes
    achieved = bytes_per_sweep * BATCH_PT_PER_STEP / launch_s / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "attempts/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "strong", "vs_baseline": None, "dtype": "int8 spins, int32 fields/energies", "data": "synthetic",
        "config": {"workload": BATCH_WORKLOAD if args.batch_count == BATCH_COUNT else
                   BATCH_WORKLOAD.replace("1024 uneven", f"{args.batch_count} uneven"),
                   "instances": len(all_insts), "instances_rank0": len(insts), "sites_per_sweep": total_sites,
                   "parallelism": f"instances split over {world} GPUs by cost (replicas only)" if world > 1
                   else "1 GPU",
                   "l2": "flushed between steps (256 MB write); the working set also exceeds L2",
                   "lanes": info.lanes, "jobs": info.jobs, "chunk_pt_steps": info.chunk, "smem_bytes": info.smem_bytes,
                   "predicted_makespan_us_per_pt_step": info.makespan_us,
                   "groups": {str(k): int(v) for k, v in zip(*np.unique(g, return_counts=True))},
                   "staged_instances": int(staged.sum()), "autotune_s": t_tune, "generate_s": t_gen,
                   "wall_s": wall, "verify_mismatches_after": mism},
        "e2e": {"value": total_sites * BATCH_PT_PER_STEP / statistics.median(e2e_t), "unit": "attempts/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": 16 * len(insts),
                "what": "all problems from host edge lists (colouring on all host cores) + ladders + states + "
                        "100 PT steps + per-instance best energies back"},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None,
                     "note": f"algorithmic bytes 2N+12M per replica-sweep summed over instances; peak {peak_kind}"},
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


LARGE_WORKLOAD = ("random +-1 MaxCut graph N=20000, mean degree 40 (M=400000, seed 5), 128 temperatures linear "
                  "in beta for T 0.5..9.5 x 4 replicas per temperature, ICM on; four replicas per block with their "
                  "spins and the cluster search's scratch in shared memory, fields gathered at each visit, "
                  "adjacency and overlap lists in device memory; 20 PT steps per bench step")


def run_gpu_large(args):
    import numpy as np
    import torch
    import pticm
    from pticm import instances as I

    from pticm import surrogate as S

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    inst = I.c5()
    prob = pticm.Problem.from_instance(inst)
    info = prob.info()
    # the ladder: 128 temperatures from the surrogate network, checked by a
    # short PT run, with the multihistogram ladder as fallback (the learned
    # ladder); ascending in beta, so that ICM takes the coldest slots
    t_lad = time.perf_counter()
    lad_info = None
    if args.large_ladder == "linear":
        beta = pticm.beta_linspace(0.5, 9.5, 128)
    else:
        if args.ladder_net:
            net = S.load(args.ladder_net)
        else:
            recs = S.make_records(I.ladder_mix(args.large_train, seed0=100), nt=32, burn_in=1000, samples=2000,
                                  seed=3)
            net, _ = S.train(recs, steps=3000, batch=1024, lr=1e-3, seed=1)
        beta, lad_info = S.learned_ladder(prob, net, 0.5, 9.5, 128, seed=21)
        beta = np.sort(np.asarray(beta, np.float64))
    t_lad = time.perf_counter() - t_lad
    NTL = len(beta)
    ctx = pticm.Context(prob, nt=NTL, chains=4, seed=1, icm=True)
    ctx.set_ladder(beta)
    ctx.init_states(2)
    steps_per = 20
    for _ in range(args.warmup):
        ctx.run(steps_per)
    if ctx.verify():
        raise RuntimeError("verify found mismatches after warm-up")
    dev_ms = []
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            ctx.run(steps_per)
            dev_ms.append(ctx.stats()[0].last_run_ms)
    total_ms = sum(dev_ms)
    if args.phases:
        print(json.dumps({"phase_split": phase_split(ctx, 40, steps_per)}), file=sys.stderr, flush=True)
    sites = 4 * NTL * inst.n
    value = sites * steps_per * args.steps / (total_ms / 1000.0)
    mism = ctx.verify()
    # end to end from host buffers: the problem from its edge list, the
    # ladder, the warmed-up replicas as initial states (each to the replica
    # that starts at its temperature), 100 PT steps, best state and
    # statistics back
    s_now, _, _, slot_now = ctx.replicas()
    by_slot = np.empty_like(s_now)
    by_slot[slot_now] = s_now
    states_host = torch.from_numpy(by_slot).pin_memory()
    src = np.ascontiguousarray(inst.src, np.int32)
    dst = np.ascontiguousarray(inst.dst, np.int32)
    w = np.ascontiguousarray(inst.w, np.float64)
    e2e_pt = 100
    h2d = src.nbytes + dst.nbytes + w.nbytes + beta.nbytes + states_host.numel()
    d2h = 0
    e2e_t = []
    for i in range(args.e2e_steps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        p2 = pticm.Problem.from_coo(inst.n, src, dst, w)
        c2 = pticm.Context(p2, nt=NTL, chains=4, seed=100 + i, icm=True)
        c2.set_ladder(beta)
        c2.set_states(states_host.numpy())
        c2.run(e2e_pt)
        E, sweep, best, rep = c2.best()
        st2, att, suc = c2.stats()
        d2h = best.nbytes + 16 + att.nbytes + suc.nbytes + 64
        del c2, p2
        torch.cuda.synchronize()
        if i > 0:
            e2e_t.append(time.perf_counter() - t0)
    peak, peak_kind = _peaks()
    bytes_per_sweep = (2 * inst.n + 12 * inst.m) * 4 * NTL
    achieved = bytes_per_sweep * steps_per / (total_ms / 1000.0 / args.steps) / 1e9
    lay = ctx.layout()
    workload = LARGE_WORKLOAD if args.large_ladder == "linear" else LARGE_WORKLOAD.replace(
        "128 temperatures linear in beta for T 0.5..9.5", f"{NTL} temperatures of the learned ladder for T 0.5..9.5")
    line = {"metric": METRIC, "value": value, "unit": "attempts/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int8 spins, int32 fields/energies",
            "data": "synthetic", "config": {"workload": workload, "ncolors": info.ncolors,
                                            "icm_pairs": int(ctx.ladder()[2]), "verify_mismatches_after": mism,
                                            "l2": "flushed between steps (256 MB write)",
                                            "layout": {"replicas_per_block": lay.replicas_per_block,
                                                       "blocks": lay.blocks, "threads": lay.threads,
                                                       "state_mode": lay.state_mode},
                                            "ladder": {"kind": args.large_ladder, "temperatures": NTL,
                                                       "beta_min": float(beta.min()), "beta_max": float(beta.max()),
                                                       "setup_s": t_lad,
                                                       "fallback": None if lad_info is None else int(lad_info.fallback),
                                                       "checks": None if lad_info is None else int(lad_info.rounds),
                                                       "mean_abs_acceptance_deviation": None if lad_info is None
                                                       else float(lad_info.mean_deviation),
                                                       "network": args.ladder_net or
                                                       f"trained in this run on {args.large_train} pilot instances"}},
            "e2e": {"value": sites * e2e_pt / statistics.median(e2e_t), "unit": "attempts/s",
                    "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "what": f"problem from its edge list (colouring on the host) + ladder + the warmed-up replicas "
                            f"from pinned host memory + {e2e_pt} PT steps + best state/statistics back, per step"},
            "gpu_launches": args.steps,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": _profiled_traffic("pt_engine_large_c5.md"),
                         "note": f"algorithmic bytes 2N+12M per replica-sweep; peak {peak_kind}; traffic = ncu DRAM "
                                 "bytes per launch (profiles/pt_engine_large_c5.md)"},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    return 0


LADDER_WORKLOAD = ("learned ladder: 4x256 SiLU MLP (BF16 weights, FP32 accumulate) on instance features + E/W, "
                   "trained on FP64 multihistogram ln g of synthetic instances (+-J lattices L 6..50, +-1 random "
                   "graphs N 100..3000, mean degree 3..20); evaluated on held-out instances: ln g error, ladder "
                   "acceptance (r=0.4, 32 temperatures), ladder cost and time-to-target vs the multihistogram ladder")


def _tmpdir():
    import tempfile
    global _TMP
    try:
        return _TMP
    except NameError:
        _TMP = tempfile.mkdtemp(prefix="pticm_bench_")
        return _TMP


def _gset_digest(inst, fname):
    """SHA-256 of the instance written in Gset layout (1-based, no extension)."""
    import hashlib
    path = inst.write_gset(os.path.join(_tmpdir(), fname))
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def _ttt_runs(prob, ladder, target, copies, chunk, max_steps, seed):
    """PT with ICM on `copies` independent copies of one instance in one
    batch: the step at which each copy's best energy first reaches target."""
    import numpy as np
    import pticm
    lad = np.sort(np.asarray(ladder))           # ascending: ICM on the coldest (as --sort-ladder)
    bat = pticm.Batch([prob] * copies, nt=len(lad), seed=seed, icm=True, exchange=1)
    bat.set_ladders(lad)
    bat.init_states(seed + 1)
    hit = np.full(copies, -1, np.int64)
    done = 0
    while done < max_steps and (hit < 0).any():
        bat.run(chunk)
        done += chunk
        best, _ = bat.best()
        newly = (hit < 0) & (best <= target)
        hit[newly] = done
    ctx = pticm.Context(prob, nt=len(lad), seed=seed + 2, icm=True)
    ctx.set_ladder(lad)
    ctx.init_states(seed + 3)
    ctx.run(50)
    ctx.run(400)
    ms_per_step = ctx.stats()[0].last_run_ms / 400
    return hit, ms_per_step


def run_gpu_ladder(args):
    import numpy as np
    import torch
    import pticm
    from pticm import instances as I, surrogate as S

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    log = (lambda *a: print(*a, file=sys.stderr, flush=True))
    t0 = time.perf_counter()
    train = I.ladder_mix(args.ladder_train, seed0=100)
    held = I.ladder_mix(args.ladder_held, seed0=900000)
    t_gen = time.perf_counter() - t0
    t0 = time.perf_counter()
    recs = S.make_records(train, nt=32, burn_in=1000, samples=2000, seed=3, log=log)
    t_data = time.perf_counter() - t0
    hrec = S.make_records(held, nt=32, burn_in=1000, samples=2000, seed=4, log=log)
    t0 = time.perf_counter()
    m, losses = S.train(recs, steps=4000, batch=1024, lr=1e-3, seed=1, log=log)
    t_train = time.perf_counter() - t0
    n_rows = len(S.training_arrays(recs)[1])
    dev = lambda a: float(np.mean(np.abs(a - 0.4)))
    rows = []
    errs = [S.lng_error(pticm.Problem.from_instance(x), m, r)[1] for x, r in zip(held, hrec)]
    for i, (x, r) in enumerate(zip(held[:args.ladder_eval], hrec[:args.ladder_eval])):
        p = pticm.Problem.from_instance(x)
        T0, T1 = S.pilot_range(x)
        err = errs[i]
        t = time.perf_counter()
        bs = S.surrogate_ladder(p, m, T0, T1, 32)
        t_s = time.perf_counter() - t
        t = time.perf_counter()
        bl, info = S.learned_ladder(p, m, T0, T1, 32, seed=11 + i)
        t_l = time.perf_counter() - t
        t = time.perf_counter()
        bm = pticm.cae_ladder(p, seed=5 + i, T0=T0, T1=T1, nt=32)
        t_m = time.perf_counter() - t
        a_s = S.ladder_acceptance(p, bs, steps=2000, burn_in=500, seed=7 + i)
        a_l = S.ladder_acceptance(p, bl, steps=2000, burn_in=500, seed=7 + i)
        a_m = S.ladder_acceptance(p, bm, steps=2000, burn_in=500, seed=7 + i)
        rows.append(dict(n=x.n, err=err, t_s=t_s, t_l=t_l, t_m=t_m, fb=int(info.fallback), d_s=dev(a_s), d_l=dev(a_l),
                         d_m=dev(a_m), sd_s=float(a_s.std()), sd_l=float(a_l.std()), sd_m=float(a_m.std()),
                         len_l=len(bl), len_m=len(bm)))
    col = lambda k: np.array([q[k] for q in rows], np.float64)
    # time to target on a subset of held-out instances
    ttt = []
    targets = {}
    tpath = os.path.join(ROOT, "tests", "golden", "ttt_targets.json")
    if os.path.exists(tpath) and args.ladder_held == 256:
        with open(tpath) as f:
            for d in json.load(f)["instances"]:
                # the instance the oracle ran (same generator output, same file)
                if _gset_digest(held[d["index"]], f"t{d['index']}") == d["graph_sha256"]:
                    targets[d["index"]] = d["target"]
    cand = [i for i, x in enumerate(held) if args.ttt_min_n <= x.n <= args.ttt_max_n][:args.ttt_count]
    clk = ClockSampler(0).__enter__()      # clocks over the time-to-target runs
    for i in cand:
        x = held[i]
        p = pticm.Problem.from_instance(x)
        T0, T1 = S.pilot_range(x)
        t = time.perf_counter()
        bm = pticm.cae_ladder(p, seed=50 + i, T0=T0, T1=T1, nt=32)
        t_m = time.perf_counter() - t
        t = time.perf_counter()
        bl, info = S.learned_ladder(p, m, T0, T1, 32, seed=60 + i)
        t_l = time.perf_counter() - t
        t = time.perf_counter()
        bs = S.surrogate_ladder(p, m, T0, T1, 32)
        t_s = time.perf_counter() - t
        # target: the best energy the reference algorithm reached (the C oracle,
        # four long runs on its linear ladder; tests/golden/ttt_targets.json),
        # else the best of a long multihistogram-laddered run of 32 copies
        if i in targets:
            target, tsrc = targets[i], "reference algorithm (oracle), best of 4 x 10000 PT steps"
        else:
            tb = pticm.Batch([p] * 32, nt=len(bm), seed=80 + i, icm=True, exchange=1)
            tb.set_ladders(np.sort(bm))
            tb.init_states(81 + i)
            tb.run(args.ttt_target_steps)
            target, tsrc = float(tb.best()[0].min()), "32 copies of a multihistogram-laddered GPU run"
            del tb
        res = {"n": x.n, "name": x.name, "target": target, "target_source": tsrc}
        for nm, lad, tl in (("mhist", bm, t_m), ("learned", bl, t_l), ("surrogate", bs, t_s)):
            hit, msps = _ttt_runs(p, lad, target, args.ttt_copies, args.ttt_chunk, args.ttt_max_steps, 90 + i)
            ok = hit >= 0
            q = float(np.quantile(np.where(ok, hit, np.inf), 0.99))
            res[nm] = {"ladder_s": tl, "temps": len(lad), "ms_per_step": msps, "success": float(ok.mean()),
                       "steps_q99": q if np.isfinite(q) else None,
                       "ttt99_s": (tl + q * msps / 1000.0) if np.isfinite(q) else None}
        res["learned_fallback"] = int(info.fallback)
        ttt.append(res)
        log(json.dumps(res))
    clk.__exit__(None, None, None)
    # the network's GEMM on the tensor cores at an inference-sized shape
    import ctypes as C
    L = pticm.lib()
    L.pticm_tc_gemm_bench.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    gemm = {}
    for (M_, N_, K_) in ((65536, 256, 256), (1024, 256, 256)):
        ms_, tf_ = C.c_double(), C.c_double()
        if L.pticm_tc_gemm_bench(M_, N_, K_, 20, C.byref(ms_), C.byref(tf_)) == 0:
            gemm[f"{M_}x{N_}x{K_}"] = {"ms": ms_.value, "tflops": tf_.value}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            bf16_peak, peak_kind = float(json.load(f)["bf16_tflops"]), "measured"
    except Exception:
        bf16_peak, peak_kind = 1900.0, "fallback"

    def gmean_speedup(name):
        both = [t for t in ttt if t["mhist"]["ttt99_s"] and t[name]["ttt99_s"]]
        sp = [t["mhist"]["ttt99_s"] / t[name]["ttt99_s"] for t in both]
        return float(np.exp(np.mean(np.log(sp)))) if sp else None

    line = {
        "metric": "time-to-target energy at 99% run success, surrogate vs multihistogram ladder",
        "value": gmean_speedup("surrogate"), "unit": "x (geometric mean of multihistogram TTT99 / surrogate TTT99)",
        "learned_speedup": gmean_speedup("learned"),
        "higher_is_better": True, "n_gpus": 1, "data": "synthetic",
        "dtype": "bf16 network, fp64 multihistogram", "config": {"workload": LADDER_WORKLOAD,
        "train_instances": len(train), "held_out": len(held), "acceptance_evaluated": len(rows),
        "training_rows": n_rows, "generate_s": t_gen,
        "training_data_s": t_data, "train_s": t_train, "final_loss": float(losses[-50:].mean())},
        "lng_error_per_spin": {"mean": float(np.mean(errs)), "median": float(np.median(errs)),
                               "p90": float(np.quantile(errs, 0.9)), "instances": len(errs)},
        "acceptance_mean_abs_dev": {"surrogate": float(col("d_s").mean()), "learned": float(col("d_l").mean()),
                                    "multihistogram": float(col("d_m").mean())},
        "acceptance_std": {"surrogate": float(col("sd_s").mean()), "learned": float(col("sd_l").mean()),
                           "multihistogram": float(col("sd_m").mean())},
        "fallback_rate": float(col("fb").mean()),
        "ladder_seconds": {"surrogate_mean": float(col("t_s").mean()), "learned_mean": float(col("t_l").mean()),
                           "learned_accepted_mean": float(col("t_l")[col("fb") == 0].mean()) if (col("fb") == 0).any() else None,
                           "multihistogram_mean": float(col("t_m").mean())},
        "time_to_target": ttt,
        "clocks": clk.summary(),
        "roofline": {"bound": "tensor", "kernel": "tc_gemm_tma_kernel (TMA loads, tcgen05 MMA, BF16, FP32 accumulate)",
                     "achieved": gemm.get("65536x256x256", {}).get("tflops"), "peak": bf16_peak, "unit": "TFLOP/s",
                     "frac": (gemm.get("65536x256x256", {}).get("tflops") or 0.0) / bf16_peak,
                     "note": f"one 256x256 layer of the network on 65536 rows; peak {peak_kind} cuBLAS bf16",
                     "shapes": gemm},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--cpu-pts", type=int, default=300)
    ap.add_argument("--ref-pts", type=int, default=0, help="reference arm: PT steps per process per bench step "
                    "(0: the workload's default, 20 for c2, 200 for c1)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="c2", choices=["c2", "c1", "batched", "ladder", "large"],
                    help="c2: the headline single-instance workload; c1: the +-J L=20 lattice; batched: 1024 "
                         "uneven instances; ladder: the learned temperature ladder; large: N=20000, R=512")
    ap.add_argument("--batch-count", type=int, default=BATCH_COUNT)
    ap.add_argument("--large-ladder", default="learned", choices=["learned", "linear"],
                    help="large workload: the learned ladder (surrogate + checks + multihistogram fallback, the "
                         "workload's definition) or 128 temperatures linear in beta")
    ap.add_argument("--large-train", type=int, default=1024,
                    help="large workload: pilot instances the in-run surrogate network trains on")
    ap.add_argument("--ladder-net", default="", help="a saved surrogate network (pticm_mlp_save) to use instead")
    ap.add_argument("--ladder-train", type=int, default=4096)
    ap.add_argument("--ladder-held", type=int, default=256)
    ap.add_argument("--ladder-eval", type=int, default=64)
    ap.add_argument("--ttt-count", type=int, default=32)
    ap.add_argument("--ttt-min-n", type=int, default=200)
    ap.add_argument("--ttt-max-n", type=int, default=3000)
    ap.add_argument("--ttt-copies", type=int, default=100)
    ap.add_argument("--ttt-chunk", type=int, default=50)
    ap.add_argument("--ttt-max-steps", type=int, default=10000)
    ap.add_argument("--ttt-target-steps", type=int, default=10000)
    ap.add_argument("--phases", action="store_true",
                    help="c2/c1/large: after the timed region, print where a PT step's time goes (JSON, stderr)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args, SPECS.get(args.workload, SPECS["c2"]))
    if args.workload == "batched":
        return run_gpu_batched(args)
    if args.workload == "ladder":
        return run_gpu_ladder(args)
    if args.workload == "large":
        return run_gpu_large(args)
    return run_gpu(args, SPECS[args.workload])


if __name__ == "__main__":
    sys.exit(main())
