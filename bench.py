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

N_SPINS, M_EDGES, NT, T0, T1 = 2000, 19990, 64, 0.5, 15.0
PT_PER_STEP = 1000
METRIC = "spin-flip attempts/s"
WORKLOAD = ("random MaxCut N=2000 M=19990 w=+1 (seed 2), Nt=64 x 2 chains (R=128), "
            "T 0.5..15 linear in beta, ICM on, 1 sweep per PT step, 1000 PT steps per bench step")


def _graph():
    from pticm import instances
    return instances.c2()


def _profiled_traffic():
    """DRAM bytes per engine launch from the committed ncu summary."""
    try:
        with open(os.path.join(ROOT, "profiles", "pt_engine_c2_bench.md")) as f:
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


# ---------------------------------------------------------------- CPU legs
def _cpu_sample(args):
    """One oracle solve on a bounded sample of the workload (worker)."""
    seed, pts, path = args
    from oracle import pyoracle as O
    O.build()
    p = O.Problem.load(path, seed)
    t = time.perf_counter()
    O.solve(p, seed=seed, Nt=NT, pts=pts, icm=True, T0=T0, T1=T1)
    return time.perf_counter() - t


def _write_graph_tmp():
    import tempfile
    d = tempfile.mkdtemp(prefix="pticm_bench_")
    return _graph().write_gset(os.path.join(d, "c2"))   # no extension: 1-based like Gset


def cpu_baseline(pts=400):
    """Oracle port on one core: about 10 s of CPU work."""
    path = _write_graph_tmp()
    sec = _cpu_sample((1, pts, path))
    attempts = 2 * NT * N_SPINS * pts
    return {"value": attempts / sec, "unit": METRIC, "cores": 1, "kind": "port",
            "sample": f"{pts} PT steps of the workload (ICM on), one process, {sec:.2f} s"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from oracle import pyoracle as O
    O.build()
    path = _write_graph_tmp()
    cores = os.cpu_count() or 1
    pts = args.ref_pts
    ctx = mp.get_context("spawn")
    times = []
    with ctx.Pool(cores) as pool:
        for step in range(args.warmup + args.steps):
            t = time.perf_counter()
            pool.map(_cpu_sample, [(1000 + step * cores + i, pts, path) for i in range(cores)])
            dt = time.perf_counter() - t
            if step >= args.warmup:
                times.append(dt)
    total = sum(times)
    attempts = args.steps * cores * 2 * NT * N_SPINS * pts
    value = attempts / total
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "attempts/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000 * total / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD.replace("1000 PT steps per bench step",
                                                    f"{pts} PT steps per process per bench step"),
                       "parallelism": f"{cores} independent single-rank processes"},
            "cpu_baseline": {"value": value, "unit": "attempts/s", "cores": cores, "kind": "port",
                             "sample": f"{cores} processes x {pts} PT steps per bench step"},
            "e2e": {"value": value, "unit": "attempts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------- GPU leg
def run_gpu(args):
    import numpy as np
    import torch
    import pticm

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    inst = _graph()
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
    total_ms = sum(dev_ms)
    if dist:
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * attempts_per_step * args.steps / (total_ms / 1000.0)
    mism = ctx.verify()

    # end-to-end through the C ABI from host buffers, per step
    states_host = torch.empty((2 * NT, N_SPINS), dtype=torch.uint8).pin_memory()
    states_host.copy_(torch.from_numpy(np.random.default_rng(7 + rank).integers(0, 2, size=(2 * NT, N_SPINS), dtype=np.uint8)))
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
    line = {
        "metric": METRIC, "value": value, "unit": "attempts/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int8 spins, int32 fields/energies",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "l2": "flushed between steps (256 MB write)",
                   "replicas_per_gpu": 2 * NT, "ncolors": info.ncolors, "icm_pairs": ctx.ladder()[2],
                   "parallelism": "replicas only" if world > 1 else "1 GPU",
                   "wall_s": wall, "verify_mismatches_after": mism},
        "e2e": {"value": e2e_value, "unit": "attempts/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h),
                "what": "problem upload + ladder + initial states from pinned host memory + "
                        "1000 PT steps + best state/statistics read back, per step"},
        "gpu_launches": args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": _profiled_traffic(),
                     "note": f"algorithmic bytes 2N+12M per replica-sweep; peak {peak_kind} HBM copy; "
                             "data is shared-memory resident; traffic = ncu DRAM bytes per launch "
                             "(profiles/pt_engine_c2_bench.md)"},
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.cpu_pts)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--cpu-pts", type=int, default=400)
    ap.add_argument("--ref-pts", type=int, default=20)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
