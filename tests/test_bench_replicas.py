"""bench.py's host logic on the CPU: the replicas-only N>1 path on two gloo
ranks (the job time is the slowest rank's, the throughput counts every
rank's work), and the reference arm's JSON line (rank 0 prints it, other
ranks exit without work)."""
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


def _run_bench(args, env_extra=None):
    import subprocess
    env = dict(os.environ)
    env.update(env_extra or {})
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, cwd=ROOT, env=env,
                          capture_output=True, text=True, timeout=600)


def test_reference_arm_prints_one_contract_line():
    """`bench.py --impl reference` on a tiny sample: one JSON line with the
    contract's keys, the CPU baseline describing the run, e2e without copies."""
    import json
    r = _run_bench(["--impl", "reference", "--steps", "1", "--warmup", "0", "--ref-pts", "2"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["value"] > 0 and d["steps"] == 1 and d["higher_is_better"] is True
    assert "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["cores"] >= 1 and cb["kind"] in ("port", "reference") and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_exit_quietly():
    r = _run_bench(["--impl", "reference", "--steps", "1", "--warmup", "0", "--ref-pts", "2"], {"RANK": "1"})
    assert r.returncode == 0
    assert r.stdout.strip() == ""


class _FakeStats:
    def __init__(self, ms):
        self.last_run_ms = ms


class _FakeCtx:
    """Stands in for pticm.Context in bench.phase_split: run() records the
    phase mask, stats() reports a step time per mask, profile() returns
    per-phase milliseconds summed over the profiled steps."""

    NAMES = ("sweep", "barrier", "exchange", "icm", "total", "icm_diff", "icm_seed", "icm_union", "icm_flip",
             "icm_energy", "x_draw", "x_levels", "x_apply", "x_shuffle", "uf_link0", "uf_compress", "uf_link1",
             "uf_vote", "uf_outside", "uf_s_unions", "uf_size", "sweep_icm", "icm_pairs")

    def __init__(self):
        self.mask = 7
        self.steps = 0
        self.profiling = False

    def run(self, steps, mask=7):
        self.mask, self.steps = mask, steps

    def stats(self):
        us = {1: 10.0, 3: 12.0, 7: 20.0}[self.mask]
        return _FakeStats(us * self.steps / 1e3), None, None

    def set_profiling(self, on=True):
        self.profiling = on

    def profile(self):
        mean = {k: 0.0 for k in self.NAMES}
        mean.update(sweep=0.008 * self.steps, icm=0.004 * self.steps, uf_link0=0.001 * self.steps,
                    icm_pairs=0.5 * self.steps)
        return mean, dict(mean)


def test_phase_split_units():
    sys.path.insert(0, ROOT)
    import bench
    ctx = _FakeCtx()
    out = bench.phase_split(ctx, 200, 100)
    assert out["masked_us_per_step"] == pytest.approx({"sweep": 10.0, "sweep+exchange": 12.0, "all": 20.0})
    assert out["us_per_step"]["sweep"][0] == pytest.approx(8.0)       # 0.008 ms per step
    assert out["us_per_step"]["icm"][0] == pytest.approx(4.0)
    assert out["icm_pairs_per_block"] == pytest.approx(0.5)
    # per pair: 0.004 ms per step over 0.5 pairs per step
    assert out["us_per_icm_pair"]["icm"] == pytest.approx(8.0)
    assert out["us_per_icm_pair"]["uf_link0"] == pytest.approx(2.0)
    assert "x_draw" not in out["us_per_step"] and not ctx.profiling
