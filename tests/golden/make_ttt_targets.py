"""Time-to-target targets for the learned-ladder benchmark (bench.py --workload
ladder): the best energy the reference algorithm reaches on each of 32
held-out instances of the learned-ladder workload.

The C oracle (the reference's algorithm and random stream, pinned to the
reference build) runs solve() with ICM on the reference's own ladder -- 32
temperatures linear in beta over the instance's pilot range -- for `pts` PT
steps, four seeds per instance; the target is the lowest best energy of the
four runs (gather_best_energy_values, src/mpi_utils.cc:103-163).  The
instances are the first 32 of the held-out set (ladder_mix(256,
seed0=900000)) with 200 <= N <= 3000.  Written to ttt_targets.json.

    python tests/golden/make_ttt_targets.py [--procs P] [--pts PTS]
"""
import argparse
import hashlib
import json
import multiprocessing as mp
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "pt-icm_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

HELD_COUNT, HELD_SEED0 = 256, 900000
MIN_N, MAX_N, COUNT, SEEDS = 200, 3000, 32, 4


def held_out():
    from pticm import instances as I
    held = I.ladder_mix(HELD_COUNT, seed0=HELD_SEED0)
    return [(i, x) for i, x in enumerate(held) if MIN_N <= x.n <= MAX_N][:COUNT]


def _one(args):
    idx, seed, pts, path, T0, T1 = args
    from oracle import pyoracle as O
    o = O.solve(O.Problem.load(path, seed), seed=seed, Nt=32, pts=pts, icm=True, T0=T0, T1=T1)
    return idx, seed, float(o["best_energy"])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--procs", type=int, default=os.cpu_count())
    ap.add_argument("--pts", type=int, default=10000)
    args = ap.parse_args()
    from pticm import surrogate as S
    scratch = os.path.join(HERE, "_scratch")
    os.makedirs(scratch, exist_ok=True)
    jobs, meta = [], {}
    for idx, x in held_out():
        path = x.write_gset(os.path.join(scratch, f"ttt_{idx}"))     # 1-based
        with open(path, "rb") as f:
            digest = hashlib.sha256(f.read()).hexdigest()
        T0, T1 = S.pilot_range(x)
        meta[idx] = dict(index=idx, name=x.name, n=x.n, m=x.m, T0=T0, T1=T1, graph_sha256=digest)
        jobs += [(idx, 1000 + s, args.pts, path, T0, T1) for s in range(SEEDS)]
    jobs.sort(key=lambda j: -meta[j[0]]["n"])          # the longest first
    ctx = mp.get_context("spawn")
    with ctx.Pool(args.procs) as pool:
        res = pool.map(_one, jobs, chunksize=1)
    for idx, seed, best in res:
        meta[idx].setdefault("best_by_seed", {})[str(seed)] = best
    out = []
    for idx in sorted(meta):
        d = meta[idx]
        d["target"] = min(d["best_by_seed"].values())
        out.append(d)
    with open(os.path.join(HERE, "ttt_targets.json"), "w") as f:
        json.dump(dict(made_by="tests/golden/make_ttt_targets.py (C oracle solve, ICM on, linear ladder, 32 "
                               "temperatures over the pilot range)", pts=args.pts, seeds=SEEDS, instances=out), f,
                  indent=1)
    print(len(out), "targets")


if __name__ == "__main__":
    main()
