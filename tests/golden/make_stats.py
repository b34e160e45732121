"""Oracle statistics for the statistical parity tests (tests/test_gpu_stats.py).

Runs the C oracle (the reference's sequential algorithm and random stream,
pinned to the reference build) for several seeds of each configuration and
stores, per seed, the per-temperature mean energy after the burn-in (slot
energies after the sweeps of each step, both chains merged) and the exchange
acceptance of every neighbouring pair (both chains merged), as the GPU test
computes them.  Only equilibrium statistics are comparable: the engine's
colour-class sweeps and the reference's sequential sweeps share the
stationary distribution but relax at different rates.  So the fixture also
stores, per temperature, how far the mean energies of the two halves of the
window are apart (half_window_z, in units of their seed-to-seed spread); the
coldest temperatures of the glassy C2 instance are still relaxing after
64000 steps, and the tests compare only the temperatures where the two
halves agree.  The
runs are long at the C2 shape (16 ms a PT step on one core), so they are
made once here and committed as stats_<name>.json.

Configurations:
  pmL20_c1    +-J lattice L=20 (N=400), 32 temperatures T 0.5..3.0 (the C1 ladder), ICM
  rnd200_w1   random N=200 graph, w=+1, 10 temperatures T 0.5..15, ICM
  rnd1000_pm  random N=1000, M=5000 graph, +-1, 24 temperatures T 0.5..5, ICM
  c2          random N=2000, M=19990 graph, w=+1, 64 temperatures T 0.5..15, ICM (the C2 shape)
  c5_hot      the C5 graph (N=20000, M=400000, +-1), 6 temperatures T 6..9.5: the paramagnetic end of
              the C5 ladder, run in the large-instance layout (its ICM temperatures, T <= 1, lie deep
              in the glass phase and do not equilibrate in reach of the oracle)

    python tests/golden/make_stats.py [name ...] [--procs P]
"""
import argparse
import hashlib
import json
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "pt-icm_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

SEEDS = 16

CONFIGS = {
    "pmL20_c1": dict(graph="pmL20_c1.gset", nt=32, T0=0.5, T1=3.0, pts=30000, burn=15000),
    "rnd200_w1": dict(graph="rnd200_w1", nt=10, T0=0.5, T1=15.0, pts=8000, burn=4000),
    "rnd1000_pm": dict(graph="rnd1000_pm", nt=24, T0=0.5, T1=5.0, pts=16000, burn=8000),
    "c2": dict(graph="c2", nt=64, T0=0.5, T1=15.0, pts=64000, burn=32000),
    "c5_hot": dict(graph="c5", nt=6, T0=6.0, T1=9.5, pts=4000, burn=2000),
}


def graph_path(name, scratch):
    """Committed golden graphs, or the seeded C2 / C5 instances written to `scratch`."""
    if name in ("c2", "c5"):
        from pticm import instances
        return getattr(instances, name)().write_gset(os.path.join(scratch, name))   # 1-based, like Gset
    return os.path.join(HERE, "graphs", name)


def file_digest(path):
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def _one(args):
    name, path, seed = args
    from oracle import pyoracle as O
    c = CONFIGS[name]
    o = O.solve(O.Problem.load(path, seed), seed=seed, Nt=c["nt"], pts=c["pts"], icm=True, T0=c["T0"],
                T1=c["T1"], energies=True)
    nt = c["nt"]
    se = o["step_energy"][c["burn"]:]                       # [steps, 2 nt] by slot
    mean = se.reshape(-1, 2, nt).mean(axis=(0, 1))
    half = len(se) // 2                                     # the two halves of the window
    halves = [se[:half].reshape(-1, 2, nt).mean(axis=(0, 1)).tolist(),
              se[half:].reshape(-1, 2, nt).mean(axis=(0, 1)).tolist()]
    att = o["swap_attempts"].astype(float)
    suc = o["swap_successes"].astype(float)
    rate = (suc[:nt - 1] + suc[nt:2 * nt - 1]) / np.maximum(att[:nt - 1] + att[nt:2 * nt - 1], 1)
    return seed, mean.tolist(), rate.tolist(), float(o["best_energy"]), int(o["Nc"]), halves


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("names", nargs="*", default=list(CONFIGS))
    ap.add_argument("--procs", type=int, default=os.cpu_count())
    args = ap.parse_args()
    scratch = os.path.join(HERE, "_scratch")
    os.makedirs(scratch, exist_ok=True)
    ctx = mp.get_context("spawn")
    with ctx.Pool(args.procs) as pool:
        for name in args.names:
            c = CONFIGS[name]
            path = graph_path(c["graph"], scratch)
            seeds = list(range(100, 100 + SEEDS))
            res = sorted(pool.map(_one, [(name, path, s) for s in seeds]))
            # equilibrium check: the mean energies of the two halves of the
            # measuring window must agree (seed-to-seed spread)
            h0 = np.array([r[5][0] for r in res])
            h1 = np.array([r[5][1] for r in res])
            zh = np.abs(h0.mean(0) - h1.mean(0)) / (np.sqrt(h0.var(0, ddof=1) / len(h0) +
                                                            h1.var(0, ddof=1) / len(h1)) + 1e-12)
            out = dict(config=c, graph_sha256=file_digest(path), seeds=[r[0] for r in res],
                       mean_energy=[r[1] for r in res], acceptance=[r[2] for r in res],
                       best_energy=[r[3] for r in res], nc=res[0][4],
                       half_window_z=zh.tolist(), half_window_z_max=float(zh.max()),
                       made_by="tests/golden/make_stats.py (C oracle, energies after the sweeps of each step)")
            with open(os.path.join(HERE, f"stats_{name}.json"), "w") as f:
                json.dump(out, f)
            print(name, "done; largest |z| between the window halves %.2f" % zh.max(), flush=True)


if __name__ == "__main__":
    main()
