"""Regenerate the golden fixtures under tests/golden/.

Run here, where the reference sources exist (they do not travel to the GPU
host):

    python tests/golden/make_golden.py [REFERENCE_DIR]

It
  1. builds the unmodified reference single-rank (oracle/build_ref.sh),
  2. writes small seeded synthetic instances to tests/golden/graphs/,
  3. runs the reference CLI on each configuration and stores its printed
     report in tests/golden/ref_runs.json,
  4. compiles tests/golden/rng_kat.cc with the system g++ (the libstdc++ the
     reference's randomness comes from) and stores tests/golden/rng_kat.json.

The fixtures pin the C oracle (oracle/pticm_oracle.c) on any host.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "pt-icm_gb300"))

from oracle import pyoracle  # noqa: E402
from pticm import instances  # noqa: E402

GRAPHS = os.path.join(HERE, "graphs")

# (file name, instance factory)
INSTANCES = [
    ("pmL6.gset", lambda: instances.pm_lattice(6, seed=11)),            # dense (density 0.114)
    ("pmL10.gset", lambda: instances.pm_lattice(10, seed=12)),
    ("ferroL12.gset", lambda: instances.pm_lattice(12, seed=0, ferro=True)),
    ("pmL20_c1.gset", lambda: instances.pm_lattice(20, seed=1)),         # the C1 instance
    ("rnd60_pm", lambda: instances.random_graph(60, 150, seed=13, signed=True)),   # 1-based
    ("rnd200_w1", lambda: instances.random_graph(200, 1000, seed=14, signed=False)),
    ("lin40.ising", None),                                               # linear terms
]


def _lin40():
    import numpy as np
    inst = instances.random_graph(40, 90, seed=15, signed=True)
    rng = np.random.default_rng(15)
    inst.h = rng.choice(np.array([-1.0, 0.0, 1.0]), size=inst.n)
    return inst


RUNS = [
    # (graph, kwargs)
    ("pmL6.gset", dict(seed=1, Nt=6, pts=150, icm=True, T0=0.5, T1=3.0)),
    ("pmL10.gset", dict(seed=1, Nt=8, pts=200, icm=True, T0=0.5, T1=3.0)),
    ("pmL10.gset", dict(seed=2, Nt=9, pts=120, icm=False, T0=0.4, T1=2.5, sweeps=2)),
    ("pmL10.gset", dict(seed=3, Nt=8, pts=60, icm=True, T0=0.6, T1=2.8, preprocess=True,
                        pre_samples=300)),
    ("ferroL12.gset", dict(seed=4, Nt=10, pts=150, icm=True, T0=0.5, T1=3.5)),
    ("pmL20_c1.gset", dict(seed=1, Nt=32, pts=300, icm=True, T0=0.5, T1=3.0)),
    ("rnd60_pm", dict(seed=5, Nt=8, pts=200, icm=True, T0=0.5, T1=3.0)),
    ("rnd200_w1", dict(seed=6, Nt=12, pts=100, icm=True, T0=0.5, T1=15.0)),
    ("rnd200_w1", dict(seed=7, Nt=5, pts=80, icm=True, T0=0.3, T1=2.0, inverse=True)),
    ("lin40.ising", dict(seed=8, Nt=8, pts=150, icm=True, T0=0.5, T1=3.0)),
]


def main():
    ref_dir = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PTICM_REFERENCE_DIR")
    if not ref_dir:
        sys.exit("usage: make_golden.py REFERENCE_DIR (or set PTICM_REFERENCE_DIR)")
    subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh"), ref_dir])
    os.makedirs(GRAPHS, exist_ok=True)
    for fname, fac in INSTANCES:
        inst = _lin40() if fac is None else fac()
        inst.write_gset(os.path.join(GRAPHS, fname))
    runs = []
    for g, kw in RUNS:
        rep = pyoracle.run_reference(os.path.join(GRAPHS, g), **kw)
        runs.append(dict(graph=g, args=kw, report=rep))
        print(g, kw, "best", rep["best_energy"], "flips", rep["num_of_flips"])
    with open(os.path.join(HERE, "ref_runs.json"), "w") as f:
        json.dump(runs, f, indent=1)
    with tempfile.TemporaryDirectory() as td:
        exe = os.path.join(td, "rng_kat")
        subprocess.check_call(["g++", "-std=c++17", "-O2", "-o", exe, os.path.join(HERE, "rng_kat.cc")])
        out = subprocess.check_output([exe], text=True)
    kat = json.loads(out)
    with open(os.path.join(HERE, "rng_kat.json"), "w") as f:
        json.dump(kat, f, indent=1)
    print("wrote", len(runs), "reference runs and the RNG known answers")


if __name__ == "__main__":
    main()
