"""Writes tests/golden/lattice20_exact.json: the exact finite-size energy per
spin u(T) and specific heat c(T) of the periodic L=20 Ising ferromagnet that
the reference ships (data/lattice_2d_20_u.csv, data/lattice_2d_20_c.csv; the
graph is example_graphs/lattice_2d_20.gset), on its 0.01 temperature grid.

Run in a container that has the reference checked out:
    python tests/golden/make_lattice20_exact.py /path/to/reference
"""
import csv
import json
import os
import sys


def read(path):
    with open(path) as f:
        rows = list(csv.reader(f))
    return {round(float(r[0]), 2): float(r[1]) for r in rows[1:]}


def main(ref):
    u = read(os.path.join(ref, "data", "lattice_2d_20_u.csv"))
    c = read(os.path.join(ref, "data", "lattice_2d_20_c.csv"))
    T = sorted(set(u) & set(c))
    out = {"source": "data/lattice_2d_20_{u,c}.csv of the reference (exact, L=20 periodic ferromagnet)",
           "T": T, "u": [u[t] for t in T], "c": [c[t] for t in T]}
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lattice20_exact.json")
    with open(dst, "w") as f:
        json.dump(out, f)
    print(dst, len(T))


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PTICM_REFERENCE_DIR")
    if not ref:
        sys.exit("usage: make_lattice20_exact.py REFERENCE_DIR (or set PTICM_REFERENCE_DIR)")
    main(ref)
