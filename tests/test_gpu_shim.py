"""Code written in the reference's shape reproduces the reference's run.

tests/shim_driver.cc is written against the libreplica interface this
library keeps (pt-icm_gb300/host/pticm_gb300.hh): the main loop of the
reference's solve() (src/solver.cc:67-127) over Replica::sweep,
try_replica_exchange and icm, and the pilot loop of get_beta's gather_samples
(src/cae_estimator.cc:76-140).  It is compiled with g++ against the shim
archive and the native library; its sweeps, overlaps and cluster searches
run on the GPU while the host draws from the same std::mt19937_64 as the
reference.  For the same seed it must print what the oracle (pinned to the
reference build) computes, bit for bit: swap counts, best energy, sweep and
state, flip and swap totals, and every replica's final state and energy;
and, for the pilot loop, the same energy samples at every temperature.
"""
import os
import subprocess

import numpy as np
import pytest

from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PKG = os.path.join(ROOT, "pt-icm_gb300", "pticm")
G = os.path.join(HERE, "golden", "graphs")


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    import pticm
    from pticm import _build
    pticm.lib()
    _build.build_shim()
    exe = str(tmp_path_factory.mktemp("drv") / "shim_driver")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                           "-I", os.path.join(ROOT, "pt-icm_gb300", "host"), os.path.join(HERE, "shim_driver.cc"),
                           os.path.join(PKG, "libpticm_shim.a"), "-L", PKG, "-lpticm_gb300",
                           "-Wl,-rpath," + PKG, "-o", exe])
    return exe


def _run(exe, *args):
    out = subprocess.run([exe] + [str(a) for a in args], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    return out.stdout.splitlines()


def _parse_solve(lines):
    d, reps = {}, {}
    for ln in lines:
        if ln.startswith("replica "):
            _, r, e, bits = ln.split()
            reps[int(r)] = (float(e), np.frombuffer(bits.encode(), np.uint8) - ord("0"))
            continue
        k, v = ln.split(":", 1)
        d[k] = v.strip()
    return d, reps


@pytest.mark.parametrize("g,seed,nt,pts,icm,T0,T1,sweeps", [
    ("pmL10.gset", 3, 8, 40, 1, 0.5, 3.0, 1),
    ("rnd60_pm", 5, 8, 40, 1, 0.5, 3.0, 1),
    ("lin40.ising", 8, 8, 30, 1, 0.5, 3.0, 1),
    ("pmL6.gset", 2, 6, 30, 1, 0.4, 2.5, 1),
    ("rnd200_w1", 6, 6, 25, 1, 0.5, 15.0, 2),
    ("ferroL12.gset", 4, 10, 30, 0, 0.5, 3.5, 1),
])
def test_reference_shaped_solve_loop_matches_the_oracle(driver, g, seed, nt, pts, icm, T0, T1, sweeps):
    path = os.path.join(G, g)
    d, reps = _parse_solve(_run(driver, "solve", path, seed, nt, pts, icm, T0, T1, sweeps))
    o = O.solve(O.Problem.load(path, seed), seed=seed, Nt=nt, pts=pts, sweeps=sweeps, icm=bool(icm), T0=T0, T1=T1)
    R = 2 * nt
    assert int(d["nc"]) == o["Nc"]
    assert [int(x) for x in d["swap_attempts"].split()] == o["swap_attempts"][:R].tolist()
    assert [int(x) for x in d["swap_successes"].split()] == o["swap_successes"][:R].tolist()
    assert float(d["best_energy"]) == o["best_energy"]
    assert int(d["best_sweep"]) == o["best_sweep"]
    assert float(d["best_maxcut"]) == o["best_maxcut"]
    assert int(d["num_of_flips"]) == o["flips_u64"]
    assert int(d["num_of_swaps"]) == o["swaps"]
    best = np.frombuffer(d["best_state"].encode(), np.uint8) - ord("0")
    assert np.array_equal(best, o["best_state"])
    for r in range(R):
        e, s = reps[r]
        assert e == o["final_energy"][r], f"replica {r} energy"
        assert np.array_equal(s, o["states"][r]), f"replica {r} state"
    assert d["incremental_dE_matches"] == "1"


@pytest.mark.parametrize("g,seed,nt,samples,burn", [("pmL10.gset", 2, 6, 60, 40), ("rnd60_pm", 7, 5, 50, 30)])
def test_reference_shaped_pilot_loop_matches_the_oracle(driver, g, seed, nt, samples, burn):
    path = os.path.join(G, g)
    T0, T1 = 0.5, 3.0
    lines = _run(driver, "pilot", path, seed, nt, samples, burn, T0, T1)
    # the pilot ladder of get_beta (src/cae_estimator.cc:308-328)
    b0, b1 = max(1 / T0, 1 / T1), min(1 / T0, 1 / T1)
    step = (b1 - b0) / (nt - 1)
    hb, b = [], b0
    for _ in range(nt):
        hb.append(b)
        b += step
    p = O.pilot(O.Problem.load(path, seed), seed=seed, hist_betas=np.array(hb), estep=2.0, samples=samples,
                burn_in=burn)
    for j, ln in enumerate(lines):
        _, jj, n, s, s2, lo, hi = ln.split()
        row = p["hist"][int(p["hist_off"][j]):int(p["hist_off"][j] + p["hist_len"][j])]
        E = p["emin"][j] + 2.0 * np.arange(len(row))
        assert int(n) == int(row.sum()) == samples
        assert float(s) == float((row * E).sum())
        assert float(s2) == float((row * E * E).sum())
        assert float(lo) == p["emin"][j] and float(hi) == p["emax"][j]
