"""Pins of the C oracle (oracle/pticm_oracle.c).

* against libstdc++ known answers for the random facilities the reference
  draws from (tests/golden/rng_kat.json, made by tests/golden/rng_kat.cc);
* against the reports of the unmodified reference built single-rank
  (tests/golden/ref_runs.json, made by tests/golden/make_golden.py);
* live against that reference build when it exists on this host (random
  graphs, and dense, --preprocess, multi-sweep, inverse-temperature,
  linear-term and larger configurations).
"""
import json
import os

import numpy as np
import pytest

from oracle import pyoracle as O

G = os.path.join(os.path.dirname(__file__), "golden")


def _kat():
    with open(os.path.join(G, "rng_kat.json")) as f:
        return json.load(f)


def test_mt64_known_answers():
    L = O.lib()
    import ctypes as C
    g = (C.c_uint64 * 313)()
    L.orc_mt64_seed(g, 5489)
    v = 0
    for _ in range(10000):
        v = L.orc_mt64_next(g)
    kat = _kat()
    assert str(v) == kat["mt64_default_10000th"] == "9981545732273789042"
    L.orc_mt64_seed(g, 12345)
    assert [str(L.orc_mt64_next(g)) for _ in range(8)] == kat["mt64_seed12345_first8"]


def test_canonical_bernoulli_known_answers():
    import ctypes as C
    L = O.lib()
    kat = _kat()
    g = (C.c_uint64 * 313)()
    L.orc_mt64_seed(g, 7)
    got = [L.orc_canonical(g) for _ in range(16)]
    assert got == kat["canonical_seed7_first16"]
    L.orc_mt64_seed(g, 99)
    assert [int(L.orc_canonical(g) < 0.5) for _ in range(64)] == kat["bernoulli_seed99_first64"]


def test_shuffle_sample_known_answers():
    import ctypes as C
    L = O.lib()
    kat = _kat()
    g = (C.c_uint64 * 313)()
    L.orc_mt64_seed(g, 2024)
    for n, want in zip([1, 2, 3, 7, 8, 31, 63, 64], kat["shuffle_seed2024"]):
        a = np.arange(n, dtype=np.uint32)
        L.orc_shuffle_u32(a.ctypes.data_as(C.c_void_p), n, g)
        assert a.tolist() == want
    L.orc_mt64_seed(g, 31337)
    for n, idx in kat["sample1_seed31337"]:
        assert L.orc_sample_one(n, g) == idx


def _runs():
    with open(os.path.join(G, "ref_runs.json")) as f:
        return json.load(f)


def _compare(rep, o):
    assert rep["num_of_flips"] == o["flips"]
    assert rep["num_of_swaps"] == o["swaps"]
    assert rep["best_energy"] == o["best_energy"]
    assert rep["best_state_energy"] == o["best_state_energy"]
    assert rep["best_maxcut"] == o["best_maxcut"]
    assert rep["best_state_sweep"] == o["best_sweep"]
    assert rep["best_state"] == o["best_state"].tolist()
    assert rep["swap_attempts"] == o["swap_attempts"].tolist()
    assert rep["swap_successes"] == o["swap_successes"].tolist()
    nt = o["Nt"]
    assert np.allclose(rep["ladder"], o["beta"][:nt], rtol=0, atol=5e-7)


@pytest.mark.parametrize("k", range(len(_runs())))
def test_oracle_matches_reference_reports(k):
    run = _runs()[k]
    kw = dict(run["args"])
    p = O.Problem.load(os.path.join(G, "graphs", run["graph"]), kw["seed"])
    o = O.solve(p, **kw)
    _compare(run["report"], o)


@pytest.mark.skipif(not O.have_reference(), reason="reference build absent on this host")
@pytest.mark.parametrize("seed", [21, 22, 23])
def test_oracle_matches_reference_live(seed, tmp_path):
    from pticm import instances
    inst = instances.random_graph(80, 240, seed=seed, signed=True)
    path = inst.write_gset(str(tmp_path / f"g{seed}"))
    kw = dict(seed=seed, Nt=6 + seed % 3, pts=120, icm=True, T0=0.4, T1=3.0)
    rep = O.run_reference(path, **kw)
    o = O.solve(O.Problem.load(path, seed), **kw)
    _compare(rep, o)


LIVE_CASES = [
    # (instance factory, file name, solve arguments)
    ("lattice6_dense_pre", lambda I: I.pm_lattice(6, seed=31), "l6.gset",
     dict(seed=31, Nt=6, pts=80, icm=True, T0=0.5, T1=3.0, preprocess=True, pre_samples=200)),
    ("lattice8_sweeps3", lambda I: I.pm_lattice(8, seed=32), "l8.gset",
     dict(seed=32, Nt=7, pts=90, icm=False, T0=0.4, T1=2.6, sweeps=3)),
    ("random_inverse", lambda I: I.random_graph(120, 500, seed=33, signed=True), "r120",
     dict(seed=33, Nt=6, pts=100, icm=True, T0=0.3, T1=2.5, inverse=True)),
    ("random500_deg10", lambda I: I.random_graph(500, 2500, seed=34, signed=False), "r500",
     dict(seed=34, Nt=10, pts=60, icm=True, T0=0.5, T1=10.0)),
    ("linear_terms", None, "lin.ising",
     dict(seed=35, Nt=6, pts=100, icm=True, T0=0.5, T1=3.0)),
]


def _linear_instance(I):
    inst = I.random_graph(50, 120, seed=35, signed=True)
    inst.h = np.random.default_rng(35).choice(np.array([-2.0, -1.0, 0.0, 1.0, 2.0]), size=inst.n)
    return inst


@pytest.mark.skipif(not O.have_reference(), reason="reference build absent on this host")
@pytest.mark.parametrize("case", LIVE_CASES, ids=[c[0] for c in LIVE_CASES])
def test_oracle_matches_reference_live_configurations(case, tmp_path):
    """Dense and sparse files, --preprocess, several sweeps, inverse
    temperatures, linear terms and a larger graph, each run by the reference
    build and by the oracle with the same seed."""
    from pticm import instances as I
    _, fac, fname, kw = case
    inst = _linear_instance(I) if fac is None else fac(I)
    path = inst.write_gset(str(tmp_path / fname))
    rep = O.run_reference(path, **kw)
    o = O.solve(O.Problem.load(path, kw["seed"]), **kw)
    _compare(rep, o)


def test_beta_linspace_accumulates_like_reference():
    b = O.beta_linspace(0.5, 3.0, 32)
    assert b[0] == 1 / 3.0
    step = (1 / 0.5 - 1 / 3.0) / 31
    acc = 1 / 3.0
    for i in range(32):
        assert b[i] == acc
        acc += step
