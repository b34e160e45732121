"""GPU parity tests of the PT-ICM engine against the C oracle.

* Philox4x32-10 on the device vs a numpy restatement and a published
  known-answer vector.
* Problem::energy / maxcut / calculate_dE on the device vs the oracle.
* Bit-exact from-scratch recompute of fields and energies after every phase
  (sweep, exchange, ICM) in both block layouts.
* Replay: the reference's sequential algorithm driven by the oracle's trace
  reproduces its final states, energies, flip and swap counts, per-slot
  exchange statistics and best state bit for bit.
"""
import json
import os

import numpy as np
import pytest

from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

G = os.path.join(os.path.dirname(__file__), "golden")
GRAPHS = os.path.join(G, "graphs")


@pytest.fixture(scope="module")
def pticm():
    import pticm as P
    P.lib()
    return P


def philox_np(ctr, key):
    c = [int(x) for x in ctr]
    k = [int(x) for x in key]
    M0, M1 = 0xD2511F53, 0xCD9E8D57
    for _ in range(10):
        p0 = M0 * c[0]
        p1 = M1 * c[2]
        c = [((p1 >> 32) ^ c[1] ^ k[0]) & 0xFFFFFFFF, p1 & 0xFFFFFFFF,
             ((p0 >> 32) ^ c[3] ^ k[1]) & 0xFFFFFFFF, p0 & 0xFFFFFFFF]
        k = [(k[0] + 0x9E3779B9) & 0xFFFFFFFF, (k[1] + 0xBB67AE85) & 0xFFFFFFFF]
    return c


def test_philox_device_matches_restatement(pticm):
    import ctypes as C
    rng = np.random.default_rng(0)
    cnt = 64
    ctr = rng.integers(0, 2**32, size=(cnt, 4), dtype=np.uint64).astype(np.uint32)
    key = rng.integers(0, 2**32, size=(cnt, 2), dtype=np.uint64).astype(np.uint32)
    ctr[0] = 0
    key[0] = 0
    out = np.zeros((cnt, 4), np.uint32)
    rc = pticm.lib().pticm_philox_probe(ctr.ctypes.data_as(C.c_void_p), key.ctypes.data_as(C.c_void_p),
                                        out.ctypes.data_as(C.c_void_p), cnt)
    assert rc == 0
    for i in range(cnt):
        assert out[i].tolist() == philox_np(ctr[i], key[i])
    # Random123 known answer for a zero counter and key
    assert out[0].tolist() == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]


GRAPH_FILES = ["pmL6.gset", "pmL10.gset", "pmL20_c1.gset", "rnd60_pm", "rnd200_w1", "lin40.ising",
               "ferroL12.gset"]


@pytest.mark.parametrize("g", GRAPH_FILES)
def test_evaluate_matches_oracle(pticm, g):
    path = os.path.join(GRAPHS, g)
    prob = pticm.Problem.load(path)
    orc = O.Problem.load(path, 0)
    n = orc.n
    rng = np.random.default_rng(1)
    states = rng.integers(0, 2, size=(5, n)).astype(np.uint8)
    E, cut, dE = prob.evaluate(states, with_dE=True)
    for k in range(5):
        Eo, dEo = orc.calculate_dE(states[k])
        assert E[k] == Eo == orc.energy(states[k])
        assert cut[k] == orc.maxcut(states[k])
        assert np.array_equal(dE[k], dEo)
    info = prob.info()
    assert info.char_scale == orc.char_scale
    assert bool(info.sparse) == orc.sparse


@pytest.mark.parametrize("algo", [0, 1, 3])   # auto (union-find), breadth-first, label propagation
@pytest.mark.parametrize("rpb", [0, 1])
@pytest.mark.parametrize("g,T0,T1,nt", [("pmL20_c1.gset", 0.5, 3.0, 32), ("rnd200_w1", 0.5, 15.0, 12),
                                         ("lin40.ising", 0.5, 3.0, 8), ("pmL6.gset", 0.5, 3.0, 6)])
def test_fields_exact_after_every_phase(pticm, g, T0, T1, nt, rpb, algo):
    prob = pticm.Problem.load(os.path.join(GRAPHS, g))
    ctx = pticm.Context(prob, nt=nt, seed=7, icm=True, replicas_per_block=rpb, icm_algo=algo)
    ctx.set_ladder(pticm.beta_linspace(T0, T1, nt))
    ctx.init_states(11)
    assert ctx.verify() == 0
    for _ in range(5):
        for ph in (pticm.PHASE_SWEEP, pticm.PHASE_EXCHANGE, pticm.PHASE_ICM):
            ctx.run(1, ph)
            assert ctx.verify() == 0
    ctx.run(50)
    assert ctx.verify() == 0
    s, E, f, slot = ctx.replicas()
    Ee, _ = prob.evaluate(s)
    assert np.array_equal(Ee, E.astype(np.float64))
    b, s2r, nc = ctx.ladder()
    assert sorted(s2r.tolist()) == list(range(2 * nt))
    for r in range(2 * nt):
        assert s2r[slot[r]] == r
    # exchange alone never moves a replica to the other chain
    ctx2 = pticm.Context(prob, nt=nt, seed=8, icm=True, replicas_per_block=rpb)
    ctx2.set_ladder(pticm.beta_linspace(T0, T1, nt))
    ctx2.init_states(12)
    ctx2.run(40, pticm.PHASE_SWEEP | pticm.PHASE_EXCHANGE)
    slot2 = ctx2.replicas()[3]
    for r in range(2 * nt):
        assert (slot2[r] >= nt) == (r >= nt)


def _golden_runs():
    with open(os.path.join(G, "ref_runs.json")) as f:
        return [r for r in json.load(f) if not r["args"].get("preprocess")]


@pytest.mark.parametrize("algo", [0, 1])   # the cluster is one set whichever search finds it
@pytest.mark.parametrize("k", range(len(_golden_runs())))
def test_replay_matches_reference_trajectory(pticm, k, algo):
    run = _golden_runs()[k]
    kw = dict(run["args"])
    path = os.path.join(GRAPHS, run["graph"])
    orc = O.solve(O.Problem.load(path, kw["seed"]), trace=True, **kw)
    tr = orc["trace"]
    nt = orc["Nt"]
    prob = pticm.Problem.load(path)
    ctx = pticm.Context(prob, nt=nt, seed=kw["seed"], sweeps=kw.get("sweeps", 1), icm=kw.get("icm", False),
                        icm_algo=algo)
    ctx.set_ladder(orc["beta"][:nt])
    ctx.set_states(tr["init_states"])
    ctx.replay(tr, kw["pts"])
    st, att, suc = ctx.stats()
    s, E, f, slot = ctx.replicas()
    assert np.array_equal(s, orc["states"])
    assert np.array_equal(E.astype(np.float64), orc["final_energy"])
    assert st.flips == orc["flips_u64"]
    assert st.swaps == orc["swaps"]
    assert att.tolist() == orc["swap_attempts"].tolist()
    assert suc.tolist() == orc["swap_successes"].tolist()
    Eb, sweep, bs, rep = ctx.best()
    assert Eb == orc["best_energy"]
    assert sweep == orc["best_sweep"]
    assert np.array_equal(bs, orc["best_state"])
    # and the reference's own printed report
    rep_ref = run["report"]
    assert rep_ref["num_of_flips"] == st.flips
    assert rep_ref["best_energy"] == Eb
    assert ctx.verify() == 0
