"""Statistical parity of production mode with the reference's algorithm.

The GPU engine and the C oracle (the reference's arithmetic and random
stream) run independent seeds of the same problem and ladder.  Per
temperature, the mean energy after burn-in and the exchange acceptance of
each neighbouring pair must agree within 3 sigma of their seed-to-seed
spread (at most one of all comparisons beyond 3 sigma, none beyond 4.5).
Both production exchange orders are checked.  On small instances the best
energy found must equal the oracle's best.

The larger shapes -- the +-J L=20 lattice on the C1 ladder (32 temperatures),
a 1000-site +-1 graph and the C2 shape (N=2000, M=19990, 64 temperatures),
all with ICM on -- compare against oracle statistics committed in
tests/golden/stats_*.json (made by tests/golden/make_stats.py: 16 seeds of
long oracle runs).  They run the block-team kernel (one replica per block,
the layout of the C1/C2 workloads) and, where the replicas fit, several
replicas per block with warp or block-wide ICM teams.  Mean energies are
compared at the temperatures where the reference algorithm is at
equilibrium over the window (its two halves agree): the engine's
colour-class sweeps and the reference's sequential sweeps share the
stationary distribution but not the relaxation, and the coldest
temperatures of the glassy C2 instance still relax after 64000 steps.  The
lowest energy of the 16 GPU runs must reach the reference runs' best.
"""
import json
import math
import os

import numpy as np
import pytest

from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

G = os.path.join(os.path.dirname(__file__), "golden", "graphs")
SEEDS = 12
BURN = 800


def _oracle_runs(path, nt, T0, T1, pts, icm):
    means, rates = [], []
    for s in range(SEEDS):
        o = O.solve(O.Problem.load(path, 100 + s), seed=100 + s, Nt=nt, pts=pts, icm=icm, T0=T0, T1=T1, trace=True)
        se = o["trace"]["step_energy"]          # [pts, 2nt] slot energies after the sweeps
        means.append(se[BURN:].reshape(-1, 2, nt).mean(axis=(0, 1)))
        att = o["swap_attempts"].astype(float)
        suc = o["swap_successes"].astype(float)
        rates.append((suc[:nt - 1] + suc[nt:2 * nt - 1]) / np.maximum(att[:nt - 1] + att[nt:2 * nt - 1], 1))
    return np.array(means), np.array(rates)


def _gpu_runs(path, nt, T0, T1, pts, icm, exchange):
    import pticm
    prob = pticm.Problem.load(path)
    beta = pticm.beta_linspace(T0, T1, nt)
    means, rates = [], []
    for s in range(SEEDS):
        ctx = pticm.Context(prob, nt=nt, seed=500 + s, icm=icm, exchange=exchange)
        ctx.set_ladder(beta)
        ctx.init_states(500 + s)
        ctx.enable_energy_histograms(BURN)
        ctx.run(pts)
        h, e = ctx.energy_histograms()
        m = (h * e[None, :]).sum(axis=1) / h.sum(axis=1)
        means.append(m.reshape(2, nt).mean(axis=0))
        _, att, suc = ctx.stats()
        att = att.astype(float)
        suc = suc.astype(float)
        rates.append((suc[:nt - 1] + suc[nt:2 * nt - 1]) / np.maximum(att[:nt - 1] + att[nt:2 * nt - 1], 1))
    return np.array(means), np.array(rates)


def _agree(a, b):
    diff = a.mean(axis=0) - b.mean(axis=0)
    sig = np.sqrt(a.var(axis=0, ddof=1) / len(a) + b.var(axis=0, ddof=1) / len(b)) + 1e-12
    z = np.abs(diff) / sig
    return z


@pytest.mark.parametrize("exchange", [1, 0])
@pytest.mark.parametrize("g,nt,T0,T1,icm", [("pmL10.gset", 8, 0.5, 3.0, True), ("rnd60_pm", 8, 0.5, 3.0, True),
                                             ("rnd200_w1", 10, 0.5, 15.0, False)])
def test_energy_and_acceptance_match_reference_algorithm(g, nt, T0, T1, icm, exchange):
    path = os.path.join(G, g)
    pts = 3000
    om, orate = _oracle_runs(path, nt, T0, T1, pts, icm)
    gm, grate = _gpu_runs(path, nt, T0, T1, pts, icm, exchange)
    z = np.concatenate([_agree(gm, om), _agree(grate, orate)])
    assert (z > 3.0).sum() <= 1, z
    assert z.max() < 4.5, z


@pytest.mark.parametrize("g,nt,T0,T1", [("pmL10.gset", 8, 0.5, 3.0), ("rnd60_pm", 8, 0.5, 3.0),
                                         ("rnd200_w1", 12, 0.5, 15.0), ("lin40.ising", 8, 0.5, 3.0),
                                         ("ferroL12.gset", 10, 0.5, 3.5)])
def test_best_energy_matches_reference_on_small_instances(g, nt, T0, T1):
    import pticm
    path = os.path.join(G, g)
    best_ref = min(O.solve(O.Problem.load(path, s), seed=s, Nt=nt, pts=600, icm=True, T0=T0, T1=T1)["best_energy"]
                   for s in range(1, 4))
    prob = pticm.Problem.load(path)
    out = pticm.solve(prob, seed=11, Nt=nt, pts=3000, T0=T0, T1=T1, icm=True)
    assert out["best_energy"] == best_ref
    E, cut = prob.evaluate(out["best_state"][None, :])
    assert E[0] == out["best_energy"]


STATS = os.path.join(os.path.dirname(__file__), "golden")


def _fixture(name):
    with open(os.path.join(STATS, f"stats_{name}.json")) as f:
        return json.load(f)


def _fixture_graph(name, fx, tmp_path):
    import hashlib
    if name in ("c2", "c5_hot"):
        from pticm import instances
        g = fx["config"]["graph"]
        path = getattr(instances, g)().write_gset(str(tmp_path / g))
    else:
        path = os.path.join(G, fx["config"]["graph"])
    with open(path, "rb") as f:
        assert hashlib.sha256(f.read()).hexdigest() == fx["graph_sha256"], "not the graph the oracle ran"
    return path


def _gpu_block_runs(path, c, seeds, exchange, rpb):
    import pticm
    prob = pticm.Problem.load(path)
    nt = c["nt"]
    beta = pticm.beta_linspace(c["T0"], c["T1"], nt)
    means, rates, nc, lay, best = [], [], None, None, []
    for s in range(seeds):
        ctx = pticm.Context(prob, nt=nt, seed=900 + s, icm=True, exchange=exchange, replicas_per_block=rpb)
        ctx.set_ladder(beta)
        ctx.init_states(900 + s)
        ctx.enable_energy_histograms(c["burn"])
        ctx.run(c["pts"])
        assert ctx.verify() == 0
        lay = ctx.layout()
        h, e = ctx.energy_histograms()
        m = (h * e[None, :]).sum(axis=1) / h.sum(axis=1)
        means.append(m.reshape(2, nt).mean(axis=0))
        st, att, suc = ctx.stats()
        nc = st.nc
        att = att.astype(float)
        suc = suc.astype(float)
        rates.append((suc[:nt - 1] + suc[nt:2 * nt - 1]) / np.maximum(att[:nt - 1] + att[nt:2 * nt - 1], 1))
        best.append(ctx.best()[0])
    return np.array(means), np.array(rates), nc, lay, np.array(best)


@pytest.mark.parametrize("exchange", [1, 0])
@pytest.mark.parametrize("name,rpb", [("pmL20_c1", 1), ("pmL20_c1", 8), ("rnd200_w1", 1), ("rnd200_w1", 4),
                                      ("rnd1000_pm", 1), ("rnd1000_pm", 4), ("c2", 1), ("c5_hot", 1), ("c5_hot", 4)])
def test_block_layouts_match_oracle_statistics(name, rpb, exchange, tmp_path):
    fx = _fixture(name)
    c = fx["config"]
    path = _fixture_graph(name, fx, tmp_path)
    gm, grate, nc, lay, gbest = _gpu_block_runs(path, c, 16, exchange, rpb)
    assert nc == fx["nc"], "ICM pairs differ from the reference's count"
    assert nc > 0 or name == "c5_hot"
    assert lay.replicas_per_block == rpb
    if rpb == 1:
        assert lay.block_team == 1, "one replica per block runs the block-team kernel"
    if name == "c5_hot":
        assert lay.state_mode == 1, "the C5 graph runs in the large-instance layout (fields gathered)"
    om = np.array(fx["mean_energy"])
    orate = np.array(fx["acceptance"])
    # equilibrium temperatures: the reference algorithm's mean energies over
    # the two halves of the window agree (the coldest temperatures of the
    # glassy C2 instance are still relaxing); pairs of two such temperatures
    eq = np.array(fx["half_window_z"]) < 3.0
    assert eq.sum() >= (0.5 if name == "c2" else 0.85) * len(eq), "too few equilibrated temperatures"
    eq_pairs = eq[:-1] & eq[1:]
    z = _agree(gm[:, eq], om[:, eq])
    # Acceptance is compared in both exchange orders where the instance
    # equilibrates (at equilibrium every swap preserves the product
    # distribution, so no attempt order changes it).  The C2 instance still
    # relaxes over the window, and the even/odd order carries replicas
    # through the ladder faster than the reference's shuffled order, so its
    # acceptance there is compared only in the reference's own order.
    if not (name == "c2" and exchange == 1):
        z = np.concatenate([z, _agree(grate[:, eq_pairs], orate[:, eq_pairs])])
    # the best energy of the reference algorithm's runs is reached (not at the
    # paramagnetic end of C5, where the best is a chance low of hot states)
    if name != "c5_hot":
        assert gbest.min() <= min(fx["best_energy"]), (gbest, fx["best_energy"])
    allowed = max(1, math.ceil(0.02 * len(z)))
    assert (z > 3.0).sum() <= allowed, (np.round(z, 2), allowed)
    assert z.max() < 4.5, np.round(z, 2)
