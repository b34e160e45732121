"""Multihistogram ladder (src/cae_estimator.cc) against the C oracle.

CPU: the constant-acceptance walk (host code, O(nbins) acceptance) gives the
oracle's ladder (O(nbins^2) acceptance, the reference's arithmetic) on the
oracle's own pilot histograms and density of states.
GPU: the FP64 multihistogram fixed point matches the oracle's; the whole
GPU ladder places temperatures whose measured exchange acceptance is close
to the target, like the reference's.
"""
import os

import numpy as np
import pytest

from oracle import pyoracle as O

G = os.path.join(os.path.dirname(__file__), "golden", "graphs")


def _pilot(graph, seed=3, T0=0.6, T1=2.8, nt=8, samples=400, burn_in=300):
    prob = O.Problem.load(os.path.join(G, graph), seed)
    bs, be = 1 / T0, 1 / T1
    step = (be - bs) / (nt - 1)
    hb, b = [], bs
    for _ in range(nt):
        hb.append(b)
        b += step
    return O.pilot(prob, seed=seed, hist_betas=hb, samples=samples, burn_in=burn_in), bs, be


@pytest.mark.parametrize("graph", ["pmL10.gset", "rnd60_pm", "pmL20_c1.gset"])
def test_cae_walk_matches_oracle(graph):
    import pticm
    pl, bs, be = _pilot(graph)
    max_emax = float(pl["emax"].max())
    dos, z, it = O.partition_iterate(pl["hist"], pl["hist_off"], pl["hist_len"], pl["hist_betas"], pl["emin"], 2.0,
                                     pl["n"], max_emax)
    min_emin = float(pl["emin"].min())
    want = O.cae_walk(dos, min_emin, 2.0, bs, be, 0.1, 0.4, 8)
    got = pticm.cae_walk(dos, min_emin, 2.0, bs, be, 0.1, 0.4, 8)
    assert len(got) == len(want)
    assert np.allclose(got, want, rtol=1e-9, atol=0)


@pytest.mark.gpu
@pytest.mark.parametrize("graph", ["pmL10.gset", "rnd60_pm", "pmL20_c1.gset", "rnd200_w1"])
def test_mhist_dos_matches_oracle(graph):
    import pticm
    pl, bs, be = _pilot(graph)
    max_emax = float(pl["emax"].max())
    dos_o, z_o, it_o = O.partition_iterate(pl["hist"], pl["hist_off"], pl["hist_len"], pl["hist_betas"], pl["emin"],
                                           2.0, pl["n"], max_emax)
    dos_g, z_g, it_g = pticm.mhist_dos(pl["hist"], pl["hist_off"], pl["hist_len"], pl["hist_betas"], pl["emin"], 2.0,
                                       pl["n"], max_emax)
    assert len(dos_g) == len(dos_o)
    filled = dos_o > -1e300
    assert np.array_equal(filled, dos_g > -1e300)
    # both stop at sum((dlnZ/lnZ)^2) <= 1e-7: ln g agrees to the convergence tolerance
    shift = np.median(dos_g[filled] - dos_o[filled])
    assert np.allclose(dos_g[filled] - shift, dos_o[filled], rtol=0, atol=2e-3 * max(1.0, np.abs(dos_o[filled]).max()))
    assert abs(it_g - it_o) <= max(2, it_o // 10)


@pytest.mark.gpu
@pytest.mark.parametrize("graph,T0,T1", [("pmL20_c1.gset", 0.6, 2.8), ("rnd200_w1", 0.8, 10.0)])
def test_cae_ladder_gives_target_acceptance(graph, T0, T1):
    import pticm
    prob = pticm.Problem.load(os.path.join(G, graph))
    beta = pticm.cae_ladder(prob, seed=5, T0=T0, T1=T1, nt=16, samples=2000, burn_in=1000)
    assert len(beta) >= 3
    assert beta[0] == pytest.approx(1 / T0)
    assert np.all(np.diff(beta) < 0)
    # run PT on the ladder (ascending order for the engine) and measure acceptance
    asc = beta[::-1].copy()
    ctx = pticm.Context(prob, nt=len(asc), seed=9, icm=False)
    ctx.set_ladder(asc)
    ctx.init_states(9)
    ctx.run(3000)
    st, att, suc = ctx.stats()
    m = len(asc) - 1
    rate = (suc[:m] + suc[len(asc):len(asc) + m]) / np.maximum(att[:m] + att[len(asc):len(asc) + m], 1)
    # the walk targets 0.4; the last pair may overshoot toward beta_end
    assert np.all(rate[1:] > 0.2), rate
    assert abs(np.median(rate) - 0.4) < 0.15, rate
