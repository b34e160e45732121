"""Observables of --log (T, C, X, u, m per temperature) against the exact
finite-size solution of the periodic L=20 Ising ferromagnet that the
reference ships (tests/golden/lattice20_exact.json, from its
data/lattice_2d_20_{u,c}.csv; the graph is its example_graphs/
lattice_2d_20.gset, the same edge set as pm_lattice(20, ferro=True))."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "lattice20_exact.json")


def test_lattice20_energy_and_specific_heat_match_exact_solution():
    import pticm
    from pticm import instances as I
    ex = json.load(open(GOLDEN))
    exact = {round(t, 2): (u, c) for t, u, c in zip(ex["T"], ex["u"], ex["c"])}
    temps = np.round(np.arange(1.5, 3.5001, 0.1), 2)
    beta = np.sort(1.0 / temps)
    prob = pticm.Problem.from_instance(I.pm_lattice(20, ferro=True))
    ctx = pticm.Context(prob, nt=len(beta), seed=4, icm=True)
    ctx.set_ladder(beta)
    ctx.init_states(5)
    ctx.enable_energy_histograms(10000)
    ctx.run(90000)
    T, C, X, u, m, n = ctx.observables()
    assert (n == 2 * 80000).all()
    for j in range(len(T)):
        ue, ce = exact[round(float(T[j]), 2)]
        assert abs(u[j] - ue) < 0.01, (T[j], u[j], ue)
        assert abs(C[j] - ce) < 0.15 * ce + 0.03, (T[j], C[j], ce)
    assert (X >= 0).all() and (np.abs(m) <= 1).all()
