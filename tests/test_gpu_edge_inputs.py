"""Edge-case instances on the GPU engine: isolated spins, a single spin,
missing weights, 0-based files, parallel edges (sparse) and overwritten
pairs (dense), blank lines, linear terms.  Device energies and cuts equal the
oracle's on random states; a short PT-ICM run stays exact (from-scratch
recompute) and finds the brute-force ground state of these tiny instances.
"""
import itertools

import numpy as np
import pytest

from oracle import pyoracle as O
from test_host_inputs import CASES

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pticm():
    import pticm as P
    P.lib()
    return P


@pytest.mark.parametrize("name", sorted(CASES))
def test_edge_instance_runs_exactly(pticm, tmp_path, name):
    path = tmp_path / name
    path.write_text(CASES[name])
    path = str(path)
    orc = O.Problem.load(path, 0)
    prob = pticm.Problem.load(path)
    n = orc.n
    rng = np.random.default_rng(3)
    states = rng.integers(0, 2, size=(16, n), dtype=np.uint8)
    E, cut = prob.evaluate(states)
    for k in range(len(states)):
        assert E[k] == orc.energy(states[k])
        assert cut[k] == orc.maxcut(states[k])
    nt = 4
    ctx = pticm.Context(prob, nt=nt, seed=5, icm=True)
    ctx.set_ladder(pticm.beta_linspace(0.5, 3.0, nt))
    ctx.init_states(9)
    ctx.run(200)
    assert ctx.verify() == 0
    if n <= 12:
        ground = min(orc.energy(np.array(s, np.uint8)) for s in itertools.product((0, 1), repeat=n))
        Eb, _, bs, _ = ctx.best()
        assert Eb == ground
        assert orc.energy(bs) == ground
