"""The sweep colouring (host only, no GPU).

The engine updates every site of a colour class at once, so the classes must
form a proper colouring of the coupling graph: no edge inside a class.  Checked
on lattices (even tori are bipartite: two classes), random graphs of several
degrees, the C2 graph, dense inputs and a sample of the batched workload.
Every class is non-empty and there are at most (maximum degree + 1) classes,
the bound of any greedy colouring.
"""
import numpy as np
import pytest

from pticm import instances as I


def _check(prob, n, src, dst):
    col = prob.colouring()
    info = prob.info()
    assert col.shape == (n,)
    assert col.min() >= 0 and col.max() < info.ncolors
    assert len(np.unique(col)) == info.ncolors
    src = np.asarray(src, np.int64)
    dst = np.asarray(dst, np.int64)
    assert not np.any(col[src] == col[dst])
    deg = np.bincount(np.concatenate([src, dst]), minlength=n)
    assert info.ncolors <= int(deg.max()) + 1
    return info.ncolors


@pytest.mark.parametrize("L", [6, 7, 10, 20, 21])
def test_lattice_colouring(L):
    import pticm
    inst = I.pm_lattice(L, seed=L)
    k = _check(pticm.Problem.from_instance(inst), inst.n, inst.src, inst.dst)
    if L % 2 == 0:
        assert k == 2   # the checkerboard
    else:
        assert k >= 3   # odd cycles around the torus


@pytest.mark.parametrize("n,m,seed", [(200, 300, 1), (500, 2500, 2), (1000, 10000, 3), (3000, 60000, 4)])
def test_random_graph_colouring(n, m, seed):
    import pticm
    inst = I.random_graph(n, m, seed=seed, signed=True)
    _check(pticm.Problem.from_instance(inst), inst.n, inst.src, inst.dst)


def test_c2_graph_colouring():
    import pticm
    inst = I.c2()
    assert _check(pticm.Problem.from_instance(inst), inst.n, inst.src, inst.dst) <= 8


def test_dense_colouring():
    import pticm
    rng = np.random.default_rng(7)
    n = 60
    J = rng.choice(np.array([-1.0, 0.0, 1.0]), size=(n, n), p=[0.3, 0.4, 0.3])
    J = np.triu(J, 1)
    J = J + J.T
    prob = pticm.Problem.from_dense(J)
    src, dst = np.nonzero(np.triu(J, 1))
    _check(prob, n, src, dst)


def test_batched_workload_sample_colouring():
    import pticm
    for inst in I.batch_mix(24, seed0=1000):
        _check(pticm.Problem.from_instance(inst), inst.n, inst.src, inst.dst)
