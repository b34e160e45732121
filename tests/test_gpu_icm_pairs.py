"""Cluster identity of the production ICM kernels against the oracle's bfs_icm.

pticm_icm_pairs runs one ICM phase of the production engine -- the same
kernel variant and block layout pticm_run uses -- with the seed site of every
pair given by the caller.  The oracle restates xor_icm's global-flip rule and
bfs_icm (src/icm.cc:8-72) on the same states from the same seeds.  With
exact=1 the engine must flip exactly the oracle's cluster; in production mode
(exact=0) it flips the smaller of the cluster C and the rest of the overlap
D\\C, so the pair must hold the oracle's two states exchanged exactly when
2|C| > |D|.  Fields and energies must equal a from-scratch recompute.

Layouts: one replica per block (the block-team kernel, narrow 512-thread and
wide 1024-thread variants, as the C1/C2 workloads run), several replicas per
block with warp teams or a block-wide team, all replicas in one block, and
the large-instance modes: spins in shared memory with fields gathered (one,
two or four replicas per block) and the state in device memory (all in one
block).
"""
import os
import zlib

import numpy as np
import pytest

from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

G = os.path.join(os.path.dirname(__file__), "golden", "graphs")
NT = 6          # six pairs: identical, 5 %, 30 %, 50 %, 80 % (global flip) differing sites, skipped


def _graph(name, tmp_path_factory):
    from pticm import instances
    if name == "c2_random_2000":
        p = str(tmp_path_factory.mktemp("g") / "c2")          # 1-based, like Gset
        instances.c2().write_gset(p)
        return p
    if name == "random_20000_pm":
        p = str(tmp_path_factory.mktemp("g") / "r20k.gset")
        instances.c5().write_gset(p)
        return p
    return os.path.join(G, name)


def _pair_states(n, rng):
    """R = 2*NT states: replica k (chain 0) and NT + k (chain 1) form the pair
    at slot k, pair q = NT-1-k."""
    S = rng.integers(0, 2, size=(2 * NT, n), dtype=np.uint8)
    fracs = [0.0, 0.05, 0.3, 0.5, 0.8, 0.3]
    for q, f in enumerate(fracs):
        k = NT - 1 - q
        flip = rng.random(n) < f
        S[NT + k] = S[k] ^ flip.astype(np.uint8)
    return S


LAYOUTS = {
    "block_team": dict(),                                   # one replica per block (C1/C2 layout)
    "block_team_1024": dict(block_threads=1024),            # wide block-team variant
    "two_per_block": dict(replicas_per_block=2),            # partners in other blocks, warp/block teams
    "four_per_block": dict(replicas_per_block=4),           # (the large instance: fields gathered for 4)
    "one_block": dict(replicas_per_block=2 * NT),           # every replica in one block
}


@pytest.mark.parametrize("algo", [1, 2, 3])
@pytest.mark.parametrize("layout", list(LAYOUTS))
@pytest.mark.parametrize("graph", ["rnd200_w1", "pmL20_c1.gset", "lin40.ising", "pmL6.gset", "rnd60_pm",
                                   "c2_random_2000", "random_20000_pm"])
def test_icm_cluster_matches_oracle_bfs(graph, layout, algo, tmp_path_factory):
    import pticm

    path = _graph(graph, tmp_path_factory)
    prob = pticm.Problem.load(path)
    oprob = O.Problem.load(path, 0)
    n = prob.n
    rng = np.random.default_rng(zlib.crc32(f"{graph}/{layout}/{algo}".encode()))
    S = _pair_states(n, rng)
    # the oracle's result per pair and the seed drawn from its overlap
    seeds = np.full(NT, -2, np.int64)
    expect = {}
    for q in range(NT - 1):
        k = NT - 1 - q
        a, sites = O.overlap(oprob, S[k], S[NT + k])
        if len(sites) == 0:
            seeds[q] = -1
            expect[q] = (a, S[NT + k].copy(), 0, 0)
            continue
        seed = int(sites[rng.integers(len(sites))])
        seeds[q] = seed
        a2, b2 = O.bfs_icm(oprob, seed, a, S[NT + k])
        csize = int((a2 != a).sum())
        expect[q] = (a2, b2, csize, len(sites))
    beta = pticm.beta_linspace(0.5, 3.0, NT)
    for exact in (1, 0):
        try:
            ctx = pticm.Context(prob, nt=NT, seed=7, icm=True, icm_algo=algo, **LAYOUTS[layout])
            ctx.set_ladder(beta, nc=NT)
            ctx.set_states(S)
        except pticm.PticmError as e:
            if e.code == 3:   # this layout does not fit the instance
                pytest.skip(str(e))
            raise
        lay = ctx.layout()
        if graph == "random_20000_pm":
            # spins in shared memory with gathered fields while they fit;
            # all 12 replicas in one block keep their state in device memory
            want = 2 if lay.replicas_per_block > 4 else 1
            assert lay.state_mode == want, (lay.replicas_per_block, lay.state_mode)
        if layout.startswith("block_team") and graph != "random_20000_pm":
            assert lay.block_team == 1 and lay.replicas_per_block == 1
        ctx.icm_pairs(seeds, exact=bool(exact))
        out, E, _, _ = ctx.replicas()
        assert ctx.verify() == 0, "fields/energies differ from a from-scratch recompute"
        Eo, _ = prob.evaluate(out)
        assert np.array_equal(Eo.astype(np.int64), E)
        for q in range(NT):
            k = NT - 1 - q
            A, B = out[k], out[NT + k]
            if q == NT - 1:   # skipped pair: untouched
                assert np.array_equal(A, S[k]) and np.array_equal(B, S[NT + k])
                continue
            a2, b2, csize, cnt = expect[q]
            swapped = (not exact) and 2 * csize > cnt
            if swapped:
                assert np.array_equal(A, b2) and np.array_equal(B, a2), f"pair {q} (smaller-side flip)"
            else:
                assert np.array_equal(A, a2) and np.array_equal(B, b2), f"pair {q}"


def test_icm_pairs_rejects_a_seed_outside_the_overlap():
    import pticm

    prob = pticm.Problem.load(os.path.join(G, "rnd200_w1"))
    rng = np.random.default_rng(1)
    S = _pair_states(prob.n, rng)
    ctx = pticm.Context(prob, nt=NT, seed=7, icm=True)
    ctx.set_ladder(pticm.beta_linspace(0.5, 3.0, NT), nc=NT)
    ctx.set_states(S)
    k = NT - 2   # pair 1: about 5 % of the sites differ
    same = np.nonzero(S[k] == S[NT + k])[0]
    seeds = np.full(NT, -2, np.int64)
    seeds[1] = same[0]
    with pytest.raises(pticm.PticmError) as e:
        ctx.icm_pairs(seeds, exact=True)
    assert e.value.code == 1 and "differ" in str(e.value)
    # the context stays usable and unchanged
    seeds[1] = -2
    ctx.icm_pairs(seeds)
    out, _, _, _ = ctx.replicas()
    assert np.array_equal(out, S)
    assert ctx.verify() == 0
