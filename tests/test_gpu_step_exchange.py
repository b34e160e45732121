"""The per-step meeting of a group of blocks: each block publishes its
replicas' energies as words tagged with the step and waits for every other
replica's word of that step.  The tags come from a counter advanced by every
launch, so a word left by an earlier step or launch never passes for the
current one:
* twenty one-step launches continue the run exactly as one twenty-step
  launch does (replicas, energies, slot map, counters, best states);
* after a checkpoint at step 5 and ten more steps, loading the checkpoint
  into the same context (the step counter goes back, the published words
  keep their later tags) reproduces the same ten steps bit for bit;
in the one-replica-per-block layout, with four replicas per block, and in
the large-instance layout (spins only in shared memory).
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GRAPHS = os.path.join(os.path.dirname(__file__), "golden", "graphs")


def _state(ctx):
    s, E, f, slot = ctx.replicas()
    st, att, suc = ctx.stats()
    Eb, sweep, bs, rep = ctx.best()
    return dict(s=s, E=E, f=f, slot=slot, flips=st.flips, swaps=st.swaps, att=att, suc=suc, Eb=Eb, bs=bs)


def _same(a, b):
    for k in a:
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k


def _ctx(layout, seed):
    import pticm
    from pticm import instances
    if layout == "large":
        prob = pticm.Problem.from_instance(instances.c5())
        ctx = pticm.Context(prob, nt=6, chains=4, seed=seed, icm=True)
        ctx.set_ladder(pticm.beta_linspace(0.5, 9.5, 6))
    else:
        prob = pticm.Problem.load(os.path.join(GRAPHS, "rnd1000_pm"))
        rpb = 4 if layout == "four_per_block" else 1
        ctx = pticm.Context(prob, nt=16, seed=seed, icm=True, replicas_per_block=rpb)
        ctx.set_ladder(pticm.beta_linspace(0.5, 3.0, 16))
    ctx.init_states(seed + 1)
    return ctx


@pytest.mark.parametrize("layout", ["block_team", "four_per_block", "large"])
def test_one_step_launches_equal_one_launch(layout):
    a = _ctx(layout, 31)
    b = _ctx(layout, 31)
    assert a.layout().blocks > 1, "the step's meeting needs several blocks"
    a.run(20)
    for _ in range(20):
        b.run(1)
    _same(_state(a), _state(b))
    assert a.verify() == 0 and b.verify() == 0


@pytest.mark.parametrize("layout", ["block_team", "four_per_block", "large"])
def test_rewound_run_repeats_itself(layout, tmp_path):
    ctx = _ctx(layout, 41)
    ctx.run(5)
    path = str(tmp_path / "ck.bin")
    ctx.checkpoint_save(path)
    ctx.run(10)
    first = _state(ctx)
    ctx.checkpoint_load(path)
    ctx.run(10)
    _same(first, _state(ctx))
    assert ctx.verify() == 0
