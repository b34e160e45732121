"""Bounded waits: a group barrier whose wait runs out ends the kernel with an
error status instead of hanging, and the context stays usable.

The reference has no failure detection (an MPI rank that stops leaves the
others blocked in MPI_Recv; src/initialization.cc:120-126 and
src/mpi_utils.cc:223-225 assert or exit).  Here every wait of a kernel on
other blocks is bounded.  pticm_set_wait_limit shortens the limit and, as a
test hook, makes each group barrier wait for one block more than the group
has -- a block that never arrives -- so every wait runs out.  Nothing faults:
the waiting blocks record the failure, raise the abort flag and return.
"""
import os
import time

import pytest

pytestmark = pytest.mark.gpu

G = os.path.join(os.path.dirname(__file__), "golden", "graphs")


def _ctx(**kw):
    import pticm
    prob = pticm.Problem.load(os.path.join(G, "rnd200_w1"))
    ctx = pticm.Context(prob, nt=8, seed=3, icm=True, **kw)
    ctx.set_ladder(pticm.beta_linspace(0.5, 15.0, 8))
    ctx.init_states(3)
    return ctx


@pytest.mark.parametrize("layout", [dict(), dict(replicas_per_block=4)])
def test_barrier_wait_runs_out_with_an_error_status(layout):
    import pticm
    ctx = _ctx(**layout)
    assert ctx.layout().blocks > 1, "the group barrier needs several blocks"
    ctx.run(20)
    ctx.set_wait_limit(limit_ns=2_000_000, phantom_arrivals=1)
    t0 = time.time()
    with pytest.raises(pticm.PticmError) as e:
        ctx.run(10)
    assert e.value.code == 5, str(e.value)
    assert "group barrier wait expired at site 1" in str(e.value)
    assert time.time() - t0 < 10.0
    # the run stopped between phases: every replica's fields and energy are
    # still exact, and the context runs on once the hook is cleared
    assert ctx.verify() == 0
    ctx.set_wait_limit(0, 0)
    ctx.run(20)
    assert ctx.verify() == 0
    # a fresh context is clean
    fresh = _ctx(**layout)
    fresh.run(20)
    assert fresh.verify() == 0


def test_wait_limit_arguments_are_checked():
    import pticm
    ctx = _ctx()
    with pytest.raises(pticm.PticmError):
        ctx.set_wait_limit(limit_ns=10 ** 12)
    with pytest.raises(pticm.PticmError):
        ctx.set_wait_limit(phantom_arrivals=2)
    ctx.set_wait_limit(limit_ns=500_000_000)   # a shorter limit alone changes nothing
    ctx.run(50)
    assert ctx.verify() == 0
    st, _, _ = ctx.stats()
    assert st.pt_steps == 50
