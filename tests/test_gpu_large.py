"""The large single instance (N=20000, 400000 +-1 edges, 128 temperatures x 4
replicas per temperature, ICM on): the replicas exceed shared memory and the
engine keeps them, with the adjacency and ICM scratch, in device memory.
Checked at full size by the properties that do not depend on size: fields
and energies equal a from-scratch recomputation after every phase, the best
energy is the energy of the best state, exchange and ICM run."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c5():
    import pticm
    from pticm import instances as I
    inst = I.c5()
    return inst, pticm.Problem.from_instance(inst)


def test_large_instance_is_exact_after_every_phase(c5):
    import pticm
    inst, prob = c5
    beta = pticm.beta_linspace(0.5, 9.5, 128)
    ctx = pticm.Context(prob, nt=128, chains=4, seed=3, icm=True)
    ctx.set_ladder(beta)
    ctx.init_states(4)
    for mask in (1, 2, 4, 7):
        ctx.run(6, mask)
        assert ctx.verify() == 0, mask
    ctx.run(40)
    assert ctx.verify() == 0
    st, att, suc = ctx.stats()
    assert st.replicas == 512 and st.attempts == (6 + 6 + 40) * 512 * inst.n
    assert att.sum() > 0 and suc.sum() > 0
    E, sweep, state, rep = ctx.best()
    assert prob.evaluate(state[None, :])[0][0] == E
