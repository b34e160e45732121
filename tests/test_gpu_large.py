"""The large single instance (N=20000, 400000 +-1 edges, 128 temperatures x 4
replicas per temperature, ICM on): spins and fields of a replica together
exceed what a block may hold, so the engine keeps only spins in shared memory
and gathers each local field at its visit.  Automatic layout: four replicas
per block (128 blocks, the cluster search's scratch beside them in shared
memory, overlap lists in device memory); one replica per block (512 blocks,
the cluster search's scratch in device memory) on request.  Checked at full
size by the properties that do not depend on size: fields and energies equal
a from-scratch recomputation after every phase, the best energy is the energy
of the best state, exchange and ICM run."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c5():
    import pticm
    from pticm import instances as I
    inst = I.c5()
    return inst, pticm.Problem.from_instance(inst)


@pytest.mark.parametrize("rpb,want_blocks", [(0, 128), (1, 512)])
def test_large_instance_is_exact_after_every_phase(c5, rpb, want_blocks):
    import pticm
    inst, prob = c5
    beta = pticm.beta_linspace(0.5, 9.5, 128)
    ctx = pticm.Context(prob, nt=128, chains=4, seed=3, icm=True, replicas_per_block=rpb)
    ctx.set_ladder(beta)
    ctx.init_states(4)
    for mask in (1, 2, 4, 7):
        ctx.run(6, mask)
        assert ctx.verify() == 0, mask
    ctx.run(40)
    assert ctx.verify() == 0
    lay = ctx.layout()
    assert lay.state_mode == 1 and lay.blocks == want_blocks, (lay.state_mode, lay.blocks)
    st, att, suc = ctx.stats()
    assert st.replicas == 512 and st.attempts == (6 + 6 + 40) * 512 * inst.n
    assert att.sum() > 0 and suc.sum() > 0
    E, sweep, state, rep = ctx.best()
    assert prob.evaluate(state[None, :])[0][0] == E
