"""Checkpoint and resume of a PT run (pticm_checkpoint_save / _load).

A run interrupted after k steps, written to a checkpoint and resumed in a new
context continues bit for bit as the uninterrupted run: replicas, energies,
slot map, flip and swap counters, best states and, when enabled, the energy
histograms and magnetisation sums.  Loading into a context of another
problem, ladder size or seed is refused.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GRAPHS = os.path.join(os.path.dirname(__file__), "golden", "graphs")


@pytest.fixture(scope="module")
def pticm():
    import pticm as P
    P.lib()
    return P


def _state(ctx):
    s, E, f, slot = ctx.replicas()
    st, att, suc = ctx.stats()
    Eb, sweep, bs, rep = ctx.best()
    return dict(s=s, E=E, f=f, slot=slot, flips=st.flips, swaps=st.swaps, steps=st.pt_steps, att=att, suc=suc,
                Eb=Eb, sweep=sweep, bs=bs)


def _same(a, b):
    for k in a:
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k


@pytest.mark.parametrize("g,nt,exchange,hist", [("rnd200_w1", 12, 1, False), ("pmL20_c1.gset", 16, 0, False),
                                                ("lin40.ising", 8, 1, True)])
def test_resume_is_bit_exact(pticm, tmp_path, g, nt, exchange, hist):
    prob = pticm.Problem.load(os.path.join(GRAPHS, g))
    beta = pticm.beta_linspace(0.5, 3.0, nt)

    def fresh():
        ctx = pticm.Context(prob, nt=nt, seed=21, icm=True, exchange=exchange)
        ctx.set_ladder(beta)
        return ctx

    a = fresh()
    a.init_states(5)
    if hist:
        a.enable_energy_histograms(40)
    a.run(120)
    path = str(tmp_path / "run.ckpt")
    a.checkpoint_save(path)
    a.run(150)
    ref = _state(a)

    b = fresh()
    b.checkpoint_load(path)
    b.run(150)
    got = _state(b)
    _same(ref, got)
    assert b.verify() == 0
    if hist:
        ha, ea = a.energy_histograms()
        hb, eb = b.energy_histograms()
        assert np.array_equal(ha, hb) and np.array_equal(ea, eb)
        for xa, xb in zip(a.observables(), b.observables()):
            assert np.array_equal(xa, xb)


def test_checkpoint_refuses_other_contexts(pticm, tmp_path):
    prob = pticm.Problem.load(os.path.join(GRAPHS, "rnd200_w1"))
    ctx = pticm.Context(prob, nt=8, seed=3, icm=True)
    ctx.set_ladder(pticm.beta_linspace(0.5, 3.0, 8))
    ctx.init_states(1)
    ctx.run(10)
    path = str(tmp_path / "a.ckpt")
    ctx.checkpoint_save(path)
    other_nt = pticm.Context(prob, nt=10, seed=3, icm=True)
    with pytest.raises(pticm.PticmError):
        other_nt.checkpoint_load(path)
    other_seed = pticm.Context(prob, nt=8, seed=4, icm=True)
    with pytest.raises(pticm.PticmError):
        other_seed.checkpoint_load(path)
    other_problem = pticm.Context(pticm.Problem.load(os.path.join(GRAPHS, "pmL6.gset")), nt=8, seed=3, icm=True)
    with pytest.raises(pticm.PticmError):
        other_problem.checkpoint_load(path)
    junk = tmp_path / "junk.ckpt"
    junk.write_bytes(b"not a checkpoint at all")
    with pytest.raises(pticm.PticmError):
        ctx.checkpoint_load(str(junk))


def _array_offsets(path, nt):
    """Byte offsets of the arrays of a checkpoint file, in file order: the
    header (magic, version, 11 identity words, padding, steps, attempts, nc,
    the ladder, the histogram range), then u64 byte count + bytes each."""
    import struct
    data = open(path, "rb").read()
    off = 8 + 4 + 4 + 11 * 8 + 8 + 8 + 8 + 8 + nt * 8 + 8 + 8 + 8
    out = []
    while off < len(data):
        (nbytes,) = struct.unpack_from("<Q", data, off)
        out.append((off + 8, nbytes))
        off += 8 + nbytes
    return data, out


@pytest.mark.parametrize("which,index", [("slot map", 9), ("exchange order", 10)])
def test_checkpoint_with_a_broken_permutation_is_refused(pticm, tmp_path, which, index):
    """The engine indexes with the slot map and the exchange order: a file
    whose map is not a permutation is refused before anything is uploaded
    (spins, fields, energies, best states, flips, best sweeps, swap attempts,
    swap successes, then the slot map and the exchange order)."""
    import struct
    prob = pticm.Problem.load(os.path.join(GRAPHS, "rnd200_w1"))
    ctx = pticm.Context(prob, nt=8, seed=3, icm=True, exchange=0)
    ctx.set_ladder(pticm.beta_linspace(0.5, 3.0, 8))
    ctx.init_states(1)
    ctx.run(10)
    path = str(tmp_path / "a.ckpt")
    ctx.checkpoint_save(path)
    data, arrays = _array_offsets(path, 8)
    off, nbytes = arrays[index]
    assert nbytes >= 8
    bad = bytearray(data)
    first = struct.unpack_from("<I", bad, off)[0]
    struct.pack_into("<I", bad, off + 4, first)       # entry 1 repeats entry 0
    broken = tmp_path / "broken.ckpt"
    broken.write_bytes(bytes(bad))
    other = pticm.Context(prob, nt=8, seed=3, icm=True, exchange=0)
    other.set_ladder(pticm.beta_linspace(0.5, 3.0, 8))
    with pytest.raises(pticm.PticmError) as e:
        other.checkpoint_load(str(broken))
    assert e.value.code == 1 and which in str(e.value) and "permutation" in str(e.value)
    out_of_range = bytearray(data)
    struct.pack_into("<I", out_of_range, off, 1000)
    broken.write_bytes(bytes(out_of_range))
    with pytest.raises(pticm.PticmError):
        other.checkpoint_load(str(broken))
    # the intact file still loads
    other.checkpoint_load(path)
    other.run(5)
    assert other.verify() == 0
