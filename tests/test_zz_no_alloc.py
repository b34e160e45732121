"""The allocation-free entry point, pticm_run_noalloc, against pticm_run.

Callers whose host framework owns every device allocation (it hands out
buffers from its own pool) cannot use the context API, which allocates
device memory.  pticm_run_noalloc runs the same engine with its working
memory in a fixed array inside the library and reads and writes only
buffers the caller passes in.  Here those buffers come from torch, and two
chained calls must give exactly the states, energies and slot maps that two
pticm_run calls give on a context started from the same spins -- and, with the
reference-order exchange, the same pair order, swap counts and best states.
A slot map or pair order that is not a permutation is refused before the
engine runs.  This file is collected last so that a failure here comes after
every other test ran.
"""
import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

G = os.path.join(os.path.dirname(__file__), "golden", "graphs")


class NoallocIO(C.Structure):
    _fields_ = [("spins_in", C.c_void_p), ("spins_out", C.c_void_p), ("energy_out", C.c_void_p),
                ("slot_to_replica", C.c_void_p), ("pair_order", C.c_void_p), ("swap_attempts", C.c_void_p),
                ("swap_successes", C.c_void_p), ("best_energy_out", C.c_void_p),
                ("best_states_out", C.c_void_p)]


def _noalloc(pticm):
    L = pticm.lib()
    f = L.pticm_run_noalloc
    f.argtypes = [C.c_void_p, C.POINTER(pticm.Opts), C.c_void_p, C.c_uint32, C.c_int32, C.POINTER(NoallocIO),
                  C.c_uint64, C.c_uint64, C.c_void_p]
    f.restype = C.c_int
    return L, f


def _opts(pticm, L, seed, nt, exchange):
    opts = pticm.Opts()
    L.pticm_opts_default(C.byref(opts))
    opts.seed, opts.nt, opts.chains, opts.sweeps, opts.icm, opts.exchange = seed, nt, 2, 1, 1, exchange
    return opts


@pytest.mark.parametrize("g,nt,T1", [("pmL20_c1.gset", 32, 3.0), ("rnd200_w1", 12, 15.0)])
def test_noalloc_matches_context_api_on_two_calls(g, nt, T1):
    torch = pytest.importorskip("torch")
    import pticm

    L, f = _noalloc(pticm)
    prob = pticm.Problem.load(os.path.join(G, g))
    n, R, seed, steps = prob.n, 2 * nt, 99, 40
    beta = pticm.beta_linspace(0.5, T1, nt)
    init = np.random.default_rng(3).integers(0, 2, size=(R, n), dtype=np.uint8)

    ctx = pticm.Context(prob, nt=nt, seed=seed, icm=True)
    ctx.set_ladder(beta)
    ctx.set_states(init)

    opts = _opts(pticm, L, seed, nt, 1)
    dev = torch.device("cuda:0")
    s_in = torch.from_numpy(init.reshape(-1).copy()).to(dev)
    s_out = torch.empty_like(s_in)
    energy = torch.empty(R, dtype=torch.int64, device=dev)
    slot = torch.arange(R, dtype=torch.int32, device=dev)
    io = NoallocIO(s_in.data_ptr(), s_out.data_ptr(), energy.data_ptr(), slot.data_ptr(), None, None, None,
                   None, None)
    for call in range(2):
        ctx.run(steps)
        rc = f(prob._h, C.byref(opts), beta.ctypes.data_as(C.c_void_p), nt, -1, C.byref(io), call * steps,
               steps, None)
        assert rc == 0, L.pticm_last_error().decode()
        torch.cuda.synchronize()
        states, E, _, _ = ctx.replicas()
        _, s2r, _ = ctx.ladder()
        assert np.array_equal(s_out.cpu().numpy().reshape(R, n), states)
        assert np.array_equal(energy.cpu().numpy(), E)
        assert np.array_equal(slot.cpu().numpy().astype(np.uint32), s2r)
        s_in.copy_(s_out)


@pytest.mark.parametrize("g,nt,T1", [("rnd200_w1", 12, 15.0), ("pmL20_c1.gset", 16, 3.0)])
def test_noalloc_reference_order_counts_and_best_states(g, nt, T1):
    """The reference-order exchange (exchange = 0): the pair order passed in
    and out, this call's swap counts and each replica's best energy and state
    of this call, against a context run over the same two intervals."""
    torch = pytest.importorskip("torch")
    import pticm

    L, f = _noalloc(pticm)
    prob = pticm.Problem.load(os.path.join(G, g))
    n, R, seed, steps = prob.n, 2 * nt, 17, 30
    beta = pticm.beta_linspace(0.5, T1, nt)
    init = np.random.default_rng(5).integers(0, 2, size=(R, n), dtype=np.uint8)
    ctx = pticm.Context(prob, nt=nt, seed=seed, icm=True, exchange=0)
    ctx.set_ladder(beta)
    ctx.set_states(init)
    order0 = ctx.exchange_order()

    opts = _opts(pticm, L, seed, nt, 0)
    dev = torch.device("cuda:0")
    s_in = torch.from_numpy(init.reshape(-1).copy()).to(dev)
    s_out = torch.empty_like(s_in)
    energy = torch.empty(R, dtype=torch.int64, device=dev)
    slot = torch.arange(R, dtype=torch.int32, device=dev)
    order = torch.from_numpy(order0.astype(np.int32)).to(dev)
    att = torch.empty(R, dtype=torch.int64, device=dev)
    suc = torch.empty(R, dtype=torch.int64, device=dev)
    best_e = torch.empty(R, dtype=torch.int64, device=dev)
    best_s = torch.empty(R * n, dtype=torch.uint8, device=dev)
    io = NoallocIO(s_in.data_ptr(), s_out.data_ptr(), energy.data_ptr(), slot.data_ptr(), order.data_ptr(),
                   att.data_ptr(), suc.data_ptr(), best_e.data_ptr(), best_s.data_ptr())
    cum_att = np.zeros(R, np.int64)
    cum_suc = np.zeros(R, np.int64)
    cum_best = np.full(R, np.iinfo(np.int64).max)
    cum_state = np.zeros((R, n), np.uint8)
    for call in range(2):
        ctx.run(steps)
        rc = f(prob._h, C.byref(opts), beta.ctypes.data_as(C.c_void_p), nt, -1, C.byref(io), call * steps,
               steps, None)
        assert rc == 0, L.pticm_last_error().decode()
        torch.cuda.synchronize()
        states, E, _, _ = ctx.replicas()
        _, s2r, _ = ctx.ladder()
        assert np.array_equal(s_out.cpu().numpy().reshape(R, n), states)
        assert np.array_equal(energy.cpu().numpy(), E)
        assert np.array_equal(slot.cpu().numpy().astype(np.uint32), s2r)
        assert np.array_equal(order.cpu().numpy().astype(np.uint32), ctx.exchange_order())
        cum_att += att.cpu().numpy()
        cum_suc += suc.cpu().numpy()
        _, catt, csuc = ctx.stats()
        assert np.array_equal(cum_att, catt.astype(np.int64))
        assert np.array_equal(cum_suc, csuc.astype(np.int64))
        # the context keeps each replica's best over both calls (a later
        # state only when strictly lower) and reports the first replica of
        # the lowest best
        be = best_e.cpu().numpy()
        bs = best_s.cpu().numpy().reshape(R, n)
        better = be < cum_best
        cum_best = np.where(better, be, cum_best)
        cum_state[better] = bs[better]
        E_ctx, _, state_ctx, rep_ctx = ctx.best()
        r = int(np.argmin(cum_best))
        assert E_ctx == cum_best[r] and rep_ctx == r
        assert np.array_equal(state_ctx, cum_state[r])
        s_in.copy_(s_out)


def test_noalloc_refuses_a_slot_map_that_is_not_a_permutation():
    torch = pytest.importorskip("torch")
    import pticm

    L, f = _noalloc(pticm)
    prob = pticm.Problem.load(os.path.join(G, "rnd200_w1"))
    nt, n = 8, prob.n
    R = 2 * nt
    beta = pticm.beta_linspace(0.5, 15.0, nt)
    opts = _opts(pticm, L, 3, nt, 0)
    dev = torch.device("cuda:0")
    s_in = torch.zeros(R * n, dtype=torch.uint8, device=dev)
    s_out = torch.empty_like(s_in)
    energy = torch.empty(R, dtype=torch.int64, device=dev)
    slot = torch.arange(R, dtype=torch.int32, device=dev)
    slot[1] = 0                                      # replica 0 twice, replica 1 never
    io = NoallocIO(s_in.data_ptr(), s_out.data_ptr(), energy.data_ptr(), slot.data_ptr(), None, None, None,
                   None, None)
    rc = f(prob._h, C.byref(opts), beta.ctypes.data_as(C.c_void_p), nt, -1, C.byref(io), 0, 5, None)
    assert rc == 1 and b"slot_to_replica" in L.pticm_last_error()
    slot[1] = 1
    order = torch.tensor([0, 1, 2, 3, 4, 5, 7], dtype=torch.int32, device=dev)   # 7 is out of range
    io.pair_order = order.data_ptr()
    rc = f(prob._h, C.byref(opts), beta.ctypes.data_as(C.c_void_p), nt, -1, C.byref(io), 0, 5, None)
    assert rc == 1 and b"pair_order" in L.pticm_last_error()
    bad_beta = beta.copy()
    bad_beta[3] = np.nan
    rc = f(prob._h, C.byref(opts), bad_beta.ctypes.data_as(C.c_void_p), nt, -1, C.byref(io), 0, 5, None)
    assert rc == 1
    order[6] = 6
    rc = f(prob._h, C.byref(opts), beta.ctypes.data_as(C.c_void_p), nt, -1, C.byref(io), 0, 5, None)
    assert rc == 0, L.pticm_last_error().decode()
