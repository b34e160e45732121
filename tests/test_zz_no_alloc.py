"""The allocation-free entry point, pticm_run_noalloc, against pticm_run.

Callers whose host framework owns every device allocation (it hands out
buffers from its own pool) cannot use the context API, which allocates
device memory.  pticm_run_noalloc runs the same engine with its working
memory in a fixed array inside the library and reads and writes only
buffers the caller passes in.  Here those buffers come from torch, and two
chained calls must give exactly the states, energies and slot maps that two
pticm_run calls give on a context started from the same spins.  This file is
collected last so that a failure here comes after every other test ran.
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


@pytest.mark.parametrize("g,nt,T1", [("pmL20_c1.gset", 32, 3.0), ("rnd200_w1", 12, 15.0)])
def test_noalloc_matches_context_api_on_two_calls(g, nt, T1):
    torch = pytest.importorskip("torch")
    import pticm

    L = pticm.lib()
    f = L.pticm_run_noalloc
    f.argtypes = [C.c_void_p, C.POINTER(pticm.Opts), C.c_void_p, C.c_uint32, C.c_int32, C.POINTER(NoallocIO),
                  C.c_uint64, C.c_uint64, C.c_void_p]
    f.restype = C.c_int
    prob = pticm.Problem.load(os.path.join(G, g))
    n, R, seed, steps = prob.n, 2 * nt, 99, 40
    beta = pticm.beta_linspace(0.5, T1, nt)
    init = np.random.default_rng(3).integers(0, 2, size=(R, n), dtype=np.uint8)

    ctx = pticm.Context(prob, nt=nt, seed=seed, icm=True)
    ctx.set_ladder(beta)
    ctx.set_states(init)

    opts = pticm.Opts()
    L.pticm_opts_default(C.byref(opts))
    opts.seed, opts.nt, opts.chains, opts.sweeps, opts.icm = seed, nt, 2, 1, 1
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
