"""The device exchange phase against a serial restatement with the same draws.

The production exchange walks the reference's attempt order
(src/replica_exchange.cc:5-100: one cursor over a shuffled pair order shared
by the chains, reshuffled on wrap) but evaluates independent attempts in
parallel.  This test replays the same Philox draws serially on the host and
requires identical slot maps and per-slot attempt/success counts.  The even/
odd mode is checked the same way.
"""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

G = os.path.join(os.path.dirname(__file__), "golden", "graphs")
M32 = 0xFFFFFFFF
TAG_EXCHANGE = 0x45584348


def philox(ctr, key):
    c = list(ctr)
    k = list(key)
    for _ in range(10):
        p0 = 0xD2511F53 * c[0]
        p1 = 0xCD9E8D57 * c[2]
        c = [((p1 >> 32) ^ c[1] ^ k[0]) & M32, p1 & M32, ((p0 >> 32) ^ c[3] ^ k[1]) & M32, p0 & M32]
        k = [(k[0] + 0x9E3779B9) & M32, (k[1] + 0xBB67AE85) & M32]
    return c


def stream_key(seed, tag):
    return [(seed & M32) ^ tag, ((seed >> 32) & M32) ^ ((tag * 0x9E3779B9) & M32)]


def u01_log(x):
    u = np.float32(((x >> 8) + 1) * (1.0 / 16777216.0))
    return float(np.log(u))


def initial_order(seed, nt):
    L = O.lib()
    g = (C.c_uint64 * 313)()
    L.orc_mt64_seed(g, (seed ^ 0x6F72646572) & 0xFFFFFFFFFFFFFFFF)
    a = np.arange(nt - 1, dtype=np.uint32)
    L.orc_shuffle_u32(a.ctypes.data_as(C.c_void_p), nt - 1, g)
    return a


def serial_reference_order(E, slot, order, beta, step, seed, nt, C_, att, suc, ambiguous):
    m = nt - 1
    total = C_ * m
    key = stream_key(seed, TAG_EXCHANGE)
    words = []
    for call in range((2 * total + 3) // 4):
        words += philox([call, 0, step & M32, step >> 32], key)
    logu = [u01_log(w) for w in words[:total]]
    xr = words[total:2 * total]
    for rnd in range(C_):
        for i in range(m):
            a = rnd * m + i
            c = a % C_
            kb = int(order[i])
            k = c * nt + kb
            r1, r2 = slot[k], slot[k + 1]
            x = (beta[kb] - beta[kb + 1]) * float(E[r1] - E[r2])
            att[k] += 1
            if 0 < abs(logu[a] - x) < 1e-5:
                ambiguous.append((step, a))
            if x > 0.0 or logu[a] < x:
                suc[k] += 1
                slot[k], slot[k + 1] = r2, r1
        keys = xr[rnd * m:(rnd + 1) * m]
        idx = sorted(range(m), key=lambda j: (keys[j], j))
        order = [order[j] for j in idx]
    return order


def serial_even_odd(E, slot, beta, step, seed, nt, C_, att, suc, ambiguous):
    m = nt - 1
    key = stream_key(seed, TAG_EXCHANGE)
    for par in (0, 1):
        for c in range(C_):
            for kb in range(par, m, 2):
                k = c * nt + kb
                w = philox([(k | (par << 30)) & M32, 0, step & M32, step >> 32], key)[0]
                lu = u01_log(w)
                r1, r2 = slot[k], slot[k + 1]
                x = (beta[kb] - beta[kb + 1]) * float(E[r1] - E[r2])
                att[k] += 1
                if 0 < abs(lu - x) < 1e-5:
                    ambiguous.append((step, k))
                if x > 0.0 or lu < x:
                    suc[k] += 1
                    slot[k], slot[k + 1] = r2, r1


@pytest.mark.parametrize("exchange", [0, 1])
@pytest.mark.parametrize("rpb", [0, 1])
@pytest.mark.parametrize("g,nt,chains", [("pmL20_c1.gset", 32, 2), ("rnd200_w1", 12, 2), ("pmL10.gset", 9, 4)])
def test_exchange_matches_serial(g, nt, chains, exchange, rpb):
    import pticm
    prob = pticm.Problem.load(os.path.join(G, g))
    seed = 12345
    ctx = pticm.Context(prob, nt=nt, chains=chains, seed=seed, icm=False, exchange=exchange,
                        replicas_per_block=rpb)
    beta = pticm.beta_linspace(0.4, 3.0, nt)
    ctx.set_ladder(beta)
    ctx.init_states(5)
    ctx.run(3, pticm.PHASE_SWEEP)          # spread the energies
    R = nt * chains
    _, E, _, _ = ctx.replicas()
    _, slot, _ = ctx.ladder()
    slot = [int(x) for x in slot]
    order = list(initial_order(seed, nt))
    att = np.zeros(R, np.int64)
    suc = np.zeros(R, np.int64)
    ambiguous = []
    for step in range(3, 9):
        ctx.run(1, pticm.PHASE_EXCHANGE)
        if exchange == 0:
            order = serial_reference_order(E, slot, order, beta, step, seed, nt, chains, att, suc, ambiguous)
        else:
            serial_even_odd(E, slot, beta, step, seed, nt, chains, att, suc, ambiguous)
    assert not ambiguous
    _, dslot, _ = ctx.ladder()
    _, datt, dsuc = ctx.stats()
    assert dslot.tolist() == slot
    assert datt.tolist() == att.tolist()
    assert dsuc.tolist() == suc.tolist()
    assert suc.sum() > 0
