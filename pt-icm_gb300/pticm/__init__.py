"""Python binding of the GB300 PT-ICM engine (include/pticm.h) over ctypes.

The names mirror the reference's libreplica interface: `Problem` is
pticm::Problem (src/problem.cc), `Context` is the PTWorker state that
`solve` drives (src/solver.cc), and `solve()` runs the whole PT-ICM loop
and returns the keys the reference prints (src/solver.cc:151-163).

There is no CPU path: every call goes to libpticm_gb300.so, which needs a
CUDA device; loading fails loudly when the library has not been built.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libpticm_gb300.so")

PHASE_SWEEP, PHASE_EXCHANGE, PHASE_ICM = 1, 2, 4
PHASE_ALL = 7


class PticmError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"pticm error {code}: {msg}")
        self.code = code


class ProblemInfo(C.Structure):
    _fields_ = [("n", C.c_int64), ("m", C.c_int64), ("nnz", C.c_int64), ("sparse", C.c_int32),
                ("ncolors", C.c_int32), ("kmax", C.c_int32), ("has_linear", C.c_int32),
                ("char_scale", C.c_double), ("total_weight", C.c_double)]


class Opts(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("nt", C.c_uint32), ("chains", C.c_uint32), ("sweeps", C.c_uint32),
                ("icm", C.c_uint32), ("exchange", C.c_uint32), ("best_per_phase", C.c_uint32),
                ("block_threads", C.c_uint32), ("replicas_per_block", C.c_uint32), ("icm_algo", C.c_uint32)]


class BatchInfo(C.Structure):
    _fields_ = [("count", C.c_uint32), ("lanes", C.c_uint32), ("chunk", C.c_uint32), ("jobs", C.c_uint32),
                ("smem_bytes", C.c_uint32), ("threads", C.c_uint32), ("tuned", C.c_uint32),
                ("makespan_us", C.c_double), ("pt_steps", C.c_uint64), ("attempts", C.c_uint64),
                ("last_run_ms", C.c_double), ("launches", C.c_uint64)]


class Stats(C.Structure):
    _fields_ = [("pt_steps", C.c_uint64), ("attempts", C.c_uint64), ("flips", C.c_uint64),
                ("swaps", C.c_uint64), ("nt", C.c_uint32), ("chains", C.c_uint32), ("nc", C.c_uint32),
                ("replicas", C.c_uint32), ("last_run_ms", C.c_double)]


class Layout(C.Structure):
    _fields_ = [("replicas_per_block", C.c_uint32), ("blocks", C.c_uint32), ("threads", C.c_uint32),
                ("icm_teams", C.c_uint32), ("block_team", C.c_int32), ("narrow", C.c_int32),
                ("adjacency_staged", C.c_int32), ("state_mode", C.c_int32)]


class Trace(C.Structure):
    _fields_ = [("pt_steps", C.c_uint64), ("uniforms", C.c_void_p), ("n_uniforms", C.c_uint64),
                ("sweep_offsets", C.c_void_p), ("xchg_slot", C.c_void_p), ("xchg_logu", C.c_void_p),
                ("icm_seed", C.c_void_p)]


_lib = None


def lib():
    """Load libpticm_gb300.so (build it with __graft_entry__.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build the native library first "
                           "(python -c 'import __graft_entry__ as g; g.build()')")
    L = C.CDLL(LIB_PATH)
    P = C.c_void_p
    i64, u64, u32, i32, dbl = C.c_int64, C.c_uint64, C.c_uint32, C.c_int32, C.c_double
    sigs = {
        "pticm_problem_load_gset": [C.c_char_p, C.POINTER(P)],
        "pticm_problem_from_coo": [i64, i64, P, P, P, P, C.POINTER(P)],
        "pticm_problem_from_dense": [i64, P, P, C.POINTER(P)],
        "pticm_problem_get_info": [P, C.POINTER(ProblemInfo)],
        "pticm_problem_get_colouring": [P, P],
        "pticm_problem_evaluate": [P, i64, P, P, P, P],
        "pticm_create": [P, C.POINTER(Opts), C.POINTER(P)],
        "pticm_set_ladder": [P, P, u32, i32],
        "pticm_beta_linspace": [P, dbl, dbl, u64, C.c_int],
        "pticm_init_states": [P, u64],
        "pticm_set_states": [P, P],
        "pticm_run": [P, u64, u32],
        "pticm_get_stats": [P, C.POINTER(Stats), P, P],
        "pticm_get_best": [P, P, P, P, P],
        "pticm_get_replicas": [P, P, P, P, P],
        "pticm_get_ladder": [P, P, P, P],
        "pticm_verify": [P, P],
        "pticm_checkpoint_save": [P, C.c_char_p],
        "pticm_checkpoint_load": [P, C.c_char_p],
        "pticm_replay": [P, C.POINTER(Trace)],
        "pticm_icm_pairs": [P, P, u32, C.c_int],
        "pticm_get_exchange_order": [P, P],
        "pticm_get_layout": [P, C.POINTER(Layout)],
        "pticm_smem_copy_rate": [C.c_int, P],
        "pticm_set_wait_limit": [P, u64, u32],
        "pticm_philox_probe": [P, P, P, C.c_int],
        "pticm_set_profiling": [P, C.c_int],
        "pticm_cae_ladder": [P, u64, dbl, dbl, C.c_int, u32, dbl, dbl, dbl, u64, u64, P, P],
        "pticm_enable_energy_histograms": [P, u64],
        "pticm_get_energy_histograms": [P, P, P, P],
        "pticm_mhist_dos": [P, P, P, u32, P, P, dbl, u64, dbl, P, u64, P, P, P],
        "pticm_cae_walk": [P, u64, dbl, dbl, dbl, dbl, dbl, dbl, u32, P, P],
        "pticm_get_profile": [P, P, P],
        "pticm_get_observables": [P, P, P, P, P, P, P],
        "pticm_tc_gemm_check": [C.c_int, C.c_int, C.c_int, P, P, P, C.c_int, P, P],
        "pticm_batch_create": [P, u32, C.POINTER(Opts), C.POINTER(P)],
        "pticm_batch_set_ladders": [P, P, u32, i32],
        "pticm_batch_init_states": [P, u64],
        "pticm_batch_autotune": [P, u32],
        "pticm_batch_run": [P, u64, u32],
        "pticm_batch_get_info": [P, C.POINTER(BatchInfo)],
        "pticm_batch_get_groups": [P, P, P, P, P],
        "pticm_batch_get_best": [P, P, P],
        "pticm_batch_get_best_state": [P, u32, P],
        "pticm_batch_get_swap_stats": [P, u32, P, P],
        "pticm_batch_get_energies": [P, u32, P, P],
        "pticm_batch_verify": [P, P],
        "pticm_batch_enable_energy_histograms": [P, u64],
        "pticm_batch_get_energy_histograms": [P, u32, P, P, P],
        "pticm_batch_logdos": [P, u32, dbl, P, u64, P, P, P],
        "pticm_batch_compute_logdos": [P, dbl],
        "pticm_mlp_create": [u64, u32, C.POINTER(P)],
        "pticm_mlp_get_params": [P, P],
        "pticm_mlp_set_params": [P, P],
        "pticm_mlp_set_data": [P, P, P, u64],
        "pticm_mlp_gradients": [P, P, P, u32, P, P],
        "pticm_mlp_train": [P, P, P, u64, u32, C.c_float, u64, P],
        "pticm_mlp_predict": [P, P, u64, P],
        "pticm_mlp_save": [P, C.c_char_p],
        "pticm_mlp_load": [P, C.c_char_p],
        "pticm_problem_features": [P, P],
        "pticm_surrogate_logdos": [P, P, P, u64, P, P, P],
        "pticm_surrogate_ladder": [P, P, dbl, dbl, C.c_int, u32, dbl, dbl, P, P],
        "pticm_ladder_acceptance": [P, P, u32, u64, u64, u64, P],
        "pticm_feedback_ladder": [P, u32, P, dbl, dbl, u32, dbl, P, P],
        "pticm_learned_ladder": [P, P, dbl, dbl, C.c_int, u32, dbl, u64, dbl, u64, P, P, P],
    }
    for name, args in sigs.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_int
    L.pticm_problem_free.argtypes = [P]
    L.pticm_problem_free.restype = None
    L.pticm_destroy.argtypes = [P]
    L.pticm_destroy.restype = None
    L.pticm_opts_default.argtypes = [C.POINTER(Opts)]
    L.pticm_opts_default.restype = None
    L.pticm_batch_destroy.argtypes = [P]
    L.pticm_batch_destroy.restype = None
    L.pticm_mlp_destroy.argtypes = [P]
    L.pticm_mlp_destroy.restype = None
    L.pticm_mlp_param_count.argtypes = []
    L.pticm_mlp_param_count.restype = u64
    L.pticm_last_error.restype = C.c_char_p
    L.pticm_version.restype = C.c_char_p
    _lib = L
    return L


def _check(rc):
    if rc != 0:
        raise PticmError(rc, lib().pticm_last_error().decode())


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Problem:
    """pticm::Problem: Ising couplings J_ij and linear terms h_i."""

    def __init__(self, handle):
        self._h = handle

    @classmethod
    def load(cls, path: str) -> "Problem":
        h = C.c_void_p()
        _check(lib().pticm_problem_load_gset(os.fspath(path).encode(), C.byref(h)))
        return cls(h)

    @classmethod
    def from_coo(cls, n, src, dst, w, h=None) -> "Problem":
        src = np.ascontiguousarray(src, np.int32)
        dst = np.ascontiguousarray(dst, np.int32)
        w = np.ascontiguousarray(w, np.float64)
        hh = None if h is None else np.ascontiguousarray(h, np.float64)
        out = C.c_void_p()
        _check(lib().pticm_problem_from_coo(n, len(src), _p(src), _p(dst), _p(w), _p(hh), C.byref(out)))
        return cls(out)

    @classmethod
    def from_instance(cls, inst) -> "Problem":
        return cls.from_coo(inst.n, inst.src, inst.dst, inst.w, inst.h)

    @classmethod
    def from_dense(cls, J, h=None) -> "Problem":
        J = np.ascontiguousarray(J, np.float64)
        hh = None if h is None else np.ascontiguousarray(h, np.float64)
        out = C.c_void_p()
        _check(lib().pticm_problem_from_dense(J.shape[0], _p(J), _p(hh), C.byref(out)))
        return cls(out)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.pticm_problem_free(self._h)
            self._h = None

    def info(self) -> ProblemInfo:
        inf = ProblemInfo()
        _check(lib().pticm_problem_get_info(self._h, C.byref(inf)))
        return inf

    @property
    def n(self) -> int:
        return self.info().n

    def colouring(self):
        """The sweep's colour class of every site (host only)."""
        out = np.zeros(self.n, np.int32)
        _check(lib().pticm_problem_get_colouring(self._h, _p(out)))
        return out

    def evaluate(self, states, with_dE=False):
        """Energy, max-cut and (optionally) dE of each state (rows of 0/1)."""
        s = np.ascontiguousarray(np.atleast_2d(states), np.uint8)
        cnt, n = s.shape
        E = np.zeros(cnt)
        cut = np.zeros(cnt)
        dE = np.zeros((cnt, n)) if with_dE else None
        _check(lib().pticm_problem_evaluate(self._h, cnt, _p(s), _p(E), _p(cut), _p(dE)))
        return (E, cut, dE) if with_dE else (E, cut)


def cae_ladder(problem: Problem, *, seed, T0, T1, nt, inverse=False, estep=2.0, step_size=0.1, r=0.4,
               samples=2000, burn_in=5000):
    """get_beta (src/cae_estimator.cc:295-428) on the GPU: the multihistogram
    constant-acceptance ladder, descending in beta."""
    out = np.zeros(nt)
    cnt = C.c_uint32()
    _check(lib().pticm_cae_ladder(problem._h, seed, T0, T1, int(inverse), nt, estep, step_size, r, samples,
                                  burn_in, _p(out), C.byref(cnt)))
    return out[:cnt.value]


def mhist_dos(hist, hist_off, hist_len, beta_hist, emin, estep, n, max_emax):
    """The FP64 multihistogram fixed point on the GPU: (ln g, ln Z, iterations)."""
    hist = np.ascontiguousarray(hist, np.uint32)
    off = np.ascontiguousarray(hist_off, np.uint64)
    ln = np.ascontiguousarray(hist_len, np.uint64)
    b = np.ascontiguousarray(beta_hist, np.float64)
    e = np.ascontiguousarray(emin, np.float64)
    nt = len(b)
    cap = int(np.ceil((max_emax - e.min()) / estep)) + 1
    dos = np.zeros(max(cap, 1))
    z = np.zeros(nt)
    nb = C.c_uint64()
    it = C.c_uint64()
    _check(lib().pticm_mhist_dos(_p(hist), _p(off), _p(ln), nt, _p(b), _p(e), estep, n, max_emax, _p(dos), cap,
                                 _p(z), C.byref(nb), C.byref(it)))
    return dos[:nb.value], z, it.value


def cae_walk(logdos, min_emin, estep, beta_start, beta_end, step_size, r, num_temps):
    """The constant-acceptance walk (host code)."""
    d = np.ascontiguousarray(logdos, np.float64)
    out = np.zeros(num_temps)
    cnt = C.c_uint32()
    _check(lib().pticm_cae_walk(_p(d), len(d), min_emin, estep, beta_start, beta_end, step_size, r, num_temps,
                                _p(out), C.byref(cnt)))
    return out[:cnt.value]


def smem_copy_rate(iters=2000) -> float:
    """Measured shared-memory copy rate of the GPU (read + written GB/s)."""
    r = C.c_double()
    _check(lib().pticm_smem_copy_rate(iters, C.byref(r)))
    return r.value


def beta_linspace(T0, T1, nt, inverse=False):
    b = np.zeros(nt)
    _check(lib().pticm_beta_linspace(_p(b), T0, T1, nt, int(inverse)))
    return b


class Context:
    """All replicas of one PT run resident on the current GPU."""

    def __init__(self, problem: Problem, *, nt, chains=2, seed=0, sweeps=1, icm=True, exchange=1,
                 best_per_phase=False, block_threads=0, replicas_per_block=0, icm_algo=0):
        L = lib()
        o = Opts()
        L.pticm_opts_default(C.byref(o))
        o.seed, o.nt, o.chains, o.sweeps, o.icm = seed, nt, chains, sweeps, int(icm)
        o.exchange, o.best_per_phase = exchange, int(best_per_phase)
        o.block_threads, o.replicas_per_block, o.icm_algo = block_threads, replicas_per_block, icm_algo
        h = C.c_void_p()
        _check(L.pticm_create(problem._h, C.byref(o), C.byref(h)))
        self._h = h
        self.problem = problem
        self.nt, self.chains, self.R = nt, chains, nt * chains
        self.n = problem.n

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.pticm_destroy(self._h)
            self._h = None

    def set_ladder(self, beta, nc=-1):
        b = np.ascontiguousarray(beta, np.float64)
        _check(lib().pticm_set_ladder(self._h, _p(b), len(b), nc))

    def init_states(self, seed):
        _check(lib().pticm_init_states(self._h, seed))

    def set_states(self, states):
        s = np.ascontiguousarray(states, np.uint8).reshape(self.R, self.n)
        _check(lib().pticm_set_states(self._h, _p(s)))

    def run(self, steps, phases=PHASE_ALL):
        _check(lib().pticm_run(self._h, steps, phases))

    def stats(self):
        st = Stats()
        at = np.zeros(self.R, np.uint64)
        su = np.zeros(self.R, np.uint64)
        _check(lib().pticm_get_stats(self._h, C.byref(st), _p(at), _p(su)))
        return st, at, su

    def best(self):
        E = C.c_double()
        sw = C.c_uint64()
        rep = C.c_int64()
        s = np.zeros(self.n, np.uint8)
        _check(lib().pticm_get_best(self._h, C.byref(E), C.byref(sw), _p(s), C.byref(rep)))
        return E.value, sw.value, s, rep.value

    def replicas(self):
        s = np.zeros((self.R, self.n), np.uint8)
        E = np.zeros(self.R, np.int64)
        f = np.zeros((self.R, self.n), np.int32)
        slot = np.zeros(self.R, np.uint32)
        _check(lib().pticm_get_replicas(self._h, _p(s), _p(E), _p(f), _p(slot)))
        return s, E, f, slot

    def ladder(self):
        b = np.zeros(self.nt)
        s2r = np.zeros(self.R, np.uint32)
        nc = C.c_uint32()
        _check(lib().pticm_get_ladder(self._h, _p(b), _p(s2r), C.byref(nc)))
        return b, s2r, nc.value

    def icm_pairs(self, seeds, exact=False):
        """One ICM phase with caller seeds: seeds[q] per pair q (original site,
        -1 for the engine's draw, -2 to skip); exact flips the seed's cluster
        itself instead of the smaller side."""
        sd = np.ascontiguousarray(seeds, np.int64)
        _check(lib().pticm_icm_pairs(self._h, _p(sd), len(sd), int(exact)))

    def layout(self) -> Layout:
        """Replicas per block, blocks, threads, ICM teams, block team, narrow
        kernel, staged adjacency, state mode (0 smem, 1 field gather, 2 global)."""
        out = Layout()
        _check(lib().pticm_get_layout(self._h, C.byref(out)))
        return out

    def exchange_order(self):
        """The pair order of the reference-order exchange (nt-1 entries)."""
        o = np.zeros(max(self.nt - 1, 1), np.uint32)
        _check(lib().pticm_get_exchange_order(self._h, _p(o)))
        return o[:self.nt - 1]

    def set_wait_limit(self, limit_ns=0, phantom_arrivals=0):
        """Limit of every wait on other blocks (0: 2 s); phantom_arrivals=1
        makes every group barrier wait for a block that never comes."""
        _check(lib().pticm_set_wait_limit(self._h, int(limit_ns), int(phantom_arrivals)))

    def set_profiling(self, enable=True):
        _check(lib().pticm_set_profiling(self._h, int(enable)))

    def profile(self):
        """Mean and max over blocks of ms per phase (the last entry, icm_pairs,
        counts ICM pairs with a nonempty overlap)."""
        mean = np.zeros(23)
        mx = np.zeros(23)
        _check(lib().pticm_get_profile(self._h, _p(mean), _p(mx)))
        names = ("sweep", "barrier", "exchange", "icm", "total", "icm_diff", "icm_seed", "icm_union",
                 "icm_flip", "icm_energy", "x_draw", "x_levels", "x_apply", "x_shuffle", "uf_link0",
                 "uf_compress", "uf_link1", "uf_vote", "uf_outside", "uf_s_unions", "uf_size", "sweep_icm",
                 "icm_pairs")
        return dict(zip(names, mean)), dict(zip(names, mx))

    def enable_energy_histograms(self, from_step=0):
        _check(lib().pticm_enable_energy_histograms(self._h, from_step))

    def observables(self):
        """Per temperature (chains merged): T, C, X, u, m and the sample count
        (the table of the reference's --log)."""
        out = [np.zeros(self.nt) for _ in range(5)]
        n = np.zeros(self.nt, np.uint64)
        _check(lib().pticm_get_observables(self._h, *[_p(a) for a in out], _p(n)))
        return (*out, n)

    def energy_histograms(self):
        """(histograms [R, nbins], energies of the bins [nbins])."""
        lo = C.c_int64()
        nb = C.c_uint64()
        _check(lib().pticm_get_energy_histograms(self._h, None, C.byref(lo), C.byref(nb)))
        h = np.zeros((self.R, nb.value), np.uint32)
        _check(lib().pticm_get_energy_histograms(self._h, _p(h), C.byref(lo), C.byref(nb)))
        return h, lo.value + 2 * np.arange(nb.value)

    def verify(self) -> int:
        mm = C.c_uint64()
        _check(lib().pticm_verify(self._h, C.byref(mm)))
        return mm.value

    def checkpoint_save(self, path: str):
        """Write the PT state (replicas, ladder, slot map, counters, step)."""
        _check(lib().pticm_checkpoint_save(self._h, os.fsencode(path)))

    def checkpoint_load(self, path: str):
        """Restore a checkpoint written by a context of the same problem and
        options; the run continues bit for bit."""
        _check(lib().pticm_checkpoint_load(self._h, os.fsencode(path)))

    def replay(self, trace: dict, pt_steps: int):
        """Run the reference's sequential algorithm from a recorded trace
        (keys: uniforms, sweep_offsets, xchg_pair, xchg_logu, icm_seed)."""
        u = np.ascontiguousarray(trace["uniforms"], np.float64)
        off = np.ascontiguousarray(trace["sweep_offsets"], np.uint64)
        xs = np.ascontiguousarray(trace["xchg_pair"], np.int32)
        xl = np.ascontiguousarray(trace["xchg_logu"], np.float64)
        seeds = np.ascontiguousarray(trace["icm_seed"], np.int64)
        t = Trace(pt_steps, u.ctypes.data, len(u), off.ctypes.data, xs.ctypes.data, xl.ctypes.data,
                  seeds.ctypes.data)
        _check(lib().pticm_replay(self._h, C.byref(t)))


def solve(problem: Problem, *, seed, Nt, pts, T0=0.6, T1=2.8, inverse=False, icm=False, sweeps=1,
          ladder=None, chains=2, exchange=1, **kw):
    """The reference's solve() (src/solver.cc:16-166) on the GPU: linear-beta
    ladder (or `ladder`), Bernoulli initial states, `pts` PT steps.  Returns
    the keys src/solver.cc:151-163 prints."""
    beta = beta_linspace(T0, T1, Nt, inverse) if ladder is None else np.asarray(ladder, np.float64)
    ctx = Context(problem, nt=len(beta), chains=chains, seed=seed, sweeps=sweeps, icm=icm,
                  exchange=exchange, **kw)
    ctx.set_ladder(beta)
    ctx.init_states(seed)
    ctx.run(pts)
    st, att, suc = ctx.stats()
    E, sweep, state, rep = ctx.best()
    Eb, cut = problem.evaluate(state[None, :])
    rates = np.where(att > 0, suc / np.maximum(att, 1), 0.0)
    return dict(swap_rates=rates, swap_attempts=att, swap_successes=suc, best_state_energy=float(Eb[0]),
                best_state_sweep=sweep, best_energy=E, best_maxcut=float(cut[0]), num_of_flips=st.flips,
                num_of_swaps=st.swaps, best_state=state, beta=beta, attempts=st.attempts,
                device_ms=st.last_run_ms, context=ctx)


class MLP:
    """The surrogate ln g(E) network on the tensor cores (pticm_mlp_*)."""

    def __init__(self, seed=0, batch=1024):
        self._h = C.c_void_p()
        _check(lib().pticm_mlp_create(seed, batch, C.byref(self._h)))
        self.n_params = int(lib().pticm_mlp_param_count())

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.pticm_mlp_destroy(self._h)
            self._h = None

    @property
    def params(self):
        out = np.zeros(self.n_params, np.float32)
        _check(lib().pticm_mlp_get_params(self._h, _p(out)))
        return out

    @params.setter
    def params(self, value):
        v = np.ascontiguousarray(value, np.float32)
        assert v.shape == (self.n_params,)
        _check(lib().pticm_mlp_set_params(self._h, _p(v)))

    def gradients(self, X, y):
        X = np.ascontiguousarray(X, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        g = np.zeros(self.n_params, np.float32)
        loss = C.c_float()
        _check(lib().pticm_mlp_gradients(self._h, _p(X), _p(y), len(y), _p(g), C.byref(loss)))
        return loss.value, g

    def train(self, X, y, steps, lr=1e-3, seed=0):
        X = np.ascontiguousarray(X, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        losses = np.zeros(steps, np.float32)
        _check(lib().pticm_mlp_train(self._h, _p(X), _p(y), len(y), steps, lr, seed, _p(losses)))
        return losses

    def predict(self, X):
        X = np.ascontiguousarray(X, np.float32)
        out = np.zeros(len(X), np.float32)
        _check(lib().pticm_mlp_predict(self._h, _p(X), len(X), _p(out)))
        return out


class Batch:
    """Many instances in one persistent launch (pticm_batch_*)."""

    def __init__(self, problems, *, nt, chains=2, seed=1, icm=True, exchange=1, sweeps=1, replicas_per_block=0,
                 block_threads=0, icm_algo=0):
        o = Opts()
        lib().pticm_opts_default(C.byref(o))
        o.seed, o.nt, o.chains, o.sweeps, o.icm, o.exchange = seed, nt, chains, sweeps, int(icm), exchange
        o.replicas_per_block, o.block_threads, o.icm_algo = replicas_per_block, block_threads, icm_algo
        self.problems = list(problems)
        self.count, self.nt, self.R = len(self.problems), nt, nt * chains
        arr = (C.c_void_p * self.count)(*[p._h for p in self.problems])
        self._h = C.c_void_p()
        _check(lib().pticm_batch_create(arr, self.count, C.byref(o), C.byref(self._h)))

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.pticm_batch_destroy(self._h)
            self._h = None

    def set_ladders(self, beta, nc=-1):
        b = np.ascontiguousarray(np.broadcast_to(np.asarray(beta, np.float64), (self.count, self.nt)))
        _check(lib().pticm_batch_set_ladders(self._h, _p(b), self.nt, nc))

    def init_states(self, seed):
        _check(lib().pticm_batch_init_states(self._h, seed))

    def autotune(self, trial_steps=20):
        _check(lib().pticm_batch_autotune(self._h, trial_steps))

    def run(self, steps, phase_mask=7):
        _check(lib().pticm_batch_run(self._h, steps, phase_mask))

    def info(self):
        i = BatchInfo()
        _check(lib().pticm_batch_get_info(self._h, C.byref(i)))
        return i

    def groups(self):
        g = np.zeros(self.count, np.uint32)
        t = np.zeros(self.count)
        st = np.zeros(self.count, np.int32)
        tm = np.zeros(self.count, np.int32)
        _check(lib().pticm_batch_get_groups(self._h, _p(g), _p(t), _p(st), _p(tm)))
        return g, t, st, tm

    def best(self):
        e = np.zeros(self.count)
        f = np.zeros(self.count, np.uint64)
        _check(lib().pticm_batch_get_best(self._h, _p(e), _p(f)))
        return e, f

    def best_state(self, inst):
        s = np.zeros(self.problems[inst].info().n, np.uint8)
        _check(lib().pticm_batch_get_best_state(self._h, inst, _p(s)))
        return s

    def swap_stats(self, inst):
        a = np.zeros(self.R, np.uint64)
        s = np.zeros(self.R, np.uint64)
        _check(lib().pticm_batch_get_swap_stats(self._h, inst, _p(a), _p(s)))
        return a, s

    def energies(self, inst):
        e = np.zeros(self.R, np.int64)
        sl = np.zeros(self.R, np.uint32)
        _check(lib().pticm_batch_get_energies(self._h, inst, _p(e), _p(sl)))
        return e, sl

    def verify(self):
        m = C.c_uint64()
        _check(lib().pticm_batch_verify(self._h, C.byref(m)))
        return m.value

    def enable_energy_histograms(self, from_step):
        _check(lib().pticm_batch_enable_energy_histograms(self._h, from_step))

    def energy_histograms(self, inst):
        lo = C.c_int64()
        nb = C.c_uint64()
        _check(lib().pticm_batch_get_energy_histograms(self._h, inst, None, C.byref(lo), C.byref(nb)))
        h = np.zeros((self.R, nb.value), np.uint32)
        _check(lib().pticm_batch_get_energy_histograms(self._h, inst, _p(h), C.byref(lo), C.byref(nb)))
        return h, lo.value + 2 * np.arange(nb.value)

    def compute_logdos(self, estep=2.0):
        """ln g of every instance in one device launch (cached for logdos)."""
        _check(lib().pticm_batch_compute_logdos(self._h, estep))

    def logdos(self, inst, estep=2.0):
        hb = C.c_uint64()
        _check(lib().pticm_batch_get_energy_histograms(self._h, inst, None, None, C.byref(hb)))
        cap = int(np.ceil(2 * hb.value / estep)) + 2
        d = np.zeros(cap)
        nb = C.c_uint64()
        me = C.c_double()
        it = C.c_uint64()
        _check(lib().pticm_batch_logdos(self._h, inst, estep, _p(d), cap, C.byref(nb), C.byref(me), C.byref(it)))
        return d[:nb.value], me.value, it.value
