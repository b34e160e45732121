"""ctypes binding of the C oracle (oracle/pticm_oracle.c) and a runner for
the single-rank reference build (oracle/_ref/pt_icm_ref).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as
the checker and by bench.py's CPU-baseline legs.  The product never imports
this module.
"""
from __future__ import annotations

import ctypes as C
import os
import re
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_BIN = os.path.join(HERE, "_ref", "pt_icm_ref")

_lib = None


def build(force: bool = False) -> str:
    """Compile liboracle.so from pticm_oracle.c (gcc, no FMA contraction so
    that the FP64 arithmetic matches the reference's x86-64 build)."""
    src = os.path.join(HERE, "pticm_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        tmp = LIB_PATH + ".tmp"
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
                               "-o", tmp, src, "-lm"])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


class Params(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("Nt", C.c_uint64), ("pts", C.c_uint64),
                ("sweeps", C.c_uint64), ("pre_samples", C.c_uint64),
                ("pilot_burn_in", C.c_uint64), ("T0", C.c_double), ("T1", C.c_double),
                ("pre_step", C.c_double), ("inverse", C.c_int), ("preprocess", C.c_int),
                ("icm", C.c_int)]


class Result(C.Structure):
    _fields_ = [("Nt", C.c_uint64), ("Nc", C.c_uint32), ("beta", C.c_double * 2048),
                ("swap_attempts", C.c_uint32 * 2048), ("swap_successes", C.c_uint32 * 2048),
                ("swaps", C.c_uint64), ("best_energy", C.c_double), ("best_sweep", C.c_uint64),
                ("best_state_energy", C.c_double), ("best_maxcut", C.c_double),
                ("flips", C.c_uint64), ("flips_u64", C.c_uint64), ("char_scale", C.c_double)]


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        L.orc_problem_load.argtypes = [C.c_char_p, C.c_uint64, C.POINTER(P)]
        L.orc_problem_from_coo.argtypes = [C.c_int64, C.c_int64, P, P, P, P, C.c_uint64, C.POINTER(P)]
        L.orc_problem_free.argtypes = [P]
        for f in ("orc_problem_n", "orc_problem_m", "orc_problem_nnz"):
            getattr(L, f).argtypes = [P]
            getattr(L, f).restype = C.c_int64
        L.orc_problem_sparse.argtypes = [P]
        L.orc_problem_char_scale.argtypes = [P]
        L.orc_problem_char_scale.restype = C.c_double
        L.orc_problem_adjacency.argtypes = [P, P, P, P]
        L.orc_problem_linear.argtypes = [P, P]
        L.orc_problem_rng.argtypes = [P]
        L.orc_problem_rng.restype = P
        for f in ("orc_energy", "orc_maxcut"):
            getattr(L, f).argtypes = [P, P]
            getattr(L, f).restype = C.c_double
        L.orc_calculate_dE.argtypes = [P, P, P]
        L.orc_calculate_dE.restype = C.c_double
        L.orc_mt64_seed.argtypes = [P, C.c_uint64]
        L.orc_mt64_next.argtypes = [P]
        L.orc_mt64_next.restype = C.c_uint64
        L.orc_canonical.argtypes = [P]
        L.orc_canonical.restype = C.c_double
        L.orc_uniform_index.argtypes = [P, C.c_uint64]
        L.orc_uniform_index.restype = C.c_uint64
        L.orc_shuffle_u32.argtypes = [P, C.c_uint64, P]
        L.orc_sample_one.argtypes = [C.c_uint64, P]
        L.orc_sample_one.restype = C.c_int64
        L.orc_sweep_stream.argtypes = [P, C.c_double, P, P, P, P, P, P, C.c_uint64, P, C.c_uint64, P]
        L.orc_sweep_stream.restype = C.c_uint64
        L.orc_sweep.argtypes = [P, C.c_double, P, P, P, P, P, P, C.c_uint64, P, C.c_uint64, P]
        L.orc_sweep.restype = C.c_uint64
        L.orc_beta_linspace.argtypes = [P, C.c_double, C.c_double, C.c_uint64, C.c_int]
        L.orc_trace_new.restype = P
        L.orc_trace_new_energy_only.restype = P
        L.orc_overlap.argtypes = [P, P, P, P]
        L.orc_overlap.restype = C.c_int64
        L.orc_bfs_icm.argtypes = [P, C.c_int64, P, P]
        L.orc_trace_free.argtypes = [P]
        for f in ("orc_trace_n_uniforms", "orc_trace_n_sweeps", "orc_trace_n_exchange",
                  "orc_trace_n_icm", "orc_trace_n_init", "orc_trace_n_energy"):
            getattr(L, f).argtypes = [P]
            getattr(L, f).restype = C.c_uint64
        L.orc_trace_copy.argtypes = [P] + [P] * 7
        L.orc_solve.argtypes = [P, C.POINTER(Params), C.POINTER(Result), P, P, P, P]
        L.orc_solve.restype = C.c_int
        L.orc_solve_timed.argtypes = [P, C.POINTER(Params), C.POINTER(Result), C.c_uint64, P]
        L.orc_solve_timed.restype = C.c_int
        L.orc_logplusexp2.argtypes = [C.c_double, C.c_double]
        L.orc_logplusexp2.restype = C.c_double
        L.orc_partition_func.argtypes = [P, C.c_uint64, C.c_double, C.c_double, C.c_double]
        L.orc_partition_func.restype = C.c_double
        L.orc_partition_iterate.argtypes = [P, P, P, C.c_uint64, P, P, C.c_double, C.c_uint64,
                                            C.c_double, P, P]
        L.orc_partition_iterate.restype = C.c_uint64
        L.orc_acceptance_rate.argtypes = [P, C.c_uint64, P, P, C.c_double, C.c_double,
                                          C.c_double, C.c_double]
        L.orc_acceptance_rate.restype = C.c_double
        L.orc_cae_walk.argtypes = [P, C.c_uint64, C.c_double, C.c_double, C.c_double, C.c_double,
                                   C.c_double, C.c_double, C.c_uint64, P]
        L.orc_cae_walk.restype = C.c_uint64
        L.orc_get_beta.argtypes = [P, C.c_double, C.c_double, C.c_int, C.c_uint64, C.c_double,
                                   C.c_double, C.c_double, C.c_uint64, C.c_uint64, P, P, P, P]
        L.orc_get_beta.restype = C.c_uint64
        L.orc_pilot.argtypes = [P, P, C.c_uint64, C.c_double, C.c_uint64, C.c_uint64, P, C.c_uint64, P, P, P, P, P]
        L.orc_pilot.restype = C.c_uint64
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class Problem:
    """Restated `pticm::Problem` (src/problem.cc) owning its mt19937_64."""

    def __init__(self, handle):
        self.h = handle

    @classmethod
    def load(cls, path: str, seed: int = 0) -> "Problem":
        h = C.c_void_p()
        rc = lib().orc_problem_load(path.encode(), seed, C.byref(h))
        if rc:
            raise ValueError(f"oracle could not parse {path} (code {rc})")
        return cls(h)

    @classmethod
    def from_coo(cls, n, src, dst, w, h=None, seed=0) -> "Problem":
        src = np.ascontiguousarray(src, dtype=np.int32)
        dst = np.ascontiguousarray(dst, dtype=np.int32)
        w = np.ascontiguousarray(w, dtype=np.float64)
        hh = None if h is None else np.ascontiguousarray(h, dtype=np.float64)
        out = C.c_void_p()
        rc = lib().orc_problem_from_coo(n, len(src), _p(src), _p(dst), _p(w), _p(hh), seed,
                                        C.byref(out))
        if rc:
            raise ValueError(f"bad COO (code {rc})")
        return cls(out)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_problem_free(self.h)
            self.h = None

    @property
    def n(self):
        return lib().orc_problem_n(self.h)

    @property
    def m(self):
        return lib().orc_problem_m(self.h)

    @property
    def sparse(self):
        return bool(lib().orc_problem_sparse(self.h))

    @property
    def char_scale(self):
        return lib().orc_problem_char_scale(self.h)

    def adjacency(self):
        nnz = lib().orc_problem_nnz(self.h)
        row = np.zeros(self.n + 1, np.int64)
        col = np.zeros(max(nnz, 1), np.int64)
        w = np.zeros(max(nnz, 1), np.float64)
        lib().orc_problem_adjacency(self.h, _p(row), _p(col), _p(w))
        return row, col[:nnz], w[:nnz]

    def linear(self):
        h = np.zeros(self.n, np.float64)
        lib().orc_problem_linear(self.h, _p(h))
        return h

    def energy(self, s):
        s = np.ascontiguousarray(s, dtype=np.uint8)
        return lib().orc_energy(self.h, _p(s))

    def maxcut(self, s):
        s = np.ascontiguousarray(s, dtype=np.uint8)
        return lib().orc_maxcut(self.h, _p(s))

    def calculate_dE(self, s):
        s = np.ascontiguousarray(s, dtype=np.uint8)
        dE = np.zeros(self.n, np.float64)
        E = lib().orc_calculate_dE(self.h, _p(s), _p(dE))
        return E, dE

    def rng(self):
        return lib().orc_problem_rng(self.h)


def sweep_stream(prob: Problem, beta, s, uniforms, n_sweeps=1):
    """Sequential Metropolis sweeps (src/replica.cc:5-38) consuming a given
    uniform stream.  Returns a dict with the final state and bookkeeping."""
    s = np.array(s, dtype=np.uint8)
    E, dE = prob.calculate_dE(s)
    u = np.ascontiguousarray(uniforms, dtype=np.float64)
    Ec = C.c_double(E)
    bE = C.c_double(np.finfo(np.float64).max)
    bS = C.c_uint64(0)
    pos = C.c_uint64(0)
    best = s.copy()
    flips = 0
    energies = []
    for k in range(n_sweeps):
        flips += lib().orc_sweep_stream(prob.h, beta, _p(s), _p(dE), C.byref(Ec), C.byref(bE),
                                        C.byref(bS), _p(best), k, _p(u), len(u), C.byref(pos))
        energies.append(Ec.value)
    return dict(state=s, dE=dE, energy=Ec.value, best_energy=bE.value, best_sweep=bS.value,
                best_state=best, flips=flips, consumed=pos.value, energies=energies)


def overlap(prob: Problem, s1, s2):
    """xor_icm's overlap (src/icm.cc:8-31) without the seed draw: returns s1
    (negated when more than N/2 sites differ) and the differing sites."""
    a = np.array(s1, dtype=np.uint8)
    b = np.ascontiguousarray(s2, dtype=np.uint8)
    sites = np.zeros(max(prob.n, 1), np.int64)
    cnt = lib().orc_overlap(prob.h, _p(a), _p(b), _p(sites))
    return a, sites[:cnt]


def bfs_icm(prob: Problem, seed, s1, s2):
    """bfs_icm (src/icm.cc:37-72): both states with the seed's cluster of
    differing sites flipped."""
    a = np.array(s1, dtype=np.uint8)
    b = np.array(s2, dtype=np.uint8)
    lib().orc_bfs_icm(prob.h, int(seed), _p(a), _p(b))
    return a, b


def solve(prob: Problem, *, seed, Nt, pts, sweeps=1, T0=0.6, T1=2.8, inverse=False, icm=False,
          preprocess=False, pre_samples=2000, pre_step=0.1, pilot_burn_in=5000, trace=False,
          energies=False):
    """`pticm::solve` on one rank (src/solver.cc:16-166).  The problem's engine
    is re-seeded with `seed` first, as src/problem.cc:183 does.  trace=True
    records every random decision; energies=True records only the slot
    energies after the sweeps of each step (out["step_energy"], [pts, 2 Nt])."""
    L = lib()
    L.orc_mt64_seed(prob.rng(), seed)
    prm = Params(seed, Nt, pts, sweeps, pre_samples, pilot_burn_in, T0, T1, pre_step,
                 int(inverse), int(preprocess), int(icm))
    res = Result()
    n = prob.n
    best = np.zeros(n, np.uint8)
    states = np.zeros(2 * Nt * n, np.uint8)
    fe = np.zeros(2 * Nt, np.float64)
    tr = L.orc_trace_new() if trace else (L.orc_trace_new_energy_only() if energies else None)
    rc = L.orc_solve(prob.h, C.byref(prm), C.byref(res), _p(best), _p(states), _p(fe), tr)
    if rc:
        if tr:
            L.orc_trace_free(tr)
        raise RuntimeError(f"oracle solve failed ({rc})")
    nt = res.Nt
    R = 2 * nt
    out = dict(Nt=nt, Nc=res.Nc, beta=np.array(res.beta[:R]),
               swap_attempts=np.array(res.swap_attempts[:R], np.uint32),
               swap_successes=np.array(res.swap_successes[:R], np.uint32),
               swaps=res.swaps, best_energy=res.best_energy, best_sweep=res.best_sweep,
               best_state_energy=res.best_state_energy, best_maxcut=res.best_maxcut,
               flips=res.flips, flips_u64=res.flips_u64, best_state=best,
               states=states[: R * n].reshape(R, n), final_energy=fe[:R], char_scale=res.char_scale)
    if tr and not trace:
        ne = L.orc_trace_n_energy(tr)
        se = np.zeros(max(ne, 1))
        L.orc_trace_copy(tr, None, None, None, None, None, None, _p(se))
        L.orc_trace_free(tr)
        out["step_energy"] = se[:ne].reshape(-1, R) if ne else np.zeros((0, R))
    elif tr:
        nu = L.orc_trace_n_uniforms(tr)
        ns = L.orc_trace_n_sweeps(tr)
        nx = L.orc_trace_n_exchange(tr)
        ni = L.orc_trace_n_icm(tr)
        nin = L.orc_trace_n_init(tr)
        ne = L.orc_trace_n_energy(tr)
        t = dict(uniforms=np.zeros(max(nu, 1)), sweep_offsets=np.zeros(ns + 1, np.uint64),
                 xchg_pair=np.zeros(max(nx, 1), np.int32), xchg_logu=np.zeros(max(nx, 1)),
                 icm_seed=np.zeros(max(ni, 1), np.int64), init_states=np.zeros(max(nin, 1), np.uint8),
                 step_energy=np.zeros(max(ne, 1)))
        L.orc_trace_copy(tr, _p(t["uniforms"]), _p(t["sweep_offsets"]), _p(t["xchg_pair"]),
                         _p(t["xchg_logu"]), _p(t["icm_seed"]), _p(t["init_states"]),
                         _p(t["step_energy"]))
        L.orc_trace_free(tr)
        t["uniforms"] = t["uniforms"][:nu]
        t["xchg_pair"] = t["xchg_pair"][:nx]
        t["xchg_logu"] = t["xchg_logu"][:nx]
        t["icm_seed"] = t["icm_seed"][:ni]
        t["init_states"] = t["init_states"][:nin].reshape(R, n)
        t["step_energy"] = t["step_energy"][:ne].reshape(-1, R) if ne else np.zeros((0, R))
        out["trace"] = t
    return out


def solve_timed(prob: Problem, *, seed, Nt, pts, timed_from, T0=0.6, T1=2.8, icm=False, sweeps=1):
    """solve() timing its main loop from PT step `timed_from` on: (wall
    seconds of steps timed_from..pts-1, best energy)."""
    L = lib()
    L.orc_mt64_seed(prob.rng(), seed)
    prm = Params(seed, Nt, pts, sweeps, 2000, 5000, T0, T1, 0.1, 0, 0, int(icm))
    res = Result()
    sec = C.c_double()
    rc = L.orc_solve_timed(prob.h, C.byref(prm), C.byref(res), timed_from, C.byref(sec))
    if rc:
        raise RuntimeError(f"oracle solve failed ({rc})")
    return sec.value, res.best_energy


def beta_linspace(T0, T1, nt, inverse=False):
    b = np.zeros(nt)
    lib().orc_beta_linspace(_p(b), T0, T1, nt, int(inverse))
    return b


def get_beta(prob: Problem, *, seed, T0, T1, Nt, inverse=False, estep=2.0, step_size=0.1,
             r=0.4, samples=2000, burn_in=5000):
    """get_beta of src/cae_estimator.cc:295-428 (pilot run + CAE walk)."""
    L = lib()
    L.orc_mt64_seed(prob.rng(), seed)
    out = np.zeros(Nt)
    hb = np.zeros(Nt)
    emn = np.zeros(Nt)
    emx = np.zeros(Nt)
    cnt = L.orc_get_beta(prob.h, T0, T1, int(inverse), Nt, estep, step_size, r, samples, burn_in,
                         _p(out), _p(hb), _p(emn), _p(emx))
    return dict(count=cnt, beta=out[:cnt], hist_betas=hb, emin=emn, emax=emx)


def pilot(prob: Problem, *, seed, hist_betas, estep=2.0, samples=2000, burn_in=5000):
    """The pilot run and histograms of get_beta (src/cae_estimator.cc:76-151,
    45-69) on the given hist_betas."""
    L = lib()
    L.orc_mt64_seed(prob.rng(), seed)
    hb = np.ascontiguousarray(hist_betas, np.float64)
    nt = len(hb)
    off = np.zeros(nt, np.uint64)
    ln = np.zeros(nt, np.uint64)
    emn = np.zeros(nt)
    emx = np.zeros(nt)
    n = C.c_uint64()
    cap = 1 << 24
    h = np.zeros(cap, np.uint32)
    tot = L.orc_pilot(prob.h, _p(hb), nt, estep, samples, burn_in, _p(h), cap, _p(off), _p(ln), _p(emn), _p(emx),
                      C.byref(n))
    return dict(hist=h[:tot].copy(), hist_off=off, hist_len=ln, emin=emn, emax=emx, n=n.value, hist_betas=hb)


def partition_iterate(hist, hist_off, hist_len, beta_hist, emin, estep, n, max_emax):
    """get_partition_iterate (src/cae_estimator.cc:228-253): (ln g, ln Z)."""
    L = lib()
    nt = len(beta_hist)
    nb = int(np.ceil((max_emax - np.min(emin)) / estep))
    dos = np.zeros(max(nb, 1))
    z = np.zeros(nt)
    hist = np.ascontiguousarray(hist, np.uint32)
    off = np.ascontiguousarray(hist_off, np.uint64)
    ln = np.ascontiguousarray(hist_len, np.uint64)
    b = np.ascontiguousarray(beta_hist, np.float64)
    e = np.ascontiguousarray(emin, np.float64)
    it = L.orc_partition_iterate(_p(hist), _p(off), _p(ln), nt, _p(b), _p(e), estep, n, max_emax, _p(dos), _p(z))
    return dos[:nb], z, it


def cae_walk(logdos, min_emin, estep, beta_start, beta_end, step_size, r, num_temps):
    d = np.ascontiguousarray(logdos, np.float64)
    out = np.zeros(num_temps)
    cnt = lib().orc_cae_walk(_p(d), len(d), min_emin, estep, beta_start, beta_end, step_size, r, num_temps, _p(out))
    return out[:cnt]


# ----------------------------------------------------------- reference runs
def have_reference() -> bool:
    return os.path.exists(REF_BIN)


_KEYS_INT_LIST = ("swap_attempts", "swap_successes")


def run_reference(problem_path: str, *, seed, Nt, pts, T0=0.6, T1=2.8, icm=False,
                  preprocess=False, inverse=False, sweeps=1, pre_samples=2000, pre_step=0.1,
                  timeout=600):
    """Run the unmodified reference (single-rank build) and parse its report
    (src/solver.cc:151-163)."""
    args = [REF_BIN, "-p", problem_path, "-s", str(seed), "-r", str(Nt), "--pts", str(pts),
            "-T0", repr(float(T0)), "-T1", repr(float(T1)), "--sweeps", str(sweeps),
            "--preprocess-samples", str(pre_samples), "--preprocess-stepsize", repr(float(pre_step))]
    if icm:
        args.append("--icm")
    if preprocess:
        args.append("--preprocess")
    if inverse:
        args.append("--inverse")
    out = subprocess.run(args, capture_output=True, text=True, timeout=timeout, check=True).stdout
    res = {}
    for line in out.splitlines():
        m = re.match(r"^(\w+): (.*)$", line.strip())
        if not m:
            if line.startswith("[") and "best_state" in res and "ladder" not in res:
                res["ladder"] = [float(x) for x in line.strip()[1:-1].split(",") if x.strip()]
            continue
        k, v = m.group(1), m.group(2).strip()
        if k in _KEYS_INT_LIST:
            res[k] = [int(x) for x in v[1:-1].split(",") if x.strip()]
        elif k == "swap_rates":
            res[k] = [float(x) for x in v[1:-1].split(",") if x.strip()]
        elif k == "best_state":
            res[k] = [int(x) for x in v[1:-1].split(",") if x.strip()]
        elif k in ("best_energy", "best_state_energy", "best_maxcut"):
            res[k] = float(v)
        elif k in ("num_of_flips", "num_of_swaps", "best_state_sweep"):
            res[k] = int(v)
    m = re.search(r"Total time: ([0-9.eE+-]+)", out)
    if m:
        res["total_time"] = float(m.group(1))
    return res
