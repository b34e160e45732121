"""The learned temperature ladder: data, training and evaluation.

Training data is what the method itself produces: a batched pilot PT run of
every training instance (one chain, no ICM, reference-order exchange, as the
reference's gather_samples, src/cae_estimator.cc:76-151) with per-
temperature energy histograms, and the FP64 multihistogram ln g(E) of each
instance (src/cae_estimator.cc:155-253) computed on the GPU.

ln g is known up to an additive constant.  Each estimate is anchored by the
high-temperature expansion of the partition function at the hottest pilot
temperature,

    ln Z(beta) = N ln 2 + sum_edges ln cosh(beta J_e) + sum_i ln cosh(beta h_i)

(exact on trees; closed loops add terms of order tanh(beta)^length), so the
target s = ln g / N is the entropy density, comparable across instances.

The network input is the six instance features of pticm_problem_features and
x = E / W.  Its output y is the deviation from the Gaussian (infinite-
temperature) entropy density, scaled by 10:

    s(x) = ln 2 - E^2 / (2 N V) + y / 10,     V = sum J^2 + sum h^2.

The ladder is the reference's constant-acceptance walk on the predicted
ln g at the energy levels the couplings allow, cut where ln g < 0 (no level
holds less than one state) -- the network's extrapolation below the lowest
energies it was trained on would otherwise put the cold distributions where
no state is (pticm_surrogate_ladder).
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math
import time

import numpy as np

from . import Batch, MLP, Problem, _check, _p, lib

N_FEATURES = 6


def problem_features(problem: Problem) -> np.ndarray:
    f = np.zeros(N_FEATURES, np.float32)
    _check(lib().pticm_problem_features(problem._h, _p(f)))
    return f


def pilot_range(inst) -> tuple[float, float]:
    """Temperatures the training pilots cover: T0 = 0.5 and T1 = max(3, 1.5
    sqrt(mean degree)), above the spin-glass transition of +-1 couplings on
    graphs of that degree."""
    deg = 2.0 * inst.m / max(inst.n, 1)
    return 0.5, max(3.0, 1.5 * math.sqrt(deg))


def _energy_bound(inst) -> float:
    w = float(np.abs(inst.w).sum())
    return w + (float(np.abs(inst.h).sum()) if inst.h is not None else 0.0)


def _lse(a):
    m = np.max(a)
    return m + math.log(np.exp(a - m).sum())


TARGET_SCALE = 10.0


def _variance(inst) -> float:
    v = float((inst.w ** 2).sum())
    return v + (float((inst.h ** 2).sum()) if inst.h is not None else 0.0)


@dataclasses.dataclass
class Record:
    features: np.ndarray   # 6 floats
    n: int
    W: float
    energy: np.ndarray     # exact levels with samples
    lng: np.ndarray        # anchored ln g at those levels
    T0: float
    T1: float
    V: float = 1.0


def make_records(instances, *, nt=32, burn_in=1000, samples=2000, seed=1, batch_size=512, log=None):
    """Batched pilots -> FP64 multihistogram ln g per instance, anchored."""
    records = []
    for b0 in range(0, len(instances), batch_size):
        chunk = instances[b0:b0 + batch_size]
        probs = [Problem.from_instance(x) for x in chunk]
        ladders = []
        for x in chunk:
            T0, T1 = pilot_range(x)
            ladders.append(1 / T0 + (1 / T1 - 1 / T0) * np.arange(nt) / (nt - 1))
        bat = Batch(probs, nt=nt, chains=1, seed=seed + b0, icm=False, exchange=0)
        bat.set_ladders(np.array(ladders))
        bat.init_states(seed + 7 * b0 + 1)
        bat.enable_energy_histograms(burn_in)
        t = time.perf_counter()
        bat.run(burn_in + samples)
        t_run = time.perf_counter() - t
        t = time.perf_counter()
        bat.compute_logdos()
        for i, (x, pr) in enumerate(zip(chunk, probs)):
            dos, emin, _ = bat.logdos(i)
            E = emin + 2.0 * np.arange(len(dos))
            ok = dos > -1e300
            T0, T1 = pilot_range(x)
            bmin = 1.0 / T1
            lnz_mh = _lse(dos[ok] - bmin * E[ok])
            lnz = x.n * math.log(2.0) + float(np.log(np.cosh(bmin * x.w)).sum())
            if x.h is not None:
                lnz += float(np.log(np.cosh(bmin * x.h)).sum())
            records.append(Record(problem_features(pr), x.n, _energy_bound(x), E[ok], dos[ok] + (lnz - lnz_mh),
                                  T0, T1, _variance(x)))
        if log:
            log(f"pilots {b0 + len(chunk)}/{len(instances)}: run {t_run:.2f} s, ln g {time.perf_counter() - t:.2f} s")
        del bat
    return records


def gaussian_entropy(E, n, V):
    return math.log(2.0) - np.asarray(E, np.float64) ** 2 / (2.0 * n * V)


def training_arrays(records, per_instance=96, seed=0):
    """Rows (features, x) and targets 10 (s - Gaussian s) at up to
    per_instance visited levels per record."""
    rng = np.random.default_rng(seed)
    X, y = [], []
    for r in records:
        k = len(r.energy)
        idx = np.arange(k) if k <= per_instance else np.sort(rng.choice(k, per_instance, replace=False))
        xs = r.energy[idx] / r.W
        ss = r.lng[idx] / r.n
        rows = np.empty((len(xs), N_FEATURES + 1), np.float32)
        rows[:, :N_FEATURES] = r.features
        rows[:, N_FEATURES] = xs
        X.append(rows)
        y.append((TARGET_SCALE * (ss - gaussian_entropy(xs * r.W, r.n, r.V))).astype(np.float32))
    return np.concatenate(X), np.concatenate(y)


def train(records, *, steps=3000, batch=1024, lr=1e-3, seed=0, per_instance=96, log=None):
    """The network trained on the GPU (tensor-core forward/backward, Adam):
    `steps` at lr, then steps/3 at lr/10."""
    X, y = training_arrays(records, per_instance, seed)
    m = MLP(seed=seed, batch=batch)
    t = time.perf_counter()
    l1 = m.train(X, y, steps, lr=lr, seed=seed)
    l2 = m.train(X, y, max(1, steps // 3), lr=lr / 10, seed=seed + 1)
    if log:
        log(f"trained on {len(y)} samples: loss {l1[:10].mean():.3e} -> {l2[-50:].mean():.3e} "
            f"in {time.perf_counter() - t:.2f} s")
    return m, np.concatenate([l1, l2])


def surrogate_logdos(problem: Problem, m: MLP):
    """(ln g at levels emin + k*estep <= 0, emin, estep)."""
    nb = C.c_uint64()
    emin = C.c_double()
    est = C.c_double()
    _check(lib().pticm_surrogate_logdos(problem._h, m._h, None, 0, C.byref(nb), C.byref(emin), C.byref(est)))
    d = np.zeros(nb.value)
    _check(lib().pticm_surrogate_logdos(problem._h, m._h, _p(d), nb.value, C.byref(nb), C.byref(emin),
                                        C.byref(est)))
    return d, emin.value, est.value


def lng_error(problem: Problem, m: MLP, rec: Record):
    """RMS of predicted minus multihistogram ln g over the record's levels,
    after removing the best constant (ln g is defined up to one): absolute
    and per spin."""
    d, emin, est = surrogate_logdos(problem, m)
    k = np.round((rec.energy - emin) / est).astype(np.int64)
    keep = (k >= 0) & (k < len(d)) & (np.abs(emin + k * est - rec.energy) < 0.5)
    diff = d[k[keep]] - rec.lng[keep]
    rms = float(np.sqrt(np.mean((diff - diff.mean()) ** 2)))
    return rms, rms / rec.n


def surrogate_ladder(problem: Problem, m: MLP, T0, T1, nt, r=0.4, step_size=0.1, inverse=False):
    out = np.zeros(nt)
    cnt = C.c_uint32()
    _check(lib().pticm_surrogate_ladder(problem._h, m._h, T0, T1, int(inverse), nt, step_size, r, _p(out),
                                        C.byref(cnt)))
    return out[:cnt.value]


class LearnedLadderInfo(C.Structure):
    _fields_ = [("surrogate_count", C.c_uint32), ("fallback", C.c_int32), ("mean_deviation", C.c_double),
                ("rounds", C.c_uint32), ("inserted", C.c_uint32), ("first_deviation", C.c_double)]


def feedback_ladder(beta, acc, attempts, r, nt, beta_end):
    b = np.ascontiguousarray(beta, np.float64)
    a = np.ascontiguousarray(acc, np.float64)
    out = np.zeros(nt)
    cnt = C.c_uint32()
    _check(lib().pticm_feedback_ladder(_p(b), len(b), _p(a), attempts, r, nt, beta_end, _p(out), C.byref(cnt)))
    return out[:cnt.value]


def learned_ladder(problem: Problem, m: MLP, T0, T1, nt, r=0.4, check_steps=1000, tol=0.05, seed=1,
                   inverse=False):
    out = np.zeros(nt)
    cnt = C.c_uint32()
    info = LearnedLadderInfo()
    _check(lib().pticm_learned_ladder(problem._h, m._h, T0, T1, int(inverse), nt, r, check_steps, tol, seed,
                                      _p(out), C.byref(cnt), C.byref(info)))
    return out[:cnt.value], info


def ladder_acceptance(problem: Problem, beta, steps=2000, burn_in=500, seed=1):
    b = np.ascontiguousarray(beta, np.float64)
    acc = np.zeros(max(len(b) - 1, 1))
    _check(lib().pticm_ladder_acceptance(problem._h, _p(b), len(b), seed, steps, burn_in, _p(acc)))
    return acc[:len(b) - 1]


def save(m: MLP, path: str):
    _check(lib().pticm_mlp_save(m._h, path.encode()))


def load(path: str, batch=1024) -> MLP:
    m = MLP(seed=0, batch=batch)
    _check(lib().pticm_mlp_load(m._h, path.encode()))
    return m
