"""Seeded synthetic instances in the shapes the PT-ICM workloads are quoted on,
and a Gset writer.

Gset text layout (read by src/problem.cc:183-247 of the reference): a header
``N M`` (``N num_linear M`` for ``.ising``), then one ``u v w`` line per edge.
Vertices are 0-based when the file name contains ``.gset`` or ``.ising`` and
1-based otherwise (src/problem.cc:208).

Workload shapes:
  * ``pm_lattice(L)``  2-D toroidal Edwards-Anderson lattice, J = +-1
    equiprobable, edges site->right and site->down (C1: L=20).
  * ``random_graph(n, m)``  m distinct uniform pairs, weights +1 or +-1
    (C2: n=2000, m=19990, w=+1; C5: n=20000, m=400000, +-1).
  * ``batch_mix(count)``  the uneven 1024-instance mix of the batched workload.
  * ``ladder_mix(count)``  lattices and random graphs of the learned-ladder
    workload (training and held-out sets).
"""
from __future__ import annotations

import dataclasses
import math
import os

import numpy as np


@dataclasses.dataclass
class Instance:
    n: int
    src: np.ndarray          # int32, 0-based
    dst: np.ndarray          # int32, 0-based
    w: np.ndarray            # float64 couplings J_ij
    h: np.ndarray | None = None  # float64 linear terms or None
    name: str = ""

    @property
    def m(self) -> int:
        return int(self.src.shape[0])

    def write_gset(self, path: str) -> str:
        """Write in Gset layout; the index base follows the file name rule."""
        zero = (".gset" in path) or (".ising" in path)
        off = 0 if zero else 1
        lines = []
        if ".ising" in path:
            hh = self.h if self.h is not None else np.zeros(self.n)
            nz = np.nonzero(hh)[0]
            lines.append(f"{self.n} {len(nz)} {self.m}")
            for i in nz:
                lines.append(f"{i + off} {_fmt(hh[i])}")
        else:
            lines.append(f"{self.n} {self.m}")
        for u, v, w in zip(self.src.tolist(), self.dst.tolist(), self.w.tolist()):
            lines.append(f"{u + off} {v + off} {_fmt(w)}")
        with open(path, "w") as f:
            f.write("\n".join(lines) + "\n")
        return path


def _fmt(x: float) -> str:
    return str(int(x)) if float(x).is_integer() else repr(float(x))


def pm_lattice(L: int, seed: int = 1, ferro: bool = False) -> Instance:
    """Periodic L x L lattice; J = +-1 equiprobable from `seed` (or -1 for a
    ferromagnet in the reference's sign convention, E = sum J s_i s_j)."""
    rng = np.random.default_rng(seed)
    src, dst = [], []
    for r in range(L):
        for c in range(L):
            i = r * L + c
            src.append(i)
            dst.append(r * L + (c + 1) % L)
            src.append(i)
            dst.append(((r + 1) % L) * L + c)
    m = len(src)
    w = -np.ones(m) if ferro else rng.choice(np.array([-1.0, 1.0]), size=m)
    return Instance(L * L, np.array(src, np.int32), np.array(dst, np.int32), w,
                    name=f"pm_lattice_L{L}_s{seed}")


def random_graph(n: int, m: int, seed: int = 2, signed: bool = False) -> Instance:
    """m distinct unordered pairs drawn uniformly; w = +1, or +-1 if signed."""
    rng = np.random.default_rng(seed)
    total = n * (n - 1) // 2
    if m > total:
        raise ValueError("more edges than vertex pairs")
    seen = set()
    src = np.empty(m, np.int32)
    dst = np.empty(m, np.int32)
    k = 0
    while k < m:
        need = m - k
        a = rng.integers(0, n, size=2 * need + 16)
        b = rng.integers(0, n, size=2 * need + 16)
        for x, y in zip(a.tolist(), b.tolist()):
            if x == y:
                continue
            key = (x, y) if x < y else (y, x)
            if key in seen:
                continue
            seen.add(key)
            src[k], dst[k] = key
            k += 1
            if k == m:
                break
    w = rng.choice(np.array([-1.0, 1.0]), size=m) if signed else np.ones(m)
    return Instance(n, src, dst, w, name=f"random_n{n}_m{m}_s{seed}")


def batch_mix(count: int = 1024, seed0: int = 1000):
    """The uneven batched workload: half +-J lattices with L from {10,20,32,50},
    half random graphs with n log-uniform in [200, 5000], mean degree uniform
    in [3, 20] and +-1 weights; instance i uses seed seed0 + i."""
    out = []
    for i in range(count):
        rng = np.random.default_rng(seed0 + i)
        if i % 2 == 0:
            L = int(rng.choice([10, 20, 32, 50]))
            out.append(pm_lattice(L, seed=seed0 + i))
        else:
            n = int(round(math.exp(rng.uniform(math.log(200), math.log(5000)))))
            deg = rng.uniform(3, 20)
            m = max(1, int(round(n * deg / 2)))
            out.append(random_graph(n, m, seed=seed0 + i, signed=True))
    return out


def ladder_mix(count: int, seed0: int = 5000, L_range=(6, 50), n_range=(100, 3000), deg_range=(3.0, 20.0)):
    """Instances of the learned-ladder workload: half +-J toroidal lattices
    with L uniform in L_range, half random +-1 graphs with n log-uniform in
    n_range and mean degree uniform in deg_range; instance i uses seed
    seed0 + i."""
    out = []
    for i in range(count):
        rng = np.random.default_rng(seed0 + i)
        if i % 2 == 0:
            out.append(pm_lattice(int(rng.integers(L_range[0], L_range[1] + 1)), seed=seed0 + i))
        else:
            n = int(round(math.exp(rng.uniform(math.log(n_range[0]), math.log(n_range[1])))))
            deg = rng.uniform(*deg_range)
            m = min(n * (n - 1) // 2, max(1, int(round(n * deg / 2))))
            out.append(random_graph(n, m, seed=seed0 + i, signed=True))
    return out


def c1() -> Instance:
    """+-J lattice L=20 (N=400, M=800) from seed 1."""
    return pm_lattice(20, seed=1)


def c2() -> Instance:
    """Random sparse MaxCut graph N=2000, M=19990, w=+1, from seed 2."""
    return random_graph(2000, 19990, seed=2, signed=False)


def c5() -> Instance:
    """Random +-1 MaxCut graph N=20000, mean degree 40 (M=400000), seed 5."""
    return random_graph(20000, 400000, seed=5, signed=True)


def write_to(inst: Instance, directory: str, fname: str) -> str:
    os.makedirs(directory, exist_ok=True)
    return inst.write_gset(os.path.join(directory, fname))
