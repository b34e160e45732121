"""The C ABI library loads and exports every function include/pticm.h
declares (no GPU calls)."""
import ctypes as C
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "pticm.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pticm_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_function():
    import pticm
    L = pticm.lib()
    names = _declared()
    assert len(names) > 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_host_only_entry_points_without_a_gpu():
    import numpy as np
    import pticm
    b = pticm.beta_linspace(0.5, 3.0, 8)
    assert b[0] == 1 / 3.0 and len(b) == 8
    assert pticm.lib().pticm_version().startswith(b"pticm-gb300")
    prob = pticm.Problem.load(os.path.join(ROOT, "tests", "golden", "graphs", "pmL10.gset"))
    info = prob.info()
    assert info.n == 100 and info.nnz == 400 and info.ncolors == 2
