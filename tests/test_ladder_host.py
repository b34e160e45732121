"""Host code of the learned ladder (no GPU): the feedback placement from
measured acceptances and the network's instance features."""
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_feedback_ladder_follows_the_gaussian_acceptance_model():
    special = pytest.importorskip("scipy.special")
    from pticm import surrogate as S
    lad = np.array([2.0, 1.5, 1.0, 0.5])
    acc = np.array([0.1, 0.4, 0.8])
    out = S.feedback_ladder(lad, acc, 400, 0.4, 32, 0.5)
    sigma = 2 * special.erfcinv(acc) / 0.5
    step = 2 * special.erfcinv(0.4)
    # walk: cold gap -> steps of step/sigma0, then the middle gap, then the hot gap
    b, want = 2.0, [2.0]
    while True:
        k = 0 if b > 1.5 else (1 if b > 1.0 else 2)
        nb = b - step / sigma[k]
        if nb <= 0.5:
            want.append(0.5)
            break
        want.append(nb)
        b = nb
    assert np.allclose(out, want, rtol=1e-9)
    # descending, starts at the coldest, ends at the hottest
    assert out[0] == 2.0 and out[-1] == 0.5 and np.all(np.diff(out) < 0)


def test_feedback_ladder_handles_gaps_without_exchanges_and_the_length_cap():
    from pticm import surrogate as S
    lad = np.array([2.0, 1.5, 1.0, 0.5])
    out = S.feedback_ladder(lad, np.array([0.0, 0.4, 1.0]), 400, 0.4, 32, 0.5)
    assert np.all(np.isfinite(out)) and np.all(np.diff(out) < 0) and out[-1] == 0.5
    capped = S.feedback_ladder(lad, np.array([0.0, 0.0, 0.0]), 400, 0.4, 6, 0.5)
    assert len(capped) == 6


def test_problem_features():
    import pticm
    from pticm import instances as I
    from pticm import surrogate as S
    lat = pticm.Problem.from_instance(I.pm_lattice(10, seed=1))
    f = S.problem_features(lat)
    assert np.isclose(f[0], np.log(100) / 10, atol=1e-6)      # ln N / 10
    assert np.isclose(f[1], np.log(200) / 12, atol=1e-6)      # ln M / 12
    assert np.isclose(f[2], 4 / 20, atol=1e-6)                # mean degree / 20
    assert abs(f[3]) < 1e-6                                   # regular lattice
    assert abs(f[4]) < 0.2 and np.isclose(f[5], np.sqrt(1 - f[4] ** 2), atol=1e-5)
    fer = S.problem_features(pticm.Problem.from_instance(I.pm_lattice(6, ferro=True)))
    assert np.isclose(fer[4], -1.0) and abs(fer[5]) < 1e-6
