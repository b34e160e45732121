"""The learned temperature ladder end to end on the GPU, at a small scale.

Training data comes from batched pilot runs and the FP64 multihistogram;
the network is trained by the tensor-core kernels.  On held-out instances:
* the predicted ln g agrees with the multihistogram ln g (after the free
  additive constant) to better than 2e-2 per spin;
* what the network gains over the method without it: its ladder's measured
  exchange acceptance is closer to the target than that of a ladder placed
  linearly in beta over the same range with the same number of temperatures,
  and the learned ladder (surrogate + acceptance check + feedback, with the
  multihistogram fallback) costs less time than the multihistogram ladder
  whenever it is accepted, at a measured acceptance within the tolerance;
* a saved network loads back to identical predictions.
"""
import os
import tempfile
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def trained():
    from pticm import instances as I, surrogate as S
    train = I.ladder_mix(384, seed0=100, L_range=(8, 24), n_range=(100, 600), deg_range=(3, 10))
    held = I.ladder_mix(8, seed0=700000, L_range=(8, 24), n_range=(100, 600), deg_range=(3, 10))
    recs = S.make_records(train, nt=24, burn_in=800, samples=2000, seed=3)
    hrec = S.make_records(held, nt=24, burn_in=800, samples=2000, seed=4)
    m, losses = S.train(recs, steps=2500, batch=1024, lr=1e-3, seed=1)
    return m, losses, held, hrec


def test_training_converges(trained):
    m, losses, _, _ = trained
    assert losses[-50:].mean() < 0.05 * losses[:10].mean()


def test_lng_error_against_multihistogram(trained):
    import pticm
    from pticm import surrogate as S
    m, _, held, hrec = trained
    errs = [S.lng_error(pticm.Problem.from_instance(x), m, r)[1] for x, r in zip(held, hrec)]
    assert np.mean(errs) < 2e-2, errs


def test_network_gains_over_the_method_without_it(trained):
    import pticm
    from pticm import surrogate as S
    m, _, held, _ = trained
    dev = lambda a: float(np.mean(np.abs(a - 0.4)))
    sur, lin, accepted = [], [], 0
    for i, x in enumerate(held):
        p = pticm.Problem.from_instance(x)
        T0, T1 = S.pilot_range(x)
        bs = S.surrogate_ladder(p, m, T0, T1, 24)
        bl = np.linspace(bs[0], bs[-1], len(bs))
        sur.append(dev(S.ladder_acceptance(p, bs, steps=2000, burn_in=400, seed=5 + i)))
        lin.append(dev(S.ladder_acceptance(p, bl, steps=2000, burn_in=400, seed=5 + i)))
        t = time.perf_counter()
        b_l, info = S.learned_ladder(p, m, T0, T1, 24, seed=9 + i)
        t_l = time.perf_counter() - t
        t = time.perf_counter()
        pticm.cae_ladder(p, seed=9 + i, T0=T0, T1=T1, nt=24)
        t_m = time.perf_counter() - t
        if not info.fallback:
            accepted += 1
            assert info.mean_deviation <= 0.05
            assert t_l < t_m, (t_l, t_m)
        else:
            assert len(b_l) >= 2
    assert np.mean(sur) < np.mean(lin), (sur, lin)
    assert accepted >= 1


def test_saved_network_predicts_the_same(trained):
    import pticm
    from pticm import surrogate as S
    m, _, held, _ = trained
    p = pticm.Problem.from_instance(held[0])
    d0 = S.surrogate_logdos(p, m)[0]
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "net.bin")
        S.save(m, path)
        m2 = S.load(path)
    assert np.array_equal(S.surrogate_logdos(p, m2)[0], d0)


def test_cli_learned_ladder(trained):
    """pt_icm --learned-ladder: the ladder comes from the saved network (or
    its multihistogram fallback) and the run reports as usual."""
    import re
    import subprocess
    from pticm import surrogate as S
    m, _, _, _ = trained
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    cli = os.path.join(root, "pt-icm_gb300", "bin", "pt_icm")
    graph = os.path.join(root, "tests", "golden", "graphs", "pmL20_c1.gset")
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "net.bin")
        S.save(m, path)
        out = subprocess.run([cli, "-p", graph, "-s", "3", "-r", "24", "--pts", "2000", "--icm", "-T0", "0.5",
                              "-T1", "3.0", "--learned-ladder", path, "--sort-ladder", "--verbose", "1"],
                             capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    m_l = re.search(r"learned ladder: (\d+) temperatures, (accepted|multihistogram fallback)", out.stdout)
    assert m_l and int(m_l.group(1)) >= 2
    assert re.search(r"^best_energy: -?[0-9.]+", out.stdout, re.M)
