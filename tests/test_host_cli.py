"""The pt_icm command line's argument handling (host only, no GPU): --help
lists the reference's flags (src/main.cc:33-48) and exits 0; an unknown
argument or a missing --problem prints the error and the usage and exits 1;
an unreadable problem file fails; without a GPU the run fails loudly (the
engine has no CPU path)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "pt-icm_gb300", "bin", "pt_icm")
G = os.path.join(ROOT, "tests", "golden", "graphs")

REFERENCE_FLAGS = ["-s", "--seed", "-p", "--problem", "-b", "--burn_in", "--sweeps", "-r", "--replicas", "--pts",
                   "--preprocess-samples", "--preprocess-stepsize", "-T0", "--temp0", "-T1", "--temp1", "-i",
                   "--inverse", "--preprocess", "--log", "--icm", "--verbose"]


@pytest.fixture(scope="module")
def cli():
    if not os.path.exists(CLI):
        pytest.skip("pt_icm is not built (python -c 'import __graft_entry__ as g; g.build()')")
    return CLI


def _run(cli, *args):
    return subprocess.run([cli, *args], capture_output=True, text=True, timeout=120)


def test_help_lists_the_reference_flags(cli):
    r = _run(cli, "--help")
    assert r.returncode == 0
    for flag in REFERENCE_FLAGS:
        assert flag in r.stdout, flag


def test_unknown_argument_exits_1(cli):
    r = _run(cli, "-p", os.path.join(G, "pmL6.gset"), "--no-such-flag")
    assert r.returncode == 1
    assert "unknown argument --no-such-flag" in r.stdout
    assert "Usage:" in r.stdout


def test_missing_problem_exits_1(cli):
    r = _run(cli, "-s", "3")
    assert r.returncode == 1
    assert "--problem is required" in r.stdout


def test_unreadable_problem_fails(cli, tmp_path):
    r = _run(cli, "-p", str(tmp_path / "missing"), "-s", "1")
    assert r.returncode != 0
    assert "cannot open" in r.stdout + r.stderr


def test_run_without_a_gpu_fails_loudly(cli):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = _run(cli, "-p", os.path.join(G, "pmL6.gset"), "-s", "1", "-r", "4", "--pts", "10")
    assert r.returncode != 0
    assert "no CUDA device" in r.stdout + r.stderr
