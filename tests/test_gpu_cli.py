"""The pt_icm command line (src/main.cc) on the GPU engine: the reference's
flags, the reference's report keys, internally consistent values."""
import os
import re
import subprocess

import pytest

from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "pt-icm_gb300", "bin", "pt_icm")
G = os.path.join(ROOT, "tests", "golden", "graphs")


def _run(*args):
    out = subprocess.run([CLI, *args], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    return out.stdout


def _parse(text):
    rep = {}
    for line in text.splitlines():
        m = re.match(r"^(\w+): (.*)$", line.strip())
        if m:
            rep[m.group(1)] = m.group(2).strip()
    return rep


@pytest.mark.parametrize("flag", ["-p", "-g"])
def test_cli_report(flag):
    path = os.path.join(G, "pmL10.gset")
    text = _run(flag, path, "-s", "3", "-r", "8", "--pts", "500", "--icm", "-T0", "0.5", "-T1", "3.0")
    assert re.search(r"^Total time: [0-9.]+$", text, re.M)
    rep = _parse(text)
    for key in ("swap_rates", "swap_attempts", "swap_successes", "best_state_energy", "best_state_sweep",
                "best_energy", "best_maxcut", "num_of_flips", "num_of_swaps", "best_state"):
        assert key in rep, key
    att = [int(x) for x in rep["swap_attempts"][1:-1].split(",")]
    suc = [int(x) for x in rep["swap_successes"][1:-1].split(",")]
    assert len(att) == 16 and sum(suc) == int(rep["num_of_swaps"])
    assert float(rep["best_state_energy"]) == float(rep["best_energy"])
    # the ground state of this +-J lattice, as the reference finds it
    best_ref = min(O.solve(O.Problem.load(path, s), seed=s, Nt=8, pts=400, icm=True, T0=0.5, T1=3.0)["best_energy"]
                   for s in (1, 2))
    assert float(rep["best_energy"]) == best_ref


def test_cli_preprocess_ladder():
    path = os.path.join(G, "pmL10.gset")
    text = _run("-p", path, "-s", "4", "-r", "10", "--pts", "200", "--preprocess", "--preprocess-samples", "500")
    lines = [l for l in text.splitlines() if l.startswith("[")]
    ladder = [float(x) for x in lines[-1][1:-1].split(",")]
    assert ladder[0] == pytest.approx(1 / 0.6, rel=1e-6)
    assert all(a > b for a, b in zip(ladder, ladder[1:]))


def test_cli_log_prints_observables():
    """--log: the T,C,X,u,m table of the reference's legacy logging, one row per
    temperature, from the steps after the burn-in."""
    path = os.path.join(G, "pmL10.gset")
    text = _run("-p", path, "-s", "2", "-r", "8", "--pts", "3000", "-b", "500", "--icm", "-T0", "0.5", "-T1", "3.0",
                "--log")
    lines = text.splitlines()
    i = lines.index("T,C,X,u,m")
    rows = [[float(x) for x in l.split(",")] for l in lines[i + 1:i + 9]]
    assert len(rows) == 8
    for T, C, X, u, m in rows:
        assert 0.5 - 1e-9 <= T <= 3.0 + 1e-9
        assert C >= 0 and X >= 0 and -2.0 <= u <= 0.0 and abs(m) <= 1.0


def test_cli_checkpoint_resume(tmp_path):
    """--checkpoint after k steps, --resume for k more equals one 2k-step run."""
    path = os.path.join(G, "pmL10.gset")
    common = ["-p", path, "-s", "9", "-r", "8", "--icm", "-T0", "0.5", "-T1", "3.0"]
    ck = str(tmp_path / "half.ckpt")
    _run(*common, "--pts", "150", "--checkpoint", ck)
    resumed = _parse(_run(*common, "--pts", "150", "--resume", ck))
    whole = _parse(_run(*common, "--pts", "300"))
    for key in ("swap_attempts", "swap_successes", "best_energy", "best_state_sweep", "num_of_flips",
                "num_of_swaps", "best_state"):
        assert resumed[key] == whole[key], key


def test_cli_folder_csv(tmp_path):
    """The folder mode: one CSV row per (problem, restart) with the
    reference's columns; each row's energy and cut are those of its state."""
    import csv
    import shutil
    d = tmp_path / "problems"
    d.mkdir()
    names = ["pmL6.gset", "pmL10.gset", "rnd60_pm"]
    for name in names:
        shutil.copy(os.path.join(G, name), d / name)
    out = tmp_path / "runs.csv"
    _run("--folder", str(d), "--csv", str(out), "--restarts", "2", "-s", "5", "-r", "8", "--pts", "300", "--icm",
         "-T0", "0.5", "-T1", "3.0")
    with open(out) as f:
        rows = list(csv.DictReader(f))
    assert list(rows[0].keys()) == ["problem", "iter", "pts", "replicas", "tlist", "pswap", "icm", "preprocess",
                                    "burn_in", "inverse", "sweeps", "ene", "state", "cut", "flips"]
    assert len(rows) == len(names) * 2
    assert [os.path.basename(r["problem"]) for r in rows] == [n for n in sorted(names) for _ in range(2)]
    assert [int(r["iter"]) for r in rows] == [0, 1] * len(names)
    for r in rows:
        assert int(r["pts"]) == 300 and int(r["replicas"]) == 8 and r["icm"] == "1"
        tlist = [float(x) for x in r["tlist"][1:-1].split(";")]
        pswap = [float(x) for x in r["pswap"][1:-1].split(";")]
        assert len(tlist) == 16 and len(pswap) == 16 and all(0.0 <= p <= 1.0 for p in pswap)
        assert tlist[0] == pytest.approx(1 / 3.0, rel=1e-5) and tlist[7] == pytest.approx(2.0, rel=1e-5)
        prob = O.Problem.load(r["problem"], 0)
        state = [int(c) for c in r["state"]]
        assert len(state) == prob.n
        assert float(r["ene"]) == pytest.approx(prob.energy(state), abs=1e-9)
        assert float(r["cut"]) == pytest.approx(prob.maxcut(state), abs=1e-9)
        assert int(r["flips"]) > 0


def test_cli_folder_preprocess_groups_by_ladder_length(tmp_path):
    """With --preprocess every problem gets its own multihistogram ladder;
    runs with ladders of different lengths go to different batches, and each
    row reports its own ladder."""
    import csv
    import shutil
    d = tmp_path / "problems"
    d.mkdir()
    names = ["pmL6.gset", "pmL10.gset", "rnd200_w1"]
    for name in names:
        shutil.copy(os.path.join(G, name), d / name)
    out = tmp_path / "runs.csv"
    _run("--folder", str(d), "--csv", str(out), "-s", "2", "-r", "12", "--pts", "200", "--icm",
         "--preprocess", "--preprocess-samples", "300", "--sort-ladder")
    with open(out) as f:
        rows = list(csv.DictReader(f))
    assert len(rows) == len(names)
    for r in rows:
        nt = int(r["replicas"])
        tlist = [float(x) for x in r["tlist"][1:-1].split(";")]
        assert 2 <= nt <= 12 and len(tlist) == 2 * nt
        assert all(a <= b for a, b in zip(tlist[:nt], tlist[1:nt]))   # sorted ascending
        prob = O.Problem.load(r["problem"], 0)
        state = [int(c) for c in r["state"]]
        assert float(r["ene"]) == pytest.approx(prob.energy(state), abs=1e-9)
