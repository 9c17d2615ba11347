"""The covsearch2e-compatible command line: argument handling on the host
(no GPU), and on the GPU the RESULT fingerprint, the --out file and the exit
status against the reference binary's golden runs."""
import os
import re
import subprocess
import sys
import tempfile

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(REPO, "coldcase_gb300", "bin", "covsearch_gpu")


def run_cli(args, timeout=300):
    return subprocess.run([sys.executable, CLI] + [str(a) for a in args], capture_output=True, text=True,
                          timeout=timeout, cwd=REPO)


@pytest.mark.parametrize("flag", ["--ucache", "--upick"])
def test_trajectory_switches_refused(flag):
    r = run_cli(["-q", "4", "-n", "6", "-R", "1", "-M", "420", flag])
    assert r.returncode == 2 and "trajectory" in r.stderr


def test_bad_arguments_exit_2():
    assert run_cli(["-q", "4", "-n", "6"]).returncode == 2                    # missing -R -M
    assert run_cli(["-q", "4", "-n", "6", "-R", "1", "-M", "420", "--bogus"]).returncode == 2
    assert run_cli(["-q", "4", "-n", "6", "-R", "1", "-M", "420", "--preset", "p9"]).returncode == 2
    assert run_cli(["-q", "4", "-n", "6", "-R", "1", "-M", "70000"]).returncode == 2


@pytest.mark.gpu
def test_cli_matches_reference_runs(covlib, golden):
    runs, _ = golden
    picked = [r for r in runs if r["code"] and not r["random_init"]][:6]
    picked += [r for r in runs if r["code"] and r.get("wide")]
    for r in picked:
        with tempfile.TemporaryDirectory() as td:
            inp, out = os.path.join(td, "in.txt"), os.path.join(td, "out.txt")
            with open(inp, "w") as f:
                f.write(r["code"])
            args = ["-q", r["q"], "-n", r["n"], "-R", r["R"], "-M", r["M"], "-s", r["seed"], "--iters", r["iters"],
                    "--tabu", r["tabu"], "--kick", r["kick"], "--stall", r["stall"], "--in", inp, "--out", out,
                    "--preset", "p5b", "--quiet"] + (["--wide"] if r.get("wide") else [])
            p = run_cli(args)
            m = re.search(r"RESULT .*uncovered=(\d+) iters=(\d+) kicks=(\d+)", p.stdout)
            assert m, p.stdout + p.stderr
            ref = r["ref"]
            assert (int(m.group(1)), int(m.group(2)), int(m.group(3))) == \
                (ref["uncovered"], ref["iters"], ref["kicks"]), (r["q"], r["n"], r["R"], r["M"], r["seed"])
            assert p.returncode == (0 if ref["uncovered"] == 0 else 1)
            with open(out) as f:
                assert f.read() == ref["out"]


SYM_CLI = os.path.join(REPO, "coldcase_gb300", "bin", "symsearch_gpu")


def run_sym_cli(args, timeout=300):
    return subprocess.run([sys.executable, SYM_CLI] + [str(a) for a in args], capture_output=True, text=True,
                          timeout=timeout, cwd=REPO)


def test_sym_cli_argument_errors():
    """symsearch.c:311-333: usage errors exit 2, impossible orbit counts,
    quotients or M exit 3."""
    assert run_sym_cli(["-q", "4", "-n", "6"]).returncode == 2                     # missing -R -M
    assert run_sym_cli(["-q", "4", "-n", "6", "-R", "8", "-M", "40"]).returncode == 2  # R > 7
    assert run_sym_cli(["-q", "4", "-n", "6", "-R", "1", "-M", "3"]).returncode == 2   # M < q
    assert run_sym_cli(["-q", "4", "-n", "6", "-R", "1", "-M", "40", "--bogus"]).returncode == 2
    assert run_sym_cli(["-q", "4", "-n", "6", "-R", "1", "-M", "40", "--orbits", "11"]).returncode == 3
    assert run_sym_cli(["-q", "2", "-n", "6", "-R", "1", "-M", "65536"]).returncode == 3


@pytest.mark.gpu
def test_sym_cli_matches_reference_runs(covlib, sym_golden):
    for r in [x for x in sym_golden if x["seed"] == 3][:8]:
        with tempfile.TemporaryDirectory() as td:
            out = os.path.join(td, "out.txt")
            args = ["-q", r["q"], "-n", r["n"], "-R", r["R"], "-M", r["M"], "-s", r["seed"], "--kick", r["kick"],
                    "--stall", r["stall"], "--iters", r["ref"]["iters"], "-t", 120, "--out", out, "--threads", 1]
            if r["orbits"]:
                args += ["--orbits", r["orbits"]]
            p = run_sym_cli(args)
            m = re.search(r"SYMRESULT .*orbits=(\d+) red_uncovered=(\d+) word_uncovered=(\d+) iters=(\d+) "
                          r"kicks=(\d+)", p.stdout)
            assert m, p.stdout + p.stderr
            ref = r["ref"]
            assert (int(m.group(1)), int(m.group(2)), int(m.group(4)), int(m.group(5))) == \
                (ref["orbits"], ref["red_uncovered"], ref["iters"], ref["kicks"]), (r["q"], r["n"], r["R"], r["M"])
            assert p.returncode == ref["rc"]
            with open(out) as f:
                assert f.read() == ref["out"]


def test_fix0_arguments_through_the_protocol():
    """--fix0 reaches the engine with the other flags, and the RESULT line,
    exit status and --out file equal the reference binary's; the oracle
    stands in for the GPU engine (tests/portfolio_stub.py)."""
    import json
    stub = os.path.join(REPO, "tests", "portfolio_stub.py")
    with open(os.path.join(REPO, "tests", "golden", "opt_runs.json")) as f:
        runs = [r for r in json.load(f) if r.get("fix0") and not r["code"]][:2]
    assert runs
    for r in runs:
        with tempfile.TemporaryDirectory() as td:
            out = os.path.join(td, "out.txt")
            p = subprocess.run([sys.executable, stub] + [str(a) for a in [
                "-q", r["q"], "-n", r["n"], "-R", r["R"], "-M", r["M"], "-s", r["seed"], "--iters", r["iters"],
                "--tabu", r["tabu"], "--kick", r["kick"], "--stall", r["stall"], "--out", out, "--fix0",
                "--quiet"]], capture_output=True, text=True, timeout=300, cwd=REPO)
            m = re.search(r"RESULT .*uncovered=(\d+) iters=(\d+) kicks=(\d+)", p.stdout)
            assert m, p.stdout + p.stderr
            ref = r["ref"]
            assert (int(m.group(1)), int(m.group(2)), int(m.group(3))) == (ref["uncovered"], ref["iters"], ref["kicks"])
            assert p.returncode == ref["rc"]
            with open(out) as f:
                assert f.read() == ref["out"]


def test_method_flags_through_the_protocol():
    """--sa --t0 --cool --tmin and --noise reach the engine with the other
    flags; RESULT line, exit status and --out file equal the reference
    binary's (the oracle stands in for the GPU engine,
    tests/portfolio_stub.py)."""
    import json
    stub = os.path.join(REPO, "tests", "portfolio_stub.py")
    with open(os.path.join(REPO, "tests", "golden", "method_runs.json")) as f:
        runs = json.load(f)
    picked = [r for r in runs if r["sa"] and r["ref"]["iters"] > 100][:2] + \
        [r for r in runs if r["noise"] and r["ref"]["iters"] > 100][:2]
    for r in picked:
        with tempfile.TemporaryDirectory() as td:
            out = os.path.join(td, "out.txt")
            args = ["-q", r["q"], "-n", r["n"], "-R", r["R"], "-M", r["M"], "-s", r["seed"], "--iters", r["iters"],
                    "--tabu", r["tabu"], "--kick", r["kick"], "--stall", r["stall"], "--out", out, "--quiet"]
            args += ["--wide"] if r["wide"] else []
            args += ["--fix0"] if r["fix0"] else []
            if r["sa"]:
                args += ["--sa", "--t0", repr(r["sa"][0]), "--cool", repr(r["sa"][1]), "--tmin", repr(r["sa"][2])]
            if r["noise"]:
                args += ["--noise", r["noise"]]
            p = subprocess.run([sys.executable, stub] + [str(a) for a in args], capture_output=True, text=True,
                               timeout=300, cwd=REPO)
            m = re.search(r"RESULT .*uncovered=(\d+) iters=(\d+) kicks=(\d+)", p.stdout)
            assert m, p.stdout + p.stderr
            ref = r["ref"]
            assert (int(m.group(1)), int(m.group(2)), int(m.group(3))) == (ref["uncovered"], ref["iters"], ref["kicks"])
            assert p.returncode == ref["rc"]
            with open(out) as f:
                assert f.read() == ref["out"]


def test_gpu_only_flags_parse():
    from coldcase_gb300 import covsearch_gpu as cg
    a, rc = cg.parse(["-q", "7", "-n", "9", "-R", "4", "-M", "1500", "--grid-help", "64", "--sa", "--t0", "1.5",
                      "--cool", "0.99", "--tmin", "0.1", "--noise", "20", "--cluster", "16"])
    assert rc == 0 and a["grid_help"] == 64 and a["sa"] and (a["t0"], a["cool"], a["tmin"]) == (1.5, 0.99, 0.1)
    assert a["noise"] == 20 and a["cluster"] == 16
