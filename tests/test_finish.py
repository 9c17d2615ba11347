"""The finisher (covcount: de-duplicate, top up to M distinct words, recount)
against the reference binary's outputs (tests/golden/finish_cases.json):
the oracle's restatement on the CPU, the GPU finisher and its command line
on the GPU."""
import json
import os
import re
import subprocess
import sys
import tempfile

import pytest

from oracle import pyoracle as po

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
DIG = "0123456789abcdefghijklmnopqrstuvwxyz"


@pytest.fixture(scope="module")
def cases():
    with open(os.path.join(HERE, "golden", "finish_cases.json")) as f:
        return json.load(f)


def text_of(words):
    return "".join("".join(DIG[v] for v in w) + "\n" for w in words)


def test_oracle_finisher_matches_reference(cases):
    for c in cases:
        words, unc, rc = po.finish(c["input"], c["q"], c["n"], c["R"], c["M"], fast=c["fast"])
        assert (len(words), unc, rc) == (c["words"], c["uncovered"], c["rc"]), (c["q"], c["n"], c["R"], c["M"])
        assert text_of(words) == c["out"]


@pytest.mark.gpu
def test_gpu_finisher_matches_reference(covlib, cases):
    from coldcase_gb300 import codefile, verify
    for c in cases:
        with tempfile.TemporaryDirectory() as td:
            p = os.path.join(td, "in.txt")
            with open(p, "w") as f:
                f.write(c["input"])
            code = codefile.read_code_finisher(p, c["q"], c["n"], c["M"])
        out, unc = verify.finish(code, c["q"], c["n"], c["R"], c["M"], fast=c["fast"])
        assert unc == c["uncovered"], (c["q"], c["n"], c["R"], c["M"], c["fast"])
        assert codefile.format_code(out, c["q"]) == c["out"]


@pytest.mark.gpu
def test_covcount_cli_matches_reference(covlib, cases):
    cli = os.path.join(REPO, "coldcase_gb300", "bin", "covcount_gpu")
    for c in cases[:8]:
        with tempfile.TemporaryDirectory() as td:
            inp, out = os.path.join(td, "in.txt"), os.path.join(td, "out.txt")
            with open(inp, "w") as f:
                f.write(c["input"])
            args = [sys.executable, cli, "-q", str(c["q"]), "-n", str(c["n"]), "-R", str(c["R"]), "-M", str(c["M"]),
                    "--in", inp, "--out", out] + (["--fast"] if c["fast"] else [])
            p = subprocess.run(args, capture_output=True, text=True, timeout=300)
            m = re.search(r"COUNT .*words=(\d+) uncovered=(-?\d+)", p.stdout)
            assert m, p.stdout + p.stderr
            assert (int(m.group(1)), int(m.group(2)), p.returncode) == (c["words"], c["uncovered"], c["rc"])
            assert open(out).read() == c["out"] and not os.path.exists(out + ".part")


def test_covcount_cli_bad_arguments():
    cli = os.path.join(REPO, "coldcase_gb300", "bin", "covcount_gpu")
    for args in (["-q", "4", "-n", "6"], ["-q", "4", "-n", "6", "-R", "1", "-M", "5", "--in", "x", "--bogus"]):
        assert subprocess.run([sys.executable, cli] + args, capture_output=True, timeout=120).returncode == 2
