"""The reference's optimisation-gate configurations (cov/opt/selftest.sh,
tests/golden/opt_runs.json) on the CUDA engine, with and without --wide and
--fix0 (covsearch2e.c:1241-1253: the initial code translated so that
codeword 0 is 0^n, which then is neither a candidate nor kicked).

Bit-exact: fingerprint (best uncovered, iterations, kicks) and --out file
equal the reference binary's; move records, RNG state, tabu table, code and
coverage counts equal the oracle's.
"""
import os
import re
import tempfile

import pytest

from coldcase_gb300 import codefile
from coldcase_gb300.engine import Pool
from tests.test_cli import run_cli
from tests.util import code_from_text, oracle_run

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def opt_runs():
    import json
    with open(os.path.join(HERE, "golden", "opt_runs.json")) as f:
        return json.load(f)


def first_diff(a, b):
    for k in range(min(len(a), len(b))):
        if a[k].tobytes() != b[k].tobytes():
            return k
    return min(len(a), len(b))


@pytest.mark.parametrize("cluster", [1, 4])
def test_opt_gate_runs_bit_exact(covlib, opt_runs, cluster):
    bad = []
    assert sum(1 for r in opt_runs if r.get("fix0")) >= 10
    for r in opt_runs:
        pool = Pool(1, cluster=cluster)
        code = code_from_text(r["code"], r["n"]) if r["code"] else None
        s = pool.add(r["q"], r["n"], r["R"], r["M"], code=code, random_init=r["random_init"], seed=r["seed"],
                     tabu=r["tabu"], kick=r["kick"], stall=r["stall"], trace=1, trace_cap=max(1, r["iters"]),
                     wide=r.get("wide", False), fix0=r.get("fix0", False))
        pool.run(r["iters"])
        st = pool.status(s)
        o, otr = oracle_run(r)
        gtr = pool.trace(s)
        ref = r["ref"]
        got = (st["best"], st["it"], st["kicks"])
        want = (ref["uncovered"], ref["iters"], ref["kicks"])
        out = codefile.format_code(codefile.distinct_code(pool.best(s), r["q"], r["n"], r["M"]), r["q"])
        ok = st["status"] == 0 and got == want and out == ref["out"] and gtr.tobytes() == otr.tobytes()
        ok = ok and (pool.rng(s) == o.rng()).all() and (pool.tabu(s) == o.tabu()).all()
        ok = ok and (pool.code(s) == o.code()).all() and (pool.cnt(s) == o.cnt()).all()
        if r.get("fix0"):
            # codeword 0 stays at 0^n for the whole run
            ok = ok and not pool.code(s)[0].any() and not pool.best(s)[0].any()
        if not ok:
            bad.append(dict(cell=(r["q"], r["n"], r["R"], r["M"], r["seed"], r.get("wide"), r.get("fix0")),
                            status=st["status"], got=got, want=want, out_ok=out == ref["out"],
                            ntr=(len(gtr), len(otr)), first=first_diff(gtr, otr)))
        o.close()
        pool.close()
    assert not bad, bad[:3]


def test_fix0_cli_matches_reference(covlib, opt_runs):
    """covsearch_gpu --fix0: RESULT line, exit status and --out file equal
    the reference binary's."""
    picked = [r for r in opt_runs if r.get("fix0")][:4]
    for r in picked:
        with tempfile.TemporaryDirectory() as td:
            out = os.path.join(td, "out.txt")
            args = ["-q", r["q"], "-n", r["n"], "-R", r["R"], "-M", r["M"], "-s", r["seed"], "--iters", r["iters"],
                    "--tabu", r["tabu"], "--kick", r["kick"], "--stall", r["stall"], "--out", out, "--fix0",
                    "--preset", "p5b", "--quiet"]
            p = run_cli(args)
            m = re.search(r"RESULT .*uncovered=(\d+) iters=(\d+) kicks=(\d+)", p.stdout)
            assert m, p.stdout + p.stderr
            ref = r["ref"]
            assert (int(m.group(1)), int(m.group(2)), int(m.group(3))) == \
                (ref["uncovered"], ref["iters"], ref["kicks"]), (r["q"], r["n"], r["R"], r["M"], r["seed"])
            assert p.returncode == ref["rc"]
            with open(out) as f:
                assert f.read() == ref["out"]
    # M < 2 leaves nothing to search once codeword 0 is fixed: refused
    assert run_cli(["-q", "3", "-n", "4", "-R", "1", "-M", "1", "--fix0", "--quiet"]).returncode == 2


@pytest.fixture(scope="module")
def method_runs():
    import json
    with open(os.path.join(HERE, "golden", "method_runs.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("cluster", [1, 4])
def test_method_runs_bit_exact(covlib, method_runs, cluster):
    """--sa (focused simulated annealing: one proposal, its exact delta, the
    Metropolis test, the cooling schedule and stall reheats) and --noise
    (unevaluated moves): fingerprint and --out file equal the reference
    binary's, move records and state equal the oracle's."""
    bad = []
    for r in method_runs:
        pool = Pool(1, cluster=cluster)
        code = code_from_text(r["code"], r["n"]) if r["code"] else None
        s = pool.add(r["q"], r["n"], r["R"], r["M"], code=code, random_init=r["random_init"], seed=r["seed"],
                     tabu=r["tabu"], kick=r["kick"], stall=r["stall"], trace=1, trace_cap=max(1, r["iters"]),
                     wide=r["wide"], fix0=r["fix0"], sa=tuple(r["sa"]) if r["sa"] else None, noise=r["noise"])
        pool.run(r["iters"])
        st = pool.status(s)
        o, otr = oracle_run(r)
        gtr = pool.trace(s)
        ref = r["ref"]
        got = (st["best"], st["it"], st["kicks"])
        want = (ref["uncovered"], ref["iters"], ref["kicks"])
        out = codefile.format_code(codefile.distinct_code(pool.best(s), r["q"], r["n"], r["M"]), r["q"])
        ok = st["status"] == 0 and got == want and out == ref["out"] and gtr.tobytes() == otr.tobytes()
        ok = ok and (pool.rng(s) == o.rng()).all() and (pool.tabu(s) == o.tabu()).all()
        ok = ok and (pool.code(s) == o.code()).all() and (pool.cnt(s) == o.cnt()).all()
        if not ok:
            bad.append(dict(cell=(r["q"], r["n"], r["R"], r["M"], r["seed"], r["sa"], r["noise"]),
                            status=st["status"], got=got, want=want, out_ok=out == ref["out"],
                            ntr=(len(gtr), len(otr)), first=first_diff(gtr, otr)))
        o.close()
        pool.close()
    assert not bad, bad[:3]


def test_method_cli_matches_reference(covlib, method_runs):
    """covsearch_gpu --sa --t0 --cool --tmin and --noise: RESULT line, exit
    status and --out file equal the reference binary's."""
    picked = [r for r in method_runs if r["sa"] and r["ref"]["iters"] > 100][:2]
    picked += [r for r in method_runs if r["noise"] and r["ref"]["iters"] > 100][:2]
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
            p = run_cli(args)
            m = re.search(r"RESULT .*uncovered=(\d+) iters=(\d+) kicks=(\d+)", p.stdout)
            assert m, p.stdout + p.stderr
            ref = r["ref"]
            assert (int(m.group(1)), int(m.group(2)), int(m.group(3))) == \
                (ref["uncovered"], ref["iters"], ref["kicks"]), (r["q"], r["n"], r["R"], r["M"], r["seed"])
            assert p.returncode == ref["rc"]
            with open(out) as f:
                assert f.read() == ref["out"]
