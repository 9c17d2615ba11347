"""The oracle against the reference's own outputs (tests/golden/, generated
by make_golden.py from the reference engine binary and verifiers)."""
import numpy as np
import pytest

from oracle import pyoracle as po
from coldcase_gb300 import codefile
from tests.util import code_from_text, oracle_run


def test_engine_runs_match_reference(golden):
    runs, _ = golden
    bad = []
    for r in runs:
        o, tr = oracle_run(r)
        ref = r["ref"]
        got = (o.best_uncovered(), o.iters(), o.kicks())
        want = (ref["uncovered"], ref["iters"], ref["kicks"])
        out = codefile.format_code(codefile.distinct_code(o.best(), r["q"], r["n"], r["M"]), r["q"])
        if got != want or out != ref["out"]:
            bad.append((r["q"], r["n"], r["R"], r["M"], r["seed"], got, want, out == ref["out"]))
    assert not bad, bad


def test_trace_invariants(golden):
    runs, _ = golden
    for r in runs[:30]:
        o, tr = oracle_run(r)
        if len(tr) == 0:
            continue
        assert (np.diff(tr["it"]) == 1).all()
        # every committed delta is what the commit changed
        prev = np.concatenate([[None], tr["unc_end"][:-1]])
        for k in range(1, len(tr)):
            assert tr["unc"][k] - tr["unc_end"][k - 1] == tr["delta"][k]
        assert (tr["best"][1:] <= tr["best"][:-1]).all()


def test_threads_do_not_change_trajectory(golden):
    runs, _ = golden
    for r in [x for x in runs if x["q"] ** x["n"] > 40000][:4]:
        _, t1 = oracle_run(r, threads=1)
        _, t4 = oracle_run(r, threads=4)
        assert t1.tobytes() == t4.tobytes()


def test_verify_cases(golden):
    _, cases = golden
    for c in cases:
        code = np.array(c["code"], dtype=np.uint8)
        q, n, R = c["q"], c["n"], c["R"]
        assert po.verify_pure(code, q, n, R) == c["uncovered"], c["src"]
        if q ** n <= 2_000_000 and c["hist"] is not None:
            d = po.mindist(code, q, n, threads=4)
            hist = np.bincount(d, minlength=n + 2)[: n + 2]
            assert hist.tolist() == c["hist"], c["src"]
            assert int(d.max()) == c["radius"]
            # the line-min form (the CPU baseline of the transform) gives the
            # same per-word distances as the direct minimum
            assert (po.linemin(code, q, n, threads=4) == d).all(), c["src"]
            ok, cov = po.dilate(code, q, n, R)
            assert ok == c["covers"] and int((~cov).sum()) == c["uncovered"]
            cnt = po.cover_count(code, q, n, R)
            assert int((cnt == 0).sum()) == c["uncovered"]


def test_distinct_code_matches_writer():
    rng = np.random.default_rng(3)
    for (q, n, M) in [(3, 4, 9), (4, 6, 420), (2, 3, 8), (6, 5, 40)]:
        code = rng.integers(0, q, (M, n), dtype=np.uint8)
        code[M // 2] = code[0]
        a = po.distinct_code(code, q, n, M)
        b = codefile.distinct_code(code, q, n, M)
        assert a.tobytes() == b.tobytes()
        assert len({tuple(x) for x in b.tolist()}) == len(b) == min(M, q ** n)


def test_sym_runs_match_reference(sym_golden):
    """The quotient-search restatement against the reference binary: each
    run replayed for the iterations the reference reached."""
    from tests.util import sym_oracle_run, sym_text
    bad = []
    for r in sym_golden:
        o, tr = sym_oracle_run(r)
        ref = r["ref"]
        got = (o.orbits, o.best_uncovered(), o.iters(), o.kicks())
        want = (ref["orbits"], ref["red_uncovered"], ref["iters"], ref["kicks"])
        if got != want or sym_text(o.best(), r["q"]) != ref["out"] or (ref["rc"] == 0) != (got[1] == 0):
            bad.append((r["q"], r["n"], r["R"], r["M"], r["seed"], got, want))
    assert not bad, bad


def test_sym_threads_do_not_change_trajectory(sym_golden):
    from oracle.pyoracle import SymOracle
    for r in [x for x in sym_golden if x["q"] ** (x["n"] - 1) > 20000][:3]:
        traces = []
        for th in (1, 4):
            o = SymOracle(r["q"], r["n"], r["R"], r["M"], orbits=r["orbits"], seed=r["seed"], kick=r["kick"],
                          stall=r["stall"], threads=th)
            o.init()
            traces.append(o.run(min(300, r["ref"]["iters"]), trace=True))
        assert traces[0].tobytes() == traces[1].tobytes()


def test_opt_gate_runs_match_reference():
    """The configurations of the reference's optimisation gate
    (cov/opt/selftest.sh): the oracle's fingerprint and --out file equal the
    reference engine's, with and without --wide, and the written file's
    count from the verifier equals the reported one."""
    import json
    import os
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    with open(os.path.join(here, "opt_runs.json")) as f:
        runs = json.load(f)
    bad = []
    for r in runs:
        o, _ = oracle_run(r)
        ref = r["ref"]
        got = (o.best_uncovered(), o.iters(), o.kicks())
        want = (ref["uncovered"], ref["iters"], ref["kicks"])
        out = codefile.format_code(codefile.distinct_code(o.best(), r["q"], r["n"], r["M"]), r["q"])
        words = code_from_text(ref["out"], r["n"])
        if got != want or out != ref["out"] or po.verify_pure(words, r["q"], r["n"], r["R"]) != ref["uncovered"]:
            bad.append((r["q"], r["n"], r["R"], r["M"], r["seed"], r["wide"], got, want))
    assert not bad, bad


def test_method_runs_match_reference():
    """--sa (focused simulated annealing at three cooling schedules) and
    --noise (two rates, with tabu, kicks, --wide and --fix0): the oracle's
    fingerprint and --out file equal the reference engine's
    (tests/golden/method_runs.json, made by tests/golden/make_golden.py)."""
    import json
    import os
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    with open(os.path.join(here, "method_runs.json")) as f:
        runs = json.load(f)
    assert sum(1 for r in runs if r["sa"]) >= 20 and sum(1 for r in runs if r["noise"]) >= 10
    bad = []
    for r in runs:
        o, _ = oracle_run(r)
        ref = r["ref"]
        got = (o.best_uncovered(), o.iters(), o.kicks())
        want = (ref["uncovered"], ref["iters"], ref["kicks"])
        out = codefile.format_code(codefile.distinct_code(o.best(), r["q"], r["n"], r["M"]), r["q"])
        if got != want or out != ref["out"]:
            bad.append((r["q"], r["n"], r["R"], r["M"], r["seed"], r["sa"], r["noise"], got, want, out == ref["out"]))
        o.close()
    assert not bad, bad


def test_pick_runs_match_reference():
    """The experimental pick rules --upick and --ucache (alone and together,
    with tabu and kicks): the oracle's fingerprint and --out file equal the
    reference engine's (tests/golden/pick_runs.json).  The GPU engine
    refuses these flags; the oracle restates them."""
    import json
    import os
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    with open(os.path.join(here, "pick_runs.json")) as f:
        runs = json.load(f)
    bad = []
    for r in runs:
        o, _ = oracle_run(r)
        ref = r["ref"]
        got = (o.best_uncovered(), o.iters(), o.kicks())
        want = (ref["uncovered"], ref["iters"], ref["kicks"])
        out = codefile.format_code(codefile.distinct_code(o.best(), r["q"], r["n"], r["M"]), r["q"])
        if got != want or out != ref["out"]:
            bad.append((r["q"], r["n"], r["R"], r["M"], r["seed"], r["upick"], r["ucache"], got, want))
        o.close()
    assert not bad, bad
