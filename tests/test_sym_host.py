"""Quotient search, host side (no GPU): the orbit expansion and the
quotient's uncovered count against a direct count of the whole code."""
import numpy as np

from coldcase_gb300.sym import expand, format_code
from oracle import pyoracle as po
from tests.util import code_from_text, sym_oracle_run


def test_expanded_code_has_q_times_the_quotient_uncovered(sym_golden):
    """An invariant code's uncovered words are q per uncovered quotient word
    (symsearch.c:15-31): expand the best orbits of the reference runs and
    count the whole space directly."""
    checked = 0
    for r in sym_golden:
        q, n, R = r["q"], r["n"], r["R"]
        if q ** n > 300000:
            continue
        code = code_from_text(r["ref"]["out"], n)
        reps = code[::q, 1:]
        assert (expand(reps, q) == code).all()
        assert format_code(reps, q) == r["ref"]["out"]
        assert po.verify_pure(code, q, n, R) == q * r["ref"]["red_uncovered"], (q, n, R, r["M"])
        checked += 1
    assert checked >= 20


def test_oracle_counters_match_a_direct_count(sym_golden):
    """The oracle's quotient counters equal the multiplicity of the expanded
    code restricted to words with first digit 0."""
    for r in [x for x in sym_golden if x["q"] ** x["n"] <= 100000][:10]:
        o, _ = sym_oracle_run(r, moves=50)
        q, n, R = r["q"], r["n"], r["R"]
        full = po.cover_count(expand(o.rep(), q), q, n, R)
        assert (full[: q ** (n - 1)] == o.cnt()).all(), (q, n, R, r["M"])
