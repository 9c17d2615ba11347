"""The code-file boundary (--in / --out) on the host: covsearch2e's reader,
verify_cov's strict reader, and the M-distinct writer, against the oracle's
restatement of the reference writer and the golden --out files."""
import os
import tempfile

import numpy as np
import pytest

from coldcase_gb300 import codefile
from oracle import pyoracle as po


def write(tmp, text):
    p = os.path.join(tmp, "c.txt")
    with open(p, "w") as f:
        f.write(text)
    return p


def test_read_base36_comments_and_noise():
    with tempfile.TemporaryDirectory() as td:
        # a line with a space, comma or tab is integers (atoi); else base-36
        # digits with anything else skipped (covsearch2e.c:870-898)
        p = write(td, "# header\n0a3\n\n1 2 3\nz-0.b# trailing\n7,12x,3\n")
        c = codefile.read_code(p, 3)
        assert c.tolist() == [[0, 10, 3], [1, 2, 3], [35, 0, 11], [7, 12, 3]]
        assert codefile.count_code(p) == 4


def test_read_rejects_wrong_length():
    with tempfile.TemporaryDirectory() as td:
        p = write(td, "012\n01\n")
        with pytest.raises(codefile.CodeFileError):
            codefile.read_code(p, 3)


def test_distinct_code_matches_oracle_writer():
    rng = np.random.default_rng(4)
    for q, n, M in [(4, 6, 420), (3, 4, 60), (2, 5, 32), (5, 3, 40), (6, 2, 10)]:
        code = rng.integers(0, q, (M, n), dtype=np.uint8)
        code[3] = code[0]
        got = codefile.distinct_code(code, q, n, M)
        assert got.shape == (min(M, q ** n), n)
        assert len({tuple(r) for r in got.tolist()}) == len(got)
        assert (got == po.distinct_code(code, q, n, M)).all()


def test_write_is_atomic_and_round_trips(golden):
    runs, _ = golden
    r = [x for x in runs if x["code"]][0]
    q, n, M = r["q"], r["n"], r["M"]
    with tempfile.TemporaryDirectory() as td:
        src = write(td, r["code"])
        code = codefile.read_code(src, n)
        out = os.path.join(td, "out.txt")
        codefile.write_code(out, code, q, n, M)
        assert not os.path.exists(out + ".part")
        back = codefile.read_code(out, n)
        assert (back == codefile.distinct_code(code, q, n, M)).all()
        assert open(out).read() == codefile.format_code(codefile.distinct_code(code, q, n, M), q)


def test_golden_out_files_parse_strictly(golden):
    runs, _ = golden
    for r in runs[:20]:
        with tempfile.TemporaryDirectory() as td:
            p = write(td, r["ref"]["out"])
            words, dups = codefile.parse_code(p, r["q"], r["n"])
            assert dups == 0 and len(words) == codefile.count_code(p)
