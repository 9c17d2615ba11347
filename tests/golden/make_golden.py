#!/usr/bin/env python3
"""Generate the golden fixtures of tests/golden/ from the reference itself.

Runs in the build container only (it needs the reference checkout):
  * engine_runs.json   -- the reference engine binary (oracle/_ref/covsearch2e,
                          compiled from cov/engine/covsearch2e.c by
                          `make -C oracle ref`) on a fixed list of runs: the
                          cell list of cov/engine/selftest.sh:27-38 plus runs
                          that exercise --in (exact M, fewer words = greedy
                          top-up, more words = remove-and-repair), --tabu,
                          small --stall (kicks), --random-init and --wide.  Stored:
                          arguments, input code, the RESULT fingerprint
                          uncovered/iters/kicks and the --out file.
  * finish_cases.json  -- the reference finisher (oracle/_ref/covcount,
                          compiled from cov/engine/covcount.c) on code files
                          with duplicates, malformed lines, too few and too
                          many words: COUNT line, exit status and --out file,
                          with and without --fast.
  * method_runs.json   -- the reference engine's other move methods: --sa
                          (simulated annealing, three cooling schedules)
                          and --noise (two per-mille rates, with tabu,
                          kicks, --wide and --fix0): fingerprint and --out.
  * pick_runs.json     -- the reference engine's experimental pick rules
                          --upick and --ucache (alone and together): the
                          oracle's pinning for them (the GPU refuses them).
  * opt_runs.json      -- the reference engine on the configurations of the
                          optimisation gate cov/opt/selftest.sh (p5b, with
                          and without --wide, and --fix0): fingerprint and
                          --out file.
  * sym_runs.json      -- the reference quotient search (oracle/_ref/symsearch,
                          compiled from cov/engine/symsearch.c) on a cell
                          list with plain, short-stall and kick-3 runs and
                          --orbits below M/q: its SYMRESULT fingerprint
                          (iterations reached, best quotient uncovered,
                          kicks), exit status and --out file.
  * verify_cases.json  -- codes with their uncovered counts from the
                          reference verifiers verify_pure and verify_numpy
                          (cov/verify_cov.py) and the distance histogram and
                          covering radius printed by run_mindist
                          (cov/verify_independent.py), including the known-
                          answer cases of cov/test_verify.py (whole space,
                          single word, perfect Hamming codes, direct sums).

Usage: python3 tests/golden/make_golden.py [--ref REFERENCE_CHECKOUT] [--only methods|picks]
(default: $COLDCASE_REF, else /root/reference)
"""
import argparse
import contextlib
import io
import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
DIG = "0123456789abcdefghijklmnopqrstuvwxyz"


def code_text(c):
    return "".join("".join(DIG[int(v)] for v in row) + "\n" for row in c)


def run_ref(binary, args, inp_text):
    with tempfile.TemporaryDirectory() as td:
        cmd = [binary] + [str(a) for a in args] + ["--out", os.path.join(td, "out.txt"), "--quiet",
                                                   "--preset", "p5b"]
        if inp_text is not None:
            with open(os.path.join(td, "in.txt"), "w") as f:
                f.write(inp_text)
            cmd += ["--in", os.path.join(td, "in.txt")]
        p = subprocess.run(cmd, capture_output=True, text=True)
        m = re.search(r"uncovered=(-?\d+) iters=(\d+) kicks=(\d+)", p.stdout)
        if not m:
            raise RuntimeError("no RESULT from %s: %s %s" % (cmd, p.stdout, p.stderr))
        out = open(os.path.join(td, "out.txt")).read()
        return dict(uncovered=int(m.group(1)), iters=int(m.group(2)), kicks=int(m.group(3)),
                    out=out, rc=p.returncode)


def engine_runs(binary):
    runs = []
    cells = [(2, 6, 2, 12, 300), (3, 6, 2, 12, 300), (5, 5, 2, 30, 200), (6, 6, 3, 41, 400),
             (6, 6, 3, 45, 400), (7, 4, 1, 60, 300), (3, 11, 4, 81, 120), (6, 8, 4, 169, 40),
             (4, 5, 0, 1024, 5), (5, 4, 3, 3, 50)]
    for (q, n, R, M, it) in cells:
        for s in (1, 2):
            runs.append(dict(q=q, n=n, R=R, M=M, seed=s, iters=it, tabu=0, stall=5000, kick=2,
                             random_init=False, code=None))
    for (q, n, R, M, it) in cells[:8]:
        runs.append(dict(q=q, n=n, R=R, M=M, seed=3, iters=it, tabu=7, stall=20, kick=2,
                         random_init=False, code=None))
        runs.append(dict(q=q, n=n, R=R, M=M, seed=4, iters=it, tabu=3, stall=10, kick=3,
                         random_init=True, code=None))
    # --in: exact M, fewer (greedy top-up), more (remove-and-repair)
    for (q, n, R, M, m, it) in [(4, 6, 1, 420, 420, 10000), (4, 6, 1, 420, 420, 10000),
                                (6, 6, 3, 41, 41, 400), (5, 5, 2, 30, 20, 200),
                                (3, 4, 1, 9, 12, 2000), (4, 5, 1, 40, 55, 300),
                                (5, 5, 2, 20, 30, 300), (6, 6, 3, 41, 60, 200),
                                (6, 7, 3, 100, 100, 300)]:
        for s in (1, 2):
            code = np.random.default_rng(1000 * q + 10 * n + m + s).integers(0, q, (m, n), dtype=np.uint8)
            runs.append(dict(q=q, n=n, R=R, M=M, seed=s, iters=it, tabu=10, stall=50, kick=2,
                             random_init=False, code=code_text(code)))
    # more than 2^19 uncovered words: the uncovered list is not valid, the
    # entering side is walked and pick_uncovered scans (covsearch2e.c:1327,
    # 735-753, 1004-1015); the second cell crosses into the valid regime
    for (q, n, R, M, it) in [(6, 8, 2, 20, 25), (5, 9, 3, 60, 40), (4, 10, 2, 200, 300)]:
        runs.append(dict(q=q, n=n, R=R, M=M, seed=5, iters=it, tabu=5, stall=5000, kick=2,
                         random_init=True, code=None))
    # the plain CPU configuration: q4 n6 R1 M420, tenure 10, uniform codes
    for s in range(1, 6):
        code = np.random.default_rng(s).integers(0, 4, (420, 6), dtype=np.uint8)
        runs.append(dict(q=4, n=6, R=1, M=420, seed=s, iters=10000, tabu=10, stall=5000, kick=2,
                         random_init=False, code=code_text(code)))
    # --wide: all n(q-1) moves of each candidate codeword while the uncovered
    # list is valid and short (covsearch2e.c:1353-1376); the K_3(11,4) runs
    # cross that threshold in both directions
    for (q, n, R, M, it) in [(6, 6, 3, 41, 400), (3, 11, 4, 81, 400), (6, 8, 4, 169, 60),
                             (6, 6, 3, 45, 400), (5, 6, 2, 60, 300)]:
        for s in (1, 2):
            runs.append(dict(q=q, n=n, R=R, M=M, seed=s, iters=it, tabu=7, stall=50, kick=2,
                             random_init=False, code=None, wide=True))
    for (q, n, R, M, m, it) in [(6, 6, 3, 41, 41, 600), (3, 11, 4, 81, 90, 300)]:
        code = np.random.default_rng(7000 + q + n + m).integers(0, q, (m, n), dtype=np.uint8)
        runs.append(dict(q=q, n=n, R=R, M=M, seed=3, iters=it, tabu=10, stall=40, kick=2,
                         random_init=False, code=code_text(code), wide=True))
    for r in runs:
        args = ["-q", r["q"], "-n", r["n"], "-R", r["R"], "-M", r["M"], "-s", r["seed"],
                "--iters", r["iters"], "--tabu", r["tabu"], "--stall", r["stall"], "--kick", r["kick"]]
        if r["random_init"]:
            args.append("--random-init")
        if r.get("wide"):
            args.append("--wide")
        r["ref"] = run_ref(binary, args, r["code"])
    return runs


def verify_cases(ref):
    sys.path.insert(0, os.path.join(ref, "cov"))
    import verify_cov as V                   # noqa: E402  (the reference verifier)
    import verify_independent as VI          # noqa: E402
    import constructions as C                # noqa: E402

    def mindist_report(code, q, n, R):
        C_ = np.array(code, dtype=np.uint8)
        buf = io.StringIO()
        with contextlib.redirect_stdout(buf), contextlib.redirect_stderr(io.StringIO()):
            ok = VI.run_mindist(C_, q, n, R, q ** n, len(C_), 1 << 20)
        txt = buf.getvalue()
        hist = [0] * (n + 2)
        for d, c in re.findall(r"d=(\d+)\s*:\s*(\d+)", txt):
            hist[int(d)] = int(c)
        rad = int(re.search(r"covering radius \(exact\) = (\d+)", txt).group(1))
        return hist, rad, bool(ok)

    cases = []
    rng = np.random.default_rng(20260818)
    for (q, n) in [(2, 6), (3, 5), (3, 6), (4, 5), (5, 4), (6, 4), (7, 3), (2, 9), (4, 6), (6, 6),
                   (7, 5), (5, 7)]:
        for R in range(0, min(n, 4) + 1):
            M = int(rng.integers(1, 13 if q ** n < 5000 else 60))
            code = [tuple(int(v) for v in row) for row in rng.integers(0, q, (M, n))]
            code = list(dict.fromkeys(code))
            cases.append(dict(q=q, n=n, R=R, code=code, src="random"))
    full = C.full_space(2, 5)
    cases.append(dict(q=2, n=5, R=0, code=full, src="whole space Z_2^5"))
    cases.append(dict(q=2, n=5, R=0, code=full[:-1], src="whole space minus one word"))
    cases.append(dict(q=3, n=5, R=5, code=[tuple([0] * 5)], src="single word at R=n"))
    cases.append(dict(q=3, n=5, R=4, code=[tuple([0] * 5)], src="single word at R=n-1"))
    for q, r in [(2, 3), (3, 2), (4, 2), (5, 2)]:
        H = C.hamming_code(q, r)
        nn = (q ** r - 1) // (q - 1)
        cases.append(dict(q=q, n=nn, R=1, code=H, src="Hamming q=%d r=%d" % (q, r)))
        cases.append(dict(q=q, n=nn, R=1, code=H[:-1], src="Hamming q=%d r=%d minus one" % (q, r)))
    cases.append(dict(q=3, n=6, R=1, code=C.direct_sum(C.hamming_code(3, 2), C.full_space(3, 2)),
                      src="direct sum (4,1)+(2,0)"))
    cases.append(dict(q=3, n=6, R=3, code=C.direct_sum(C.hamming_code(3, 2), [tuple([0, 0])]),
                      src="direct sum (4,1)+(2,2)"))
    out = []
    for c in cases:
        q, n, R, code = c["q"], c["n"], c["R"], [tuple(int(v) for v in w) for w in c["code"]]
        pure = V.verify_pure(code, n, q, R, want_witness=False)[0]
        nump = V.verify_numpy(code, n, q, R, want_witness=False)[0]
        hist, rad, ok = mindist_report(code, q, n, R)
        assert pure == nump, c["src"]
        out.append(dict(q=q, n=n, R=R, src=c["src"], code=[list(w) for w in code], uncovered=pure,
                        hist=hist, radius=rad, covers=ok))
    # a recorded cover from the reference's results, verified by both methods there
    rec = os.path.join(ref, "cov", "results", "K6_9_4_M660.txt")
    if os.path.exists(rec):
        code, _ = V.parse_code(rec, 6, 9)
        out.append(dict(q=6, n=9, R=4, src="cov/results/K6_9_4_M660.txt", code=[list(w) for w in code],
                        uncovered=V.verify_numpy(code, 9, 6, 4, want_witness=False)[0],
                        hist=None, radius=None, covers=True))
    return out


def finish_cases(binary):
    """The reference finisher (cov/engine/covcount.c, compiled into
    oracle/_ref/covcount) on code files with duplicates, malformed lines,
    too few and too many words, with and without --fast."""
    rng = np.random.default_rng(20261203)
    cases = []
    specs = [(4, 6, 1, 420, 400, 0), (3, 5, 2, 20, 30, 1), (5, 4, 1, 60, 40, 2), (2, 8, 2, 30, 10, 3),
             (6, 6, 3, 25, 25, 4), (7, 5, 2, 80, 70, 5), (4, 6, 2, 120, 0, 6), (3, 4, 1, 81, 90, 7),
             (6, 9, 4, 700, 690, 8), (2, 6, 5, 3, 2, 9)]
    for q, n, R, M, m, seed in specs:
        code = rng.integers(0, q, (m, n), dtype=np.uint8)
        if m > 4:
            code[m // 2] = code[1]
            code[m - 1] = code[0]
        text = code_text(code)
        if m > 3:
            lines = text.splitlines(True)
            lines.insert(2, "# a comment\n")
            lines.insert(3, DIG[q % 36] * n + "\n")      # a digit out of range: skipped
            lines.insert(4, "0" * (n + 1) + "\n")         # wrong length: skipped
            text = "".join(lines)
        for fast in (False, True):
            with tempfile.TemporaryDirectory() as td:
                inp, out = os.path.join(td, "in.txt"), os.path.join(td, "out.txt")
                with open(inp, "w") as f:
                    f.write(text)
                cmd = [binary, "-q", str(q), "-n", str(n), "-R", str(R), "-M", str(M), "--in", inp, "--out", out]
                if fast:
                    cmd.append("--fast")
                p = subprocess.run(cmd, capture_output=True, text=True)
                m2 = re.search(r"COUNT .*words=(\d+) uncovered=(-?\d+)", p.stdout)
                with open(out) as f:
                    body = f.read()
                cases.append(dict(q=q, n=n, R=R, M=M, fast=fast, input=text, rc=p.returncode,
                                  words=int(m2.group(1)), uncovered=int(m2.group(2)), out=body))
    return cases


def opt_runs(binary):
    """The configurations of the reference optimisation gate
    (cov/opt/selftest.sh:24-33 and :54-62) on the reference engine: p5b at
    seeds 1-3, and at seed 7 with and without --wide."""
    runs = []
    cfgs = [(6, 6, 3, 41, 2000), (6, 8, 4, 169, 150), (7, 5, 2, 120, 400), (3, 7, 1, 34, 1500),
            (5, 4, 0, 600, 300), (4, 5, 4, 3, 100), (2, 8, 2, 12, 800), (6, 5, 2, 66, 900)]
    for (q, n, R, M, it) in cfgs:
        for s in (1, 2, 3):
            runs.append(dict(q=q, n=n, R=R, M=M, seed=s, iters=it, tabu=0, stall=5000, kick=2,
                             random_init=False, code=None, wide=False))
    cfgs2 = [(6, 4, 2, 15, 4000), (7, 3, 1, 25, 4000), (2, 8, 2, 12, 4000), (6, 6, 3, 41, 3000),
             (3, 4, 1, 9, 4000), (5, 4, 1, 125, 2000), (6, 5, 2, 60, 1500)]
    for (q, n, R, M, it) in cfgs2:
        for wide in (False, True):
            runs.append(dict(q=q, n=n, R=R, M=M, seed=7, iters=it, tabu=0, stall=5000, kick=2,
                             random_init=False, code=None, wide=wide))
    # --fix0 (codeword 0 translated to 0^n and frozen), also with kicks and
    # from a given code
    for (q, n, R, M, it) in cfgs2[:5]:
        runs.append(dict(q=q, n=n, R=R, M=M, seed=7, iters=it, tabu=0, stall=5000, kick=2,
                         random_init=False, code=None, wide=False, fix0=True))
        runs.append(dict(q=q, n=n, R=R, M=M, seed=8, iters=it, tabu=5, stall=40, kick=2,
                         random_init=False, code=None, wide=False, fix0=True))
    code = np.random.default_rng(55).integers(0, 6, (41, 6), dtype=np.uint8)
    runs.append(dict(q=6, n=6, R=3, M=41, seed=9, iters=1500, tabu=7, stall=50, kick=2, random_init=False,
                     code=code_text(code), wide=True, fix0=True))
    for r in runs:
        args = ["-q", r["q"], "-n", r["n"], "-R", r["R"], "-M", r["M"], "-s", r["seed"], "--iters", r["iters"],
                "--threads", 1, "--tabu", r["tabu"], "--stall", r["stall"], "--kick", r["kick"]]
        if r["wide"]:
            args.append("--wide")
        if r.get("fix0"):
            args.append("--fix0")
        r["ref"] = run_ref(binary, args, r["code"])
    return runs


def method_runs(binary):
    """The reference engine's other move methods: --sa (focused simulated
    annealing, covsearch2e.c:1408-1441) at its default schedule and at fast
    cooling schedules that reheat, with short stalls; --noise PERMILLE
    (:1443-1448) with and without tabu, kicks, --wide and --fix0."""
    runs = []
    cfgs = [(6, 4, 2, 15, 3000), (7, 3, 1, 25, 3000), (2, 8, 2, 12, 3000), (6, 6, 3, 41, 2000),
            (3, 4, 1, 9, 3000), (5, 4, 1, 125, 1500), (6, 5, 2, 60, 1500), (4, 6, 1, 420, 800)]
    sa_sched = [(0.6, 0.999999, 0.02), (2.0, 0.995, 0.05), (1.0, 0.98, 0.3)]
    for k, (q, n, R, M, it) in enumerate(cfgs):
        for j, sch in enumerate(sa_sched):
            runs.append(dict(q=q, n=n, R=R, M=M, seed=11 + j, iters=it, tabu=0, stall=5000 if j == 0 else 300,
                             kick=2, random_init=False, code=None, wide=False, fix0=(k == 3 and j == 1),
                             sa=list(sch), noise=0))
    for k, (q, n, R, M, it) in enumerate(cfgs):
        for j, nz in enumerate((50, 300)):
            runs.append(dict(q=q, n=n, R=R, M=M, seed=21 + j, iters=it, tabu=0 if j == 0 else 6,
                             stall=5000 if j == 0 else 60, kick=2, random_init=False, code=None,
                             wide=(k % 3 == 1), fix0=(k == 0 and j == 1), sa=None, noise=nz))
    for r in runs:
        args = ["-q", r["q"], "-n", r["n"], "-R", r["R"], "-M", r["M"], "-s", r["seed"], "--iters", r["iters"],
                "--threads", 1, "--tabu", r["tabu"], "--stall", r["stall"], "--kick", r["kick"]]
        if r["wide"]:
            args.append("--wide")
        if r["fix0"]:
            args.append("--fix0")
        if r["sa"] is not None:
            args += ["--sa", "--t0", repr(r["sa"][0]), "--cool", repr(r["sa"][1]), "--tmin", repr(r["sa"][2])]
        if r["noise"]:
            args += ["--noise", r["noise"]]
        r["ref"] = run_ref(binary, args, r["code"])
    return runs


def pick_runs(binary):
    """The reference engine's experimental pick rules, --upick (the oldest
    listed uncovered word, covsearch2e.c:978-985) and --ucache (a cache of
    uncovered words filled by the scan and by commits, :986-1012), alone and
    together, with tabu and kicks."""
    runs = []
    cfgs = [(6, 4, 2, 15, 3000), (7, 3, 1, 25, 3000), (2, 8, 2, 12, 3000), (6, 6, 3, 41, 2000),
            (3, 4, 1, 9, 3000), (6, 5, 2, 60, 1500), (4, 6, 1, 420, 800), (5, 6, 2, 120, 1500)]
    for k, (q, n, R, M, it) in enumerate(cfgs):
        for j, (up, uc) in enumerate(((1, 0), (0, 1), (1, 1))):
            runs.append(dict(q=q, n=n, R=R, M=M, seed=31 + j, iters=it, tabu=0 if j != 1 else 6,
                             stall=5000 if j == 0 else 80, kick=2, random_init=False, code=None, wide=False,
                             fix0=False, upick=bool(up), ucache=bool(uc)))
    for r in runs:
        args = ["-q", r["q"], "-n", r["n"], "-R", r["R"], "-M", r["M"], "-s", r["seed"], "--iters", r["iters"],
                "--threads", 1, "--tabu", r["tabu"], "--stall", r["stall"], "--kick", r["kick"]]
        if r["upick"]:
            args.append("--upick")
        if r["ucache"]:
            args.append("--ucache")
        r["ref"] = run_ref(binary, args, r["code"])
    return runs


def sym_text(rep, q):
    """symsearch's --out file: orbit by orbit, its q words (j, e + j)."""
    return "".join(DIG[j] + "".join(DIG[(int(x) + j) % q] for x in e) + "\n" for e in rep for j in range(q))


def sym_runs(binary):
    """The reference quotient search on a fixed cell list.  It stops on a
    wall-clock limit only, so each run records the iteration count it
    reached; a replay makes exactly that many moves."""
    runs = []
    cells = [(6, 6, 3, 42, 0, 0.15), (3, 7, 2, 30, 0, 0.1), (4, 6, 2, 40, 0, 0.1), (5, 6, 2, 100, 0, 0.1),
             (8, 6, 2, 400, 0, 0.2), (6, 8, 4, 168, 0, 0.3), (3, 9, 2, 150, 0, 0.1), (4, 7, 1, 400, 0, 0.1),
             (3, 6, 0, 300, 0, 0.05), (6, 8, 4, 240, 20, 0.3), (4, 6, 1, 500, 0, 0.1), (7, 5, 2, 140, 0, 0.1),
             (4, 5, 1, 64, 0, 0.1), (3, 5, 1, 27, 0, 0.1)]
    # edge cells: q = 2 and 16, a one-digit quotient (n = 2), R = 0,
    # R >= n - 1, and cells covered by the initial orbits
    edge = [(2, 4, 1, 4, 0, 0.01), (2, 5, 1, 6, 0, 0.01), (3, 2, 0, 3, 0, 0.01), (3, 2, 1, 3, 0, 0.01),
            (3, 3, 1, 3, 0, 0.01), (3, 3, 2, 6, 0, 0.01), (5, 3, 1, 5, 0, 0.01), (16, 3, 1, 48, 0, 0.02),
            (16, 4, 1, 160, 0, 0.02), (9, 4, 2, 27, 0, 0.02), (4, 4, 3, 4, 0, 0.01), (2, 8, 3, 8, 0, 0.01),
            (3, 4, 0, 30, 0, 0.01)]
    for (q, n, R, M, orbits, t) in cells + edge:
        for s, stall, kick in ((1, 3000, 2), (2, 30, 2), (3, 20, 3)):
            args = ["-q", q, "-n", n, "-R", R, "-M", M, "-t", t, "-s", s, "--stall", stall, "--kick", kick,
                    "--threads", 1]
            if orbits:
                args += ["--orbits", orbits]
            with tempfile.TemporaryDirectory() as td:
                out = os.path.join(td, "out.txt")
                p = subprocess.run([binary] + [str(a) for a in args] + ["--out", out], capture_output=True,
                                   text=True)
                m = re.search(r"SYMRESULT .*orbits=(\d+) red_uncovered=(\d+) word_uncovered=(\d+) "
                              r"iters=(\d+) kicks=(\d+)", p.stdout)
                if not m:
                    raise RuntimeError("no SYMRESULT from %s: %s %s" % (args, p.stdout, p.stderr))
                with open(out) as f:
                    body = f.read()
            runs.append(dict(q=q, n=n, R=R, M=M, orbits=orbits, seed=s, stall=stall, kick=kick,
                             ref=dict(orbits=int(m.group(1)), red_uncovered=int(m.group(2)),
                                      word_uncovered=int(m.group(3)), iters=int(m.group(4)),
                                      kicks=int(m.group(5)), rc=p.returncode, out=body)))
    return runs


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("COLDCASE_REF", "/root/reference"))
    ap.add_argument("--only", choices=["methods", "picks"], help="write only this fixture")
    a = ap.parse_args()
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref", "REF=%s" % a.ref], check=True)
    binary = os.path.join(REPO, "oracle", "_ref", "covsearch2e")
    if a.only in (None, "picks"):
        pr = pick_runs(binary)
        with open(os.path.join(HERE, "pick_runs.json"), "w") as f:
            json.dump(pr, f)
        if a.only == "picks":
            print("pick runs: %d" % len(pr))
            return
    mr = method_runs(binary)
    with open(os.path.join(HERE, "method_runs.json"), "w") as f:
        json.dump(mr, f)
    if a.only == "methods":
        print("method runs: %d" % len(mr))
        return
    runs = engine_runs(binary)
    with open(os.path.join(HERE, "engine_runs.json"), "w") as f:
        json.dump(runs, f)
    vc = verify_cases(a.ref)
    with open(os.path.join(HERE, "verify_cases.json"), "w") as f:
        json.dump(vc, f)
    fc = finish_cases(os.path.join(REPO, "oracle", "_ref", "covcount"))
    with open(os.path.join(HERE, "finish_cases.json"), "w") as f:
        json.dump(fc, f)
    orr = opt_runs(binary)
    with open(os.path.join(HERE, "opt_runs.json"), "w") as f:
        json.dump(orr, f)
    sr = sym_runs(os.path.join(REPO, "oracle", "_ref", "symsearch"))
    with open(os.path.join(HERE, "sym_runs.json"), "w") as f:
        json.dump(sr, f)
    print("engine runs: %d, verify cases: %d, finish cases: %d, quotient runs: %d"
          % (len(runs), len(vc), len(fc), len(sr)))


if __name__ == "__main__":
    main()
