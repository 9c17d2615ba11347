"""covsearch2e-compatible command line on the GPU engine.

Drop-in for the binary that cov/engine/covengine (BIN['covsearch2e'],
covengine:66-72, :624-643) and cov/campaign.py (COVSEARCH_BIN, :38, :54-86)
launch: same flags (cov/engine/covsearch2e.c:1042-1095), same RESULT line
(:1585-1589), same --out publication (M distinct words, atomic, at start, on
improvement at most once a second, and at the end: :778-868) and the same
exit status (0 iff the best code covers, 1 otherwise, 2 on bad arguments).

The search is the p5b trajectory, with or without --wide (every
single-coordinate move of each candidate codeword while the uncovered list
is short, covsearch2e.c:1353-1376), --fix0 (the initial code translated
so that codeword 0 is 0^n, which then never moves, :1241-1253, :1343,
:1560), --noise PERMILLE (that share of the moves taken from the sample
unevaluated, :1443-1448) and --sa --t0 --cool --tmin (focused simulated
annealing in place of the tabu selection, :1408-1441).  Presets
base/p1..p5/p5b/best and the speed-only switches (--st --eval --walk --hoist
--early --pf --huge --threads) leave the trajectory unchanged in the
reference (cov/opt/METHODS.md:395-409) and are accepted; --ucache and
--upick, which change the trajectory, are rejected with exit status 2.
"""
import os
import sys
import time

import numpy as np

from . import codefile
from .engine import Search
from .lib import CovError

USAGE = ("usage: covsearch -q Q -n N -R R -M M [-t sec] [-s seed] [--in f] [--out f]\n"
         "                 [--cand K] [--tabu T] [--kick K] [--noise PERMILLE] [--iters I]\n"
         "                 [--stall S] [--sa --t0 T0 --cool C --tmin TMIN]\n"
         "                 [--random-init] [--wide] [--fix0] [--grid-help K]\n"
         "                 [--threads T] [--quiet]\n")

PRESETS = {"base", "p1", "p2", "p2b", "p3", "p4", "p5", "best", "p5b"}
VALUE_FLAGS = {"-q", "-n", "-R", "-M", "-t", "-s", "--in", "--out", "--cand", "--tabu", "--kick",
               "--noise", "--iters", "--stall", "--threads", "--t0", "--cool", "--tmin", "--st",
               "--eval", "--walk", "--target", "--cpu", "--preset", "--cluster", "--chunk", "--grid-help"}
SPEED_SWITCHES = {"--hoist", "--early", "--pf", "--huge"}
TRAJECTORY_SWITCHES = {"--ucache", "--upick"}


def parse(argv):
    a = dict(q=0, n=0, R=-1, M=0, t=60.0, s=12345, inp=None, out=None, cand=100000, tabu=0,
             kick=2, noise=0, iters=-1, stall=5000, random_init=False, quiet=False, target=-1,
             cluster=None, chunk=0, wide=False, fix0=False, grid_help=0, sa=False, t0=0.6, cool=0.999999,
             tmin=0.02)
    i = 0
    while i < len(argv):
        f = argv[i]
        if f in VALUE_FLAGS and i + 1 < len(argv):
            v = argv[i + 1]
            i += 2
            if f == "-q": a["q"] = int(v)
            elif f == "-n": a["n"] = int(v)
            elif f == "-R": a["R"] = int(v)
            elif f == "-M": a["M"] = int(v)
            elif f == "-t": a["t"] = float(v)
            elif f == "-s": a["s"] = int(v)
            elif f == "--in": a["inp"] = v
            elif f == "--out": a["out"] = v
            elif f == "--cand": a["cand"] = int(v)
            elif f == "--tabu": a["tabu"] = int(v)
            elif f == "--kick": a["kick"] = int(v)
            elif f == "--noise": a["noise"] = int(v)
            elif f == "--t0": a["t0"] = float(v)
            elif f == "--cool": a["cool"] = float(v)
            elif f == "--tmin": a["tmin"] = float(v)
            elif f == "--iters": a["iters"] = int(v)
            elif f == "--stall": a["stall"] = int(v)
            elif f == "--target": a["target"] = int(v)
            elif f == "--cluster": a["cluster"] = int(v)
            elif f == "--chunk": a["chunk"] = int(v)
            elif f == "--grid-help": a["grid_help"] = int(v)
            elif f == "--preset" and v not in PRESETS:
                sys.stderr.write("unknown preset %s\n" % v)
                return None, 2
            continue
        if f == "--random-init":
            a["random_init"] = True
        elif f == "--wide":
            a["wide"] = True
        elif f == "--fix0":
            a["fix0"] = True
        elif f == "--sa":
            a["sa"] = True
        elif f == "--quiet":
            a["quiet"] = True
        elif f in SPEED_SWITCHES:
            pass
        elif f in TRAJECTORY_SWITCHES:
            sys.stderr.write("%s changes the search trajectory and is not provided by the GPU engine\n" % f)
            return None, 2
        else:
            sys.stderr.write("unknown/incomplete option %s\n" % f)
            return None, 2
        i += 1
    if a["q"] < 2 or a["n"] < 1 or a["R"] < 0 or a["M"] < 1:
        sys.stderr.write(USAGE)
        return None, 2
    return a, 0


def main(argv=None):
    t_start = time.monotonic()
    a, rc = parse(sys.argv[1:] if argv is None else argv)
    if a is None:
        return rc
    q, n, R, M = a["q"], a["n"], a["R"], a["M"]
    if q ** n > 4 * 10 ** 10 or q > 16 or n > 16 or q ** n >= 2 ** 32 - 1:
        sys.stderr.write("q^n too large\n")
        return 2
    if M > 65535:
        sys.stderr.write("M > 65535 not supported (uint16 counters)\n")
        return 2
    verbose = not a["quiet"]
    N = q ** n
    V = sum(__import__("math").comb(n, i) * (q - 1) ** i for i in range(0, min(R, n) + 1))
    S = __import__("math").comb(n - 1, R) * (q - 1) ** R if R <= n - 1 else 0
    if verbose:
        print("# covsearch q=%d n=%d R=%d M=%d  q^n=%d  ball=%d  sphere-move=%d  threads=gpu"
              % (q, n, R, M, N, V, S))
        print("# sphere-covering bound: M >= %d" % ((N + V - 1) // V))
        sys.stdout.flush()
    code = None
    if a["inp"]:
        try:
            code = codefile.read_code(a["inp"], n)
        except (OSError, codefile.CodeFileError) as e:
            sys.stderr.write("%s\n" % e)
            return 1
        if len(code) and int(code.max()) >= q:
            sys.stderr.write("%s: digit out of range for q=%d\n" % (a["inp"], q))
            return 1
        if verbose and len(code) > M:
            print("# seed has %d codewords; dropping %d by remove-and-repair" % (len(code), len(code) - M))
    cluster = a["cluster"] or (8 if N >= 1 << 20 else 2)
    try:
        eng = Search(q, n, R, M, seed=a["s"], tabu=a["tabu"], kick=a["kick"], stall=a["stall"],
                     cand=a["cand"], cluster=cluster, wide=a["wide"], fix0=a["fix0"], noise=a["noise"],
                     sa=(a["t0"], a["cool"], a["tmin"]) if a["sa"] else None)
        if a["grid_help"]:
            # this process's search takes the whole GPU: helper clusters share its commits
            eng.pool.set_param("grid_help", a["grid_help"])
        unc0 = eng.load(code, random_init=a["random_init"])
    except CovError as e:
        sys.stderr.write("covsearch_gpu: %s\n" % e)
        return 2
    last_pub = [-1e9]

    def publish(force):
        if not a["out"]:
            return
        now = time.monotonic()
        if not force and now - last_pub[0] < 1.0:
            return
        last_pub[0] = now
        codefile.write_code(a["out"], eng.best(), q, n, M)

    publish(True)
    if verbose:
        print("# init uncovered=%d" % unc0)
        sys.stdout.flush()
    t0 = time.monotonic()
    st = eng.status()
    best = st["best"]
    chunk = a["chunk"] or 64
    last_report = 0.0
    while st["uncovered"] > 0 and st["status"] == 0:
        if time.monotonic() - t_start > a["t"]:
            break
        if a["iters"] >= 0 and st["it"] >= a["iters"]:
            break
        if a["target"] >= 0 and st["best"] <= a["target"]:
            break
        k = chunk if a["iters"] < 0 else min(chunk, a["iters"] - st["it"])
        tc = time.monotonic()
        st = eng.run(k, a["target"])
        dt = time.monotonic() - tc
        if not a["chunk"]:
            # aim at ~0.1 s per launch so deadlines stay tight
            if dt < 0.05:
                chunk = min(chunk * 2, 1 << 20)
            elif dt > 0.2 and chunk > 1:
                chunk = max(1, chunk // 2)
        el = time.monotonic() - t0
        if st["best"] < best:
            best = st["best"]
            if verbose:
                print("# improved: unc=%d at it=%d t=%.1fs" % (best, st["it"], el))
                sys.stdout.flush()
            publish(best == 0)
        if verbose and el - last_report > 10.0:
            last_report = el
            print("# t=%6.1fs it=%-10d unc=%-10d best=%d (%.0f it/s)"
                  % (el, st["it"], st["uncovered"], st["best"], st["it"] / el if el > 0 else 0))
            sys.stdout.flush()
    if st["status"] != 0:
        sys.stderr.write("covsearch_gpu: engine status %d\n" % st["status"])
    el = time.monotonic() - t0
    it = st["it"]
    print("RESULT q=%d n=%d R=%d M=%d uncovered=%d iters=%d kicks=%d time=%.2f rate=%.0f "
          "cpu=%.3f cpurate=%.0f target=%d ttt_cpu=-1.0000 ttt_wall=-1.0000 ttt_it=-1"
          % (q, n, R, M, st["best"], it, st["kicks"], el, it / (el if el > 0 else 1),
             time.process_time(), it / max(time.process_time(), 1e-9), a["target"]))
    sys.stdout.flush()
    publish(True)
    eng.close()
    if st["status"] != 0:
        return 2
    return 0 if st["best"] == 0 else 1


if __name__ == "__main__":
    sys.exit(main())
