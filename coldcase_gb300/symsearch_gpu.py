"""symsearch-compatible command line on the GPU quotient engine.

Drop-in for the binary covengine starts as BIN['symsearch']
(cov/engine/covengine:70, :654-660): the flags of cov/engine/symsearch.c:282-310
(-q -n -R -M -t -s --out --orbits --kick --stall --cand --threads -v), the
argument checks and exit statuses 2 and 3 (:311-333), the "# improved:
word_uncovered=" lines the driver's log parser reads (covengine:87, :194),
the SYMRESULT line (:478-482), the --out file (orbit by orbit, its q words;
written at the start, on improvement at most once a second and at the end,
:250-266, :370-383) and exit status 0 iff the quotient is covered.  The
search is the reference's trajectory; it stops on the -t wall-clock limit
like the reference, or after --iters iterations (a GPU-only flag).
"""
import os
import sys
import time

from . import sym
from .lib import CovError

USAGE = "usage: symsearch -q Q -n N -R R -M M [-t sec] [-s seed] [--out f]\n"
VALUE_FLAGS = {"-q", "-n", "-R", "-M", "-t", "-s", "--out", "--orbits", "--kick", "--stall", "--cand",
               "--threads", "--cluster", "--iters"}


def parse(argv):
    a = dict(q=0, n=0, R=0, M=0, t=60.0, s=12345, out=None, orbits=0, kick=2, stall=3000, cand=100000,
             verbose=False, cluster=None, iters=-1)
    i = 0
    while i < len(argv):
        f = argv[i]
        if f in VALUE_FLAGS and i + 1 < len(argv):
            v = argv[i + 1]
            i += 2
            try:
                if f == "-q": a["q"] = int(v)
                elif f == "-n": a["n"] = int(v)
                elif f == "-R": a["R"] = int(v)
                elif f == "-M": a["M"] = int(v)
                elif f == "-t": a["t"] = float(v)
                elif f == "-s": a["s"] = int(v)
                elif f == "--out": a["out"] = v
                elif f == "--orbits": a["orbits"] = int(v)
                elif f == "--kick": a["kick"] = int(v)
                elif f == "--stall": a["stall"] = int(v)
                elif f == "--cand": a["cand"] = int(v)
                elif f == "--cluster": a["cluster"] = int(v)
                elif f == "--iters": a["iters"] = int(v)
            except ValueError:
                sys.stderr.write("bad option %s\n" % f)
                return None, 2
            continue
        if f == "-v":
            a["verbose"] = True
            i += 1
            continue
        sys.stderr.write("bad option %s\n" % f)
        return None, 2
    if a["q"] < 2 or a["n"] < 2 or a["R"] < 0 or a["R"] > 7 or a["M"] < a["q"]:
        sys.stderr.write(USAGE)
        return None, 2
    return a, 0


def write_reps(path, reps, q):
    tmp = path + ".part"
    with open(tmp, "w") as f:
        f.write(sym.format_code(reps, q))
    os.replace(tmp, path)


def main(argv=None):
    t0 = time.monotonic()
    a, rc = parse(sys.argv[1:] if argv is None else argv)
    if a is None:
        return rc
    q, n, R, M = a["q"], a["n"], a["R"], a["M"]
    try:
        norb = sym.orbits_of(q, n, R, M, a["orbits"])
    except CovError as e:
        if e.rc == -1:
            sys.stderr.write(USAGE)
            return 2
        sys.stderr.write("symsearch_gpu: orbits, quotient or M out of range\n")
        return 3
    N = q ** (n - 1)
    cluster = a["cluster"] or (16 if N >= 1 << 22 else 8 if N >= 1 << 18 else 2)
    try:
        # one instance: its estimates spread over the whole GPU
        pool = sym.SymPool(1, cluster=cluster, budget_s=max(1.0, min(30.0, a["t"])), grid_eval=True)
        s = pool.add(q, n, R, M, orbits=a["orbits"], seed=a["s"], kick=a["kick"], stall=a["stall"], cand=a["cand"])
    except CovError as e:
        sys.stderr.write("symsearch_gpu: %s\n" % e)
        return 3
    st = pool.status(s)
    best = st["best"]
    if a["verbose"]:
        print("# symsearch q=%d n=%d R=%d M=%d orbits=%d quotient=%d init_unc=%d(x%d words)"
              % (q, n, R, M, norb, N, st["uncovered"], q))
        sys.stdout.flush()
    last_pub = [-1e9]

    def publish(force):
        if not a["out"]:
            return
        now = time.monotonic()
        if not force and now - last_pub[0] < 1.0:
            return
        last_pub[0] = now
        write_reps(a["out"], pool.best(s), q)

    publish(True)
    chunk = 16
    while st["uncovered"] > 0 and st["status"] == 0:
        if time.monotonic() - t0 > a["t"]:
            break
        if a["iters"] >= 0 and st["it"] >= a["iters"]:
            break
        k = chunk if a["iters"] < 0 else min(chunk, a["iters"] - st["it"])
        tc = time.monotonic()
        pool.run(k)
        dt = time.monotonic() - tc
        if dt < 0.05:
            chunk = min(chunk * 2, 1 << 20)
        elif dt > 0.2 and chunk > 1:
            chunk = max(1, chunk // 2)
        st = pool.status(s)
        if st["best"] < best:
            best = st["best"]
            print("# improved: word_uncovered=%d red=%d it=%d t=%.1f" % (best * q, best, st["it"],
                                                                         time.monotonic() - t0))
            sys.stdout.flush()
            publish(best == 0)
    if st["status"] != 0:
        sys.stderr.write("symsearch_gpu: engine status %d\n" % st["status"])
    el = time.monotonic() - t0
    it = st["it"]
    print("SYMRESULT q=%d n=%d R=%d M=%d orbits=%d red_uncovered=%d word_uncovered=%d iters=%d kicks=%d "
          "time=%.2f rate=%.0f" % (q, n, R, norb * q, norb, st["best"], st["best"] * q, it, st["kicks"], el,
                                   it / (el if el > 0 else 1)))
    sys.stdout.flush()
    publish(True)
    pool.close()
    if st["status"] != 0:
        return 2
    return 0 if st["best"] == 0 else 1


if __name__ == "__main__":
    sys.exit(main())
