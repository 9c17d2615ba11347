"""gpuchain-compatible command line on the GPU transform-engine LNS.

Same flags as cov/gemm2/gpuchain.py (:412-457): -q -n -R -M -t -s --out
[--in SEEDFILE] [--kmin K] [--kmax K] [--quiet]; the best code goes to --out
(atomically, on improvement, at most once a second, and at the end) and one
RESULT line reports M, uncovered, rounds, placements+removals per second,
transforms and time.  A seed file with more than M words is first ruined
down to M by the soft minimum of private coverage (lns.LNS.ruin).
"""
import argparse
import sys
import time

import numpy as np

from . import codefile
from .lns import LNS


def main(argv=None):
    ap = argparse.ArgumentParser(prog="gpuchain_gpu")
    ap.add_argument("-q", type=int, required=True)
    ap.add_argument("-n", type=int, required=True)
    ap.add_argument("-R", type=int, required=True)
    ap.add_argument("-M", type=int, required=True)
    ap.add_argument("-t", type=float, default=60.0)
    ap.add_argument("-s", type=int, default=1)
    ap.add_argument("--out", required=True)
    ap.add_argument("--in", dest="seed_code")
    ap.add_argument("--kmin", type=int, default=8)
    ap.add_argument("--kmax", type=int)
    ap.add_argument("--quiet", action="store_true")
    ap.add_argument("--rounds", type=int, help="stop after this many LNS rounds")
    a = ap.parse_args(argv)
    t_start = time.time()
    deadline = t_start + a.t
    log = (lambda *x: None) if a.quiet else print
    with LNS(a.q, a.n, a.R, seed=a.s, out=a.out, log=log, deadline=deadline) as e:
        if a.seed_code:
            e.load(codefile.read_code(a.seed_code, a.n))
            if len(e.code) > a.M:
                e.ruin(len(e.code) - a.M, "soft")
        else:
            e.load(np.zeros(0, dtype=np.int64))
        unc = e.lns(a.M, budget_s=deadline - time.time() - 5, kmin=a.kmin, kmax=a.kmax, max_rounds=a.rounds)
        if unc == 0:
            unc = e.recount_from_scratch()
        e.publish(force=True)
        dt = time.time() - t_start
        moves = e.stats["placements"] + e.stats["removals"]
        print("RESULT q=%d n=%d R=%d M=%d uncovered=%d iters=%d rate=%.1f transforms=%d time=%.1f"
              % (a.q, a.n, a.R, len(e.code), unc, e.stats["rounds"], moves / max(dt, 1e-9),
                 e.stats["transforms"], dt))
    return 0


if __name__ == "__main__":
    sys.exit(main())
