#!/usr/bin/env python3
"""Warm states of the 64-restart q7 n9 R4 M1500 workload (tenure 20).

The batched benchmark times moves 5001.. of 64 restarts, each started from
the uniform code of seed instance_seed(1, i) (i = 0..63) with search seed
instance_seed(1, i).  This script advances every restart 5000 moves on the
oracle (the CPU restatement of covsearch2e p5b) and records where it stands:

  warm_q7n9.json   per restart: seed, iterations, current and best
                   uncovered counts, kicks, the RNG state, and sha256 digests
                   of the current code, the best code, the tabu table and the
                   coverage-count array -- the GPU engine must reach exactly
                   this state (tests/test_gpu_headline.py);
  warm_q7n9.npz    the current codes of restarts 0..15 (uint8 [16, 1500, 9]):
                   the reference engine's CPU timing starts from them, so it
                   measures the same phase of the search as the GPU.

Usage: python3 tests/golden/make_warm.py [--moves 5000] [--restarts 64] [--procs 8]
"""
import argparse
import hashlib
import json
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

Q, N, R, M, TENURE, BASE_SEED = 7, 9, 4, 1500, 20, 1
KEEP_CODES = 16


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def one(args):
    i, moves = args
    from oracle.pyoracle import Oracle
    from coldcase_gb300.workloads import instance_seed, uniform_code
    seed = instance_seed(BASE_SEED, i)
    o = Oracle(Q, N, R, M, seed=seed, tabu=TENURE, threads=1)
    o.init(uniform_code(Q, N, M, seed))
    o.run(moves)
    code = o.code()
    rec = dict(restart=i, seed=seed, it=int(o.iters()), unc=int(o.uncovered()), best=int(o.best_uncovered()),
               kicks=int(o.kicks()), rng=[int(x) for x in o.rng()], code_sha=sha(code), best_sha=sha(o.best()),
               tabu_sha=sha(o.tabu()), cnt_sha=sha(o.cnt()))
    o.close()
    return rec, code


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--moves", type=int, default=5000)
    ap.add_argument("--restarts", type=int, default=64)
    ap.add_argument("--procs", type=int, default=os.cpu_count() or 1)
    a = ap.parse_args()
    with mp.get_context("spawn").Pool(a.procs) as pool:
        res = pool.map(one, [(i, a.moves) for i in range(a.restarts)])
    recs = [r for r, _ in res]
    codes = np.stack([c for _, c in res[:KEEP_CODES]]).astype(np.uint8)
    meta = dict(q=Q, n=N, R=R, M=M, tenure=TENURE, moves=a.moves, base_seed=BASE_SEED,
                note="oracle state of restart i after `moves` moves from uniform_code(q, n, M, seed), "
                     "seed = instance_seed(base_seed, i)", restarts=recs)
    with open(os.path.join(HERE, "warm_q7n9.json"), "w") as f:
        json.dump(meta, f, indent=0)
    np.savez_compressed(os.path.join(HERE, "warm_q7n9.npz"), codes=codes,
                        seeds=np.array([r["seed"] for r in recs[:KEEP_CODES]], dtype=np.int64))
    print("restarts %d, moves %d, best uncovered %s" % (len(recs), a.moves, [r["best"] for r in recs[:8]]))


if __name__ == "__main__":
    main()
