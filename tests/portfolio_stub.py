#!/usr/bin/env python3
"""Test double of the covsearch_gpu drop-in for hosts without a GPU.

Runs covsearch_gpu's own command line -- argument handling, --out
publication, RESULT line, exit status -- with the oracle (the CPU
restatement of the same p5b search) standing in for the GPU engine, so that
a portfolio driver (cov/campaign.py, cov/engine/covengine) can be exercised
against the drop-in's protocol on any host.  Test infrastructure only: the
product CLI never falls back to the oracle.
"""
import os
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)

from coldcase_gb300 import covsearch_gpu  # noqa: E402
from oracle.pyoracle import Oracle  # noqa: E402


class OracleSearch:
    """The part of engine.Search the command line uses, on the oracle."""

    def __init__(self, q, n, R, M, seed=12345, tabu=0, kick=2, stall=5000, cand=100000, cluster=1, wide=False,
                 fix0=False, sa=None, noise=0):
        self.o = Oracle(q, n, R, M, seed=seed, tabu=tabu, kick=kick, stall=stall, cand=cand, wide=wide, fix0=fix0,
                        sa=sa, noise=noise)

    def load(self, code=None, random_init=False):
        self.o.init(code, random_init=random_init)
        return self.o.uncovered()

    def status(self):
        return dict(it=self.o.iters(), uncovered=self.o.uncovered(), best=self.o.best_uncovered(),
                    kicks=self.o.kicks(), status=0)

    def run(self, moves, target=-1):
        self.o.run(moves)
        return self.status()

    def best(self):
        return self.o.best()

    def close(self):
        self.o.close()


if __name__ == "__main__":
    covsearch_gpu.Search = OracleSearch
    sys.exit(covsearch_gpu.main())
