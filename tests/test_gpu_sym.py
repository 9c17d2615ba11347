"""CUDA quotient search vs the oracle and the reference's golden runs.

Bit-exact: every move record (picked quotient word, candidate count and
sample size, committed move, its estimate, uncovered counts, kicks), the
final RNG state, the quotient counters and the best representatives must
equal the oracle's; the SYMRESULT fingerprint and the --out file must equal
the reference binary's.
"""
import numpy as np
import pytest

from coldcase_gb300.sym import SymPool, format_code
from tests.util import sym_oracle_run

pytestmark = pytest.mark.gpu


def first_diff(a, b):
    for k in range(min(len(a), len(b))):
        if a[k].tobytes() != b[k].tobytes():
            return k, a[k], b[k]
    return min(len(a), len(b)), None, None


def gpu_sym(pool, r, iters):
    s = pool.add(r["q"], r["n"], r["R"], r["M"], orbits=r["orbits"], seed=r["seed"], kick=r["kick"],
                 stall=r["stall"], trace=1, trace_cap=max(1, iters))
    return s


@pytest.mark.parametrize("cluster", [1, 4])
def test_sym_golden_runs_bit_exact(covlib, sym_golden, cluster):
    bad = []
    for r in sym_golden:
        ref = r["ref"]
        pool = SymPool(1, cluster=cluster)
        s = gpu_sym(pool, r, ref["iters"])
        pool.run(ref["iters"])
        st = pool.status(s)
        o, otr = sym_oracle_run(r)
        gtr = pool.trace(s)
        got = (st["best"], st["it"], st["kicks"])
        want = (ref["red_uncovered"], ref["iters"], ref["kicks"])
        ok = st["status"] == 0 and got == want and format_code(pool.best(s), r["q"]) == ref["out"]
        ok = ok and gtr.tobytes() == otr.tobytes() and (pool.rng(s) == o.rng()).all()
        ok = ok and (pool.cnt(s) == o.cnt()).all() and (pool.rep(s) == o.rep()).all()
        if not ok:
            k, g1, o1 = first_diff(gtr, otr)
            bad.append(dict(cell=(r["q"], r["n"], r["R"], r["M"], r["orbits"], r["seed"]), got=got, want=want,
                            status=st["status"], ntr=(len(gtr), len(otr)), first=k,
                            gpu=None if g1 is None else g1.tolist(), orc=None if o1 is None else o1.tolist()))
        pool.close()
    assert not bad, bad[:3]


def test_sym_chunks_and_batch_equal_single_runs(covlib, sym_golden):
    """Short launches equal one long one, and instances sharing a pool (one
    launch per cluster size) each follow their own trajectory."""
    runs = [r for r in sym_golden if r["seed"] == 2][:6]
    single = []
    for r in runs:
        pool = SymPool(1, cluster=2)
        s = gpu_sym(pool, r, 3000)
        left = 3000
        while left > 0:
            k = min(left, 257)
            pool.run(k)
            left -= k
        single.append(pool.trace(s))
        pool.close()
    pool = SymPool(len(runs), cluster=1)
    slots = [gpu_sym(pool, r, 3000) for r in runs]
    for k, s in enumerate(slots):
        pool.set_slot_param(s, "cluster", 1 + (k % 3))
    pool.run(3000)
    for r, s, tr in zip(runs, slots, single):
        o, otr = sym_oracle_run(r, moves=3000)
        assert tr.tobytes() == otr.tobytes(), (r["q"], r["n"], r["R"], r["M"])
        assert pool.trace(s).tobytes() == otr.tobytes(), (r["q"], r["n"], r["R"], r["M"])
    pool.close()


def test_sym_big_quotient_parity(covlib):
    """K_8(9,4) shape (quotient 8^8 = 16.7M counters, 117 orbits) for 40
    moves at cluster 16 against the oracle."""
    from oracle.pyoracle import SymOracle
    q, n, R, M = 8, 9, 4, 940
    o = SymOracle(q, n, R, M, seed=1000)
    o.init()
    otr = o.run(40, trace=True)
    with SymPool(1, cluster=16) as pool:
        s = pool.add(q, n, R, M, seed=1000, trace=1, trace_cap=40)
        pool.run(40)
        gtr = pool.trace(s)
        k, g1, o1 = first_diff(gtr, otr)
        assert len(gtr) == len(otr) and k == len(otr), (k, g1, o1)
        assert (pool.cnt(s) == o.cnt()).all()


def test_sym_timeout_resume_keeps_trajectory(covlib, sym_golden):
    """A launch deadline stops an instance between two moves (or between two
    orbit placements of its initialisation) with COV_ETIMEOUT; after
    resume the run continues on exactly the uninterrupted trajectory."""
    r = [x for x in sym_golden if (x["q"], x["n"], x["R"], x["M"]) == (6, 8, 4, 168)][0]
    moves = 120
    o, otr = sym_oracle_run(r, moves=moves)
    pool = SymPool(1, cluster=1, budget_s=0.002)
    s = gpu_sym(pool, r, moves)
    stops = 0
    for _ in range(100000):
        st = pool.status(s)
        if st["status"] == -4:
            stops += 1
            pool.resume(s)
            continue
        assert st["status"] == 0, st
        if st["it"] >= moves or st["finished"]:
            break
        pool.run(moves - st["it"])
    assert stops > 0
    gtr = pool.trace(s)
    assert gtr.tobytes() == otr.tobytes()
    assert (pool.cnt(s) == o.cnt()).all()
    pool.close()


@pytest.mark.parametrize("cell,cand,kick,stall", [((6, 8, 4, 168), 7, 0, 15), ((5, 6, 2, 100), 3, 1, 25),
                                                  ((3, 9, 2, 150), 50, 4, 40)])
def test_sym_sample_cap_and_kicks(covlib, cell, cand, kick, stall):
    """A candidate cap below the candidate count (sampled subsets), no-op
    kicks and kicks of several orbits, against the oracle move by move."""
    from oracle.pyoracle import SymOracle
    q, n, R, M = cell
    moves = 400
    o = SymOracle(q, n, R, M, seed=5, kick=kick, stall=stall, cand=cand)
    o.init()
    otr = o.run(moves, trace=True)
    with SymPool(1, cluster=2) as pool:
        s = pool.add(q, n, R, M, seed=5, kick=kick, stall=stall, cand=cand, trace=1, trace_cap=moves)
        pool.run(moves)
        gtr = pool.trace(s)
        k, g1, o1 = first_diff(gtr, otr)
        assert len(gtr) == len(otr) and k == len(otr), (k, g1, o1)
        assert (pool.cnt(s) == o.cnt()).all() and (pool.best(s) == o.best()).all()
        assert (pool.rng(s) == o.rng()).all()


def test_sym_grid_eval_bit_exact(covlib, sym_golden):
    """One instance with its estimates spread over the whole GPU (a launch
    per move) follows the same trajectory, also across runs that switch the
    mode in the middle."""
    for r in [x for x in sym_golden if x["seed"] == 1][::3]:
        moves = min(r["ref"]["iters"], 1500)
        o, otr = sym_oracle_run(r, moves=moves)
        pool = SymPool(1, cluster=4, grid_eval=True)
        s = gpu_sym(pool, r, moves)
        pool.set_slot_param(s, "it_limit", moves)
        pool.run(moves // 2)
        pool.lib.cov_sym_set_param(pool.h, b"grid_eval", 0)
        pool.run(7)
        pool.lib.cov_sym_set_param(pool.h, b"grid_eval", 1)
        pool.run(moves)
        gtr = pool.trace(s)
        k, g1, o1 = first_diff(gtr, otr)
        assert len(gtr) == len(otr) and k == len(otr), (r["q"], r["n"], r["R"], r["M"], k, g1, o1)
        assert (pool.cnt(s) == o.cnt()).all()
        pool.close()
