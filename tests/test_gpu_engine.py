"""CUDA tabu engine vs the oracle and the reference's golden runs.

Bit-exact: every move record (picked word, candidate count, committed move,
delta, uncovered counts), the final RNG state, tabu table, coverage counts
and the best code must equal the oracle's; fingerprints and --out files must
equal the reference binary's.
"""
import numpy as np
import pytest

from coldcase_gb300 import codefile
from coldcase_gb300.engine import Pool
from tests.util import code_from_text, oracle_run

pytestmark = pytest.mark.gpu


def private_counts(cnt, code, q, n, R):
    """(T_k, H_k[j]) of every codeword from a coverage array (small N only)."""
    N = q ** n
    pw = q ** np.arange(n - 1, -1, -1, dtype=np.int64)
    digits = (np.arange(N, dtype=np.int64)[:, None] // pw[None, :]) % q
    one = cnt == 1
    out = np.zeros((len(code), n + 1), dtype=np.int64)
    for k, c in enumerate(code):
        diff = digits != c[None, :].astype(np.int64)
        on = one & (diff.sum(axis=1) == R)
        out[k, 0] = on.sum()
        out[k, 1:] = diff[on].sum(axis=0)
    return out


def gpu_run(run, cluster):
    pool = Pool(1, cluster=cluster)
    code = code_from_text(run["code"], run["n"]) if run["code"] else None
    s = pool.add(run["q"], run["n"], run["R"], run["M"], code=code, random_init=run["random_init"],
                 seed=run["seed"], tabu=run["tabu"], kick=run["kick"], stall=run["stall"],
                 trace=1, trace_cap=max(1, run["iters"]), wide=run.get("wide", False))
    pool.run(run["iters"])
    return pool, s


def first_diff(a, b):
    for k in range(min(len(a), len(b))):
        if a[k].tobytes() != b[k].tobytes():
            return k, a[k], b[k]
    return min(len(a), len(b)), None, None


@pytest.mark.parametrize("cluster", [1, 4])
def test_golden_runs_bit_exact(covlib, golden, cluster):
    runs, _ = golden
    bad = []
    for r in runs:
        pool, s = gpu_run(r, cluster)
        st = pool.status(s)
        o, otr = oracle_run(r)
        gtr = pool.trace(s)
        ref = r["ref"]
        assert st["status"] == 0, (r, st)
        got = (st["best"], st["it"], st["kicks"])
        want = (ref["uncovered"], ref["iters"], ref["kicks"])
        out = codefile.format_code(codefile.distinct_code(pool.best(s), r["q"], r["n"], r["M"]), r["q"])
        ok = got == want and out == ref["out"] and gtr.tobytes() == otr.tobytes()
        ok = ok and (pool.rng(s) == o.rng()).all() and (pool.tabu(s) == o.tabu()).all()
        ok = ok and (pool.code(s) == o.code()).all() and (pool.cnt(s) == o.cnt()).all()
        if not ok:
            k, g1, o1 = first_diff(gtr, otr)
            bad.append(dict(cell=(r["q"], r["n"], r["R"], r["M"], r["seed"]), got=got, want=want,
                            out_ok=out == ref["out"], ntr=(len(gtr), len(otr)), first=k,
                            gpu=None if g1 is None else g1.tolist(),
                            orc=None if o1 is None else o1.tolist()))
        pool.close()
    assert not bad, bad[:3]


def test_private_counts_exact(covlib, golden):
    runs, _ = golden
    for r in [x for x in runs if x["q"] ** x["n"] <= 50000 and x["R"] > 0][:12]:
        pool, s = gpu_run(r, 2)
        P = pool.private(s)
        want = private_counts(pool.cnt(s), pool.code(s), r["q"], r["n"], r["R"])
        assert (P == want).all(), (r["q"], r["n"], r["R"], r["M"])
        pool.close()


def test_plain_q6_n9_parity(covlib):
    """The single-instance GPU configuration (q6 n9 R4 M700, tenure 20):
    2000 moves compared move by move with the oracle."""
    from oracle.pyoracle import Oracle
    from coldcase_gb300.workloads import uniform_code
    q, n, R, M = 6, 9, 4, 700
    code = uniform_code(q, n, M, 1)
    o = Oracle(q, n, R, M, seed=1, tabu=20, threads=8)
    o.init(code)
    otr = o.run(2000, trace=True)
    pool = Pool(1, cluster=8)
    s = pool.add(q, n, R, M, code=code, seed=1, tabu=20, trace=1, trace_cap=2000)
    for _ in range(4):
        pool.run(500)
    gtr = pool.trace(s)
    k, g1, o1 = first_diff(gtr, otr)
    assert len(gtr) == len(otr) and k == len(otr), (k, g1, o1)
    assert (pool.cnt(s) == o.cnt()).all()
    assert (pool.best(s) == o.best()).all()


def test_chunked_runs_equal_one_run(covlib, golden):
    runs, _ = golden
    r = [x for x in runs if x["q"] == 6 and x["n"] == 6 and x["code"]][0]
    a, sa = gpu_run(r, 2)
    b = Pool(1, cluster=2)
    code = code_from_text(r["code"], r["n"])
    sb = b.add(r["q"], r["n"], r["R"], r["M"], code=code, seed=r["seed"], tabu=r["tabu"],
               kick=r["kick"], stall=r["stall"], trace=1, trace_cap=r["iters"])
    left = r["iters"]
    while left > 0:
        k = min(left, 37)
        b.run(k)
        left -= k
    assert a.trace(sa).tobytes() == b.trace(sb).tobytes()


def test_wide_variants_match_oracle(covlib, golden):
    """--wide through every entering-side route: the bit-sliced and the
    pairwise list pass, one CTA or the whole cluster sharing the pass, and a
    candidate cap below the candidate count (sampled subsets)."""
    from oracle.pyoracle import Oracle
    runs, _ = golden
    wide = [r for r in runs if r.get("wide")]
    assert wide
    cases = []
    for r in wide[:4]:
        cases.append((r, dict(cluster=1, wide_sliced=0), 100000))
        cases.append((r, dict(cluster=4, neg_cluster_pairs=0), 100000))
        cases.append((r, dict(cluster=2, neg_cluster_pairs=0, wide_sliced=0), 100000))
    for r in wide[:3]:
        cases.append((r, dict(cluster=2), 37))
    bad = []
    for r, prm, cand in cases:
        pool = Pool(1, cluster=prm.get("cluster", 1))
        code = code_from_text(r["code"], r["n"]) if r["code"] else None
        s = pool.add(r["q"], r["n"], r["R"], r["M"], code=code, random_init=r["random_init"], seed=r["seed"],
                     tabu=r["tabu"], kick=r["kick"], stall=r["stall"], cand=cand, trace=1,
                     trace_cap=r["iters"], wide=True)
        for k, v in prm.items():
            if k != "cluster":
                pool.set_slot_param(s, k, v)
        pool.run(r["iters"])
        o = Oracle(r["q"], r["n"], r["R"], r["M"], seed=r["seed"], tabu=r["tabu"], kick=r["kick"],
                   stall=r["stall"], cand=cand, wide=True)
        o.init(code, random_init=r["random_init"])
        otr = o.run(r["iters"], trace=True)
        gtr = pool.trace(s)
        st = pool.status(s)
        ok = st["status"] == 0 and gtr.tobytes() == otr.tobytes() and (pool.cnt(s) == o.cnt()).all()
        ok = ok and (st["ul_valid"], st["ul_n"]) == o.ul_state()
        if not ok:
            k, g1, o1 = first_diff(gtr, otr)
            bad.append(dict(cell=(r["q"], r["n"], r["R"], r["M"], r["seed"]), prm=prm, cand=cand, first=k,
                            status=st["status"], ul=((st["ul_valid"], st["ul_n"]), o.ul_state()),
                            gpu=None if g1 is None else g1.tolist(), orc=None if o1 is None else o1.tolist()))
        pool.close()
    assert not bad, bad[:3]


@pytest.mark.parametrize("cluster", [16, 8, 2])
def test_grid_help_matches_oracle(covlib, golden, cluster):
    """One instance whose move commits are shared with helper CTAs on the
    rest of the GPU ("grid_help"): q7 n9 R4 M1500 (tenure 20) for 300 moves,
    move by move against the oracle, then golden runs (R = 0 and 1
    included) against the reference's fingerprints and the oracle's state."""
    from oracle.pyoracle import Oracle
    from coldcase_gb300.workloads import uniform_code
    q, n, R, M = 7, 9, 4, 1500
    code = uniform_code(q, n, M, 3)
    o = Oracle(q, n, R, M, seed=3, tabu=20, threads=8)
    o.init(code)
    otr = o.run(300, trace=True)
    pool = Pool(1, cluster=cluster)
    pool.set_param("grid_help", 64)
    s = pool.add(q, n, R, M, code=code, seed=3, tabu=20, trace=1, trace_cap=300)
    for _ in range(3):
        pool.run(100)
    gtr = pool.trace(s)
    k, g1, o1 = first_diff(gtr, otr)
    assert pool.status(s)["status"] == 0
    assert len(gtr) == len(otr) and k == len(otr), (k, g1, o1)
    assert (pool.cnt(s) == o.cnt()).all() and (pool.best(s) == o.best()).all()
    pool.close()
    o.close()
    runs, _ = golden
    picked = [r for r in runs if r["R"] <= 1][:3] + [r for r in runs if r["R"] >= 2 and r["code"]][:3]
    for r in picked:
        pool = Pool(1, cluster=cluster)
        pool.set_param("grid_help", 64)
        code = code_from_text(r["code"], r["n"]) if r["code"] else None
        s = pool.add(r["q"], r["n"], r["R"], r["M"], code=code, random_init=r["random_init"], seed=r["seed"],
                     tabu=r["tabu"], kick=r["kick"], stall=r["stall"], trace=1, trace_cap=max(1, r["iters"]))
        pool.run(r["iters"])
        st = pool.status(s)
        o, otr = oracle_run(r)
        assert st["status"] == 0, (r, st)
        assert (st["best"], st["it"], st["kicks"]) == (r["ref"]["uncovered"], r["ref"]["iters"], r["ref"]["kicks"])
        assert pool.trace(s).tobytes() == otr.tobytes()
        assert (pool.cnt(s) == o.cnt()).all() and (pool.tabu(s) == o.tabu()).all()
        o.close()
        pool.close()
