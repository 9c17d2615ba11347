"""Parity at the configurations the benchmark numbers are measured on.

* The batched headline: 64 restarts of q7 n9 R4 M1500 (tenure 20) in one
  pool at two CTAs per restart, advanced as bench.py advances them (direct
  launches, then replays of the captured graph).  After 5000 moves every
  restart must stand exactly where the oracle stands after 5000 moves
  (tests/golden/warm_q7n9.json, made by tests/golden/make_warm.py): the
  same iteration, uncovered and best counts, RNG state, current and best
  code, tabu table and coverage-count array.  Restart 0 is also traced and
  its first 1000 move records compared with a live oracle run.
* The served form on its largest request shape (q6 n10 R4, M from the
  request generator) and the batched uneven form on a dense cell with
  q^n >= 2e7 (q7 n9 R3 M2691), 200+ moves each, against the oracle.

Integer state throughout: the tolerance is none.
"""
import hashlib
import json
import math
import os

import numpy as np
import pytest

from coldcase_gb300.batch import Batch, size_class
from coldcase_gb300.engine import Pool
from coldcase_gb300.serve import Server
from coldcase_gb300.workloads import ball_volume, instance_seed, uniform_code

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
Q, N, R, M, TENURE = 7, 9, 4, 1500, 20


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def warm():
    with open(os.path.join(HERE, "golden", "warm_q7n9.json")) as f:
        meta = json.load(f)
    codes = np.load(os.path.join(HERE, "golden", "warm_q7n9.npz"))["codes"]
    return meta, codes


def test_batched_headline_restarts_reach_the_oracle_state(covlib):
    from oracle.pyoracle import Oracle
    meta, codes = warm()
    recs = meta["restarts"]
    assert (meta["q"], meta["n"], meta["R"], meta["M"], meta["tenure"]) == (Q, N, R, M, TENURE)
    steps = meta["moves"] // 1000
    assert steps * 1000 == meta["moves"] and steps >= 3
    pool = Pool(len(recs), cluster=2, budget_s=120.0)
    slots = []
    for r in recs:
        seed = instance_seed(meta["base_seed"], r["restart"])
        assert seed == r["seed"]
        tr = r["restart"] == 0
        slots.append(pool.add(Q, N, R, M, code=uniform_code(Q, N, M, seed), seed=seed, tabu=TENURE,
                              trace=1 if tr else 0, trace_cap=1000 if tr else 0))
    for k in range(steps):
        if k < 2:
            pool.run(1000)
        else:
            pool.graph_run(1000, 1)
            pool.sync()
    o = Oracle(Q, N, R, M, seed=recs[0]["seed"], tabu=TENURE, threads=threads())
    o.init(uniform_code(Q, N, M, recs[0]["seed"]))
    otr = o.run(1000, trace=True)
    o.close()
    gtr = pool.trace(slots[0])
    assert len(gtr) == 1000 and gtr.tobytes() == otr.tobytes()
    bad = []
    for r, s in zip(recs, slots):
        st = pool.status(s)
        got = dict(it=st["it"], unc=st["uncovered"], best=st["best"], kicks=st["kicks"],
                   rng=[int(x) for x in pool.rng(s)], code_sha=sha(pool.code(s)), best_sha=sha(pool.best(s)),
                   tabu_sha=sha(pool.tabu(s)), cnt_sha=sha(pool.cnt(s)))
        want = {k: r[k] for k in got}
        if st["status"] != 0 or got != want:
            bad.append(dict(restart=r["restart"], status=st["status"],
                            diff={k: (got[k], want[k]) for k in got if got[k] != want[k]}))
        if r["restart"] < len(codes):
            assert (pool.code(s) == codes[r["restart"]]).all()
    pool.close()
    assert not bad, bad[:3]


def _oracle(q, n, R_, M_, seed, moves, tabu=0):
    from oracle.pyoracle import Oracle
    o = Oracle(q, n, R_, M_, seed=seed, tabu=tabu, threads=threads())
    o.init(uniform_code(q, n, M_, seed))
    o.run(moves)
    return o


def test_served_largest_request_shape(covlib):
    """q6 n10 R4 with M = ceil(1.3 q^n / |B|), 240 moves, served alone and in
    a mix with smaller requests arriving while it runs."""
    q, n, R_ = 6, 10, 4
    M_ = math.ceil(1.3 * q ** n / ball_volume(q, n, R_))
    big = dict(id=0, q=q, n=n, R=R_, M=M_, moves=240, seed=instance_seed(2027, 0), arrival=0.0)
    small = [dict(id=1 + i, q=5, n=7, R=2, M=math.ceil(1.3 * 5 ** 7 / ball_volume(5, 7, 2)), moves=300,
                  seed=instance_seed(2027, 1 + i), arrival=0.001 * (i + 1)) for i in range(3)]
    o = _oracle(q, n, R_, M_, big["seed"], big["moves"])
    for reqs in ([big], [big] + small):
        with Server(max_slots=8, chunk=64) as srv:
            srv.serve(reqs)
            done = {r["id"]: r for r in srv.done}
        r = done[0]
        assert r["result"]["iters"] == o.iters()
        assert r["result"]["uncovered"] == o.best_uncovered()
        assert r["result"]["kicks"] == o.kicks()
        assert (r["best"] == o.best()).all()
        for s in small[: len(reqs) - 1]:
            os_ = _oracle(s["q"], s["n"], s["R"], s["M"], s["seed"], s["moves"])
            assert done[s["id"]]["result"]["uncovered"] == os_.best_uncovered()
            assert (done[s["id"]]["best"] == os_.best()).all()
            os_.close()
    o.close()


def test_batched_dense_large_cell(covlib):
    """A dense uneven cell with q^n >= 2e7 (q7 n9 R3, M = ceil(1.3 q^n/|B|) =
    2691, the warp-aggregated commit and the uncovered-word bitmap) beside
    two others in one batch, 220 moves, at its planned cluster sizes."""
    q, n, R_ = 7, 9, 3
    M_ = math.ceil(1.3 * q ** n / ball_volume(q, n, R_))
    assert q ** n >= 2e7 and M_ == 2691
    cells = [dict(q=q, n=n, R=R_, M=M_, moves=220, seed=instance_seed(2026, 0)),
             dict(q=8, n=8, R=2, M=math.ceil(1.3 * 8 ** 8 / ball_volume(8, 8, 2)), moves=260,
                  seed=instance_seed(2026, 1)),
             dict(q=6, n=9, R=4, M=math.ceil(1.3 * 6 ** 9 / ball_volume(6, 9, 4)), moves=200,
                  seed=instance_seed(2026, 2))]
    keys = [size_class(c["q"], c["n"], c["R"], c["M"]) for c in cells]
    for clusters in (1, dict(zip(keys, (4, 2, 8)))):
        with Batch(cells, clusters=clusters) as b:
            b.run(graph=True, segment=64)
            res = b.results()
            for i, c in enumerate(cells):
                o = _oracle(c["q"], c["n"], c["R"], c["M"], c["seed"], c["moves"])
                assert res[i]["status"] == 0
                assert res[i]["iters"] == o.iters(), (c, res[i])
                assert res[i]["uncovered"] == o.best_uncovered(), (c, res[i])
                assert (b.best(i) == o.best()).all(), c
                o.close()
