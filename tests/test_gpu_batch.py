"""Batched uneven instances and serving, against the oracle.

Every instance of a batch (one pool, slots of several cluster sizes, each
slot stopped by its own move budget) must follow exactly the trajectory the
oracle follows for that instance alone: same move records, best code and
counts.  A served request must give the same answer alone and in a mix.
"""
import numpy as np
import pytest

from coldcase_gb300.batch import Batch, size_class
from coldcase_gb300.engine import Pool
from coldcase_gb300.serve import Server
from coldcase_gb300.workloads import uniform_code

pytestmark = pytest.mark.gpu

CELLS = [  # q, n, R, M, moves, tabu
    (4, 6, 1, 420, 300, 10),
    (5, 6, 2, 90, 700, 0),
    (6, 6, 3, 18, 900, 0),
    (3, 8, 2, 60, 500, 3),
    (5, 7, 3, 40, 1200, 0),
    (7, 6, 2, 300, 450, 5),
    (4, 8, 3, 30, 800, 0),
    (6, 7, 1, 7000, 250, 0),
    # dense coverage (M = 1.3 q^n / |B|): warp-aggregated commit and the
    # uncovered-word bitmap walk
    (6, 7, 4, 14, 600, 0),
    (7, 8, 3, 570, 300, 0),
]


def oracle_of(q, n, R, M, moves, tabu, seed, wide=False):
    from oracle.pyoracle import Oracle
    o = Oracle(q, n, R, M, seed=seed, tabu=tabu, wide=wide)
    o.init(uniform_code(q, n, M, seed))
    tr = o.run(moves, trace=True)
    return o, tr


def specs():
    return [dict(q=q, n=n, R=R, M=M, moves=mv, tabu=tb, seed=1000 + i)
            for i, (q, n, R, M, mv, tb) in enumerate(CELLS)]


@pytest.mark.parametrize("graph", [True, False])
def test_batch_mixed_clusters_bit_exact(covlib, graph):
    sp = specs()
    keys = sorted({size_class(s["q"], s["n"], s["R"], s["M"]) for s in sp})
    clusters = {k: [1, 2, 4, 8][i % 4] for i, k in enumerate(keys)}
    with Batch(sp, clusters=clusters) as b:
        assert len(set(b.cluster_of)) > 1
        b.run(graph=graph)
        res = b.results()
        for i, s in enumerate(sp):
            o, tr = oracle_of(s["q"], s["n"], s["R"], s["M"], s["moves"], s["tabu"], s["seed"])
            assert res[i]["status"] == 0
            assert res[i]["iters"] == o.iters(), (s, res[i])
            assert res[i]["uncovered"] == o.best_uncovered(), (s, res[i])
            assert res[i]["kicks"] == o.kicks()
            assert (b.best(i) == o.best()).all(), s


def test_iteration_limit_across_chunks(covlib):
    """it_limit stops a slot at exactly its budget however the runs are cut."""
    q, n, R, M, moves, tabu = 5, 7, 3, 40, 1000, 0
    seed = 77
    o, otr = oracle_of(q, n, R, M, moves, tabu, seed)
    pool = Pool(2, cluster=2)
    a = pool.add(q, n, R, M, code=uniform_code(q, n, M, seed), seed=seed, tabu=tabu, trace=1, trace_cap=2000)
    b = pool.add(q, n, R, M, code=uniform_code(q, n, M, seed), seed=seed, tabu=tabu, trace=1, trace_cap=2000)
    pool.set_slot_param(a, "it_limit", moves)
    pool.set_slot_param(b, "cluster", 1)
    pool.set_slot_param(b, "it_limit", moves)
    for k in (37, 400, 1, 999, 5000):
        pool.run(k)
    for s in (a, b):
        assert pool.status(s)["it"] == min(moves, o.iters())
        assert pool.trace(s).tobytes() == otr.tobytes()
    pool.set_slot_param(a, "it_limit", -1)
    pool.run(10)
    assert pool.status(a)["it"] == pool.status(b)["it"] + 10 or pool.status(a)["finished"]
    pool.close()


def _requests():
    out = []
    for i, (q, n, R, M, mv, tb) in enumerate(CELLS):
        out.append(dict(id=i, q=q, n=n, R=R, M=M, moves=mv, tabu=tb, seed=500 + i, arrival=0.002 * i))
    return out


def test_served_result_same_alone_and_in_mix(covlib):
    """Bit-identical answers alone and under continuous batching (tolerance:
    none -- the codes, counts and iteration numbers are equal)."""
    reqs = _requests()
    mix = {}
    with Server(max_slots=4, chunk=97) as srv:
        rep = srv.serve(reqs)
        assert rep["requests"] == len(reqs)
        for r in srv.done:
            mix[r["id"]] = (r["result"], r["best"])
    for r in reqs[::3]:
        with Server(max_slots=1, chunk=1000) as alone:
            alone.serve([dict(r, arrival=0.0)])
            a = alone.done[0]
        res, best = mix[r["id"]]
        assert a["result"] == res, (r, a["result"], res)
        assert (a["best"] == best).all()
        o, _ = oracle_of(r["q"], r["n"], r["R"], r["M"], r["moves"], r["tabu"], r["seed"])
        assert res["uncovered"] == o.best_uncovered() and res["iters"] == o.iters()


def test_wide_requests_in_a_mix(covlib):
    """--wide and plain requests served together: each answer is the
    oracle's for its own flag."""
    reqs = [dict(r, wide=bool(i % 2), seed=900 + i) for i, r in enumerate(_requests())]
    with Server(max_slots=5, chunk=131) as srv:
        rep = srv.serve(reqs)
        assert rep["requests"] == len(reqs)
        done = {r["id"]: r for r in srv.done}
    for r in reqs:
        o, _ = oracle_of(r["q"], r["n"], r["R"], r["M"], r["moves"], r["tabu"], r["seed"], wide=r["wide"])
        res = done[r["id"]]["result"]
        assert res["uncovered"] == o.best_uncovered() and res["iters"] == o.iters(), (r, res)
        assert (done[r["id"]]["best"] == o.best()).all(), r


def test_admission_by_device_bytes(covlib):
    """With a byte budget for two requests, at most two are resident."""
    reqs = _requests()[:6]
    from coldcase_gb300.engine import slot_bytes
    sizes = [slot_bytes(r["q"], r["n"], r["R"], r["M"]) for r in reqs]
    budget = sorted(sizes)[-1] + sorted(sizes)[-2]
    peak = []
    with Server(max_slots=8, chunk=64, budget_bytes=budget) as srv:
        orig = srv.step

        def step():
            peak.append((len(srv.active), srv.resident))
            return orig()
        srv.step = step
        rep = srv.serve(reqs)
    assert rep["requests"] == len(reqs)
    assert max(p[1] for p in peak) <= budget
    assert max(p[0] for p in peak) >= 2


def test_batch_segmented_elastic_bit_exact(covlib):
    """Segments with clusters re-widened between them give the same results."""
    sp = specs()
    with Batch(sp, clusters=1) as b:
        b.run(segment=173)
        res = b.results()
        for i, s in enumerate(sp):
            o, tr = oracle_of(s["q"], s["n"], s["R"], s["M"], s["moves"], s["tabu"], s["seed"])
            assert res[i]["iters"] == o.iters() and res[i]["uncovered"] == o.best_uncovered(), (s, res[i])
            assert (b.best(i) == o.best()).all(), s


def test_chain_run_equals_pool_chains(covlib):
    """cov_chain_run (chain_run's arguments and buffers, rows of 16 digits)
    gives each chain exactly the trajectory of a pool slot with seed
    seed*1000003 + chain*7919."""
    import ctypes
    from coldcase_gb300 import lib as L
    q, n, R, M, nchains, iters, seed = 4, 7, 2, 40, 5, 400, 3
    rng = np.random.default_rng(11)
    codes = np.zeros((nchains, M, 16), dtype=np.uint8)
    codes[:, :, :n] = rng.integers(0, q, (nchains, M, n), dtype=np.uint8)
    best = np.zeros_like(codes)
    bu = np.zeros(nchains, np.int32)
    sv = np.zeros(nchains, np.int32)
    it = np.zeros(nchains, np.int64)
    p8 = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
    rc = covlib.cov_chain_run(q, n, R, M, nchains, iters, seed, 256, p8(codes), p8(best),
                              bu.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                              sv.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                              it.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    assert rc == 0
    assert (best[:, :, n:] == 0).all()
    for c in range(nchains):
        pool = Pool(1, cluster=1)
        s = pool.add(q, n, R, M, code=codes[c, :, :n], seed=seed * 1000003 + c * 7919)
        pool.set_slot_param(s, "it_limit", iters)
        pool.run(iters)
        st = pool.status(s)
        assert (st["best"], st["it"]) == (bu[c], it[c])
        assert sv[c] == (st["best"] == 0)
        assert (pool.best(s) == best[c, :, :n]).all()
        pool.close()
