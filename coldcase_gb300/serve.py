"""Serving: continuous batching of solve requests on one GPU.

A request is one covsearch2e job -- (q, n, R, M, seed, move budget), the
arguments covengine gives each chain (cov/engine/covengine:624-643) -- and
its answer is the best code found with its uncovered count.  The server
keeps the state of every admitted request resident on the device as one slot
of a Pool and runs steps:

  1. admit: waiting requests, oldest first, while a slot is free and the
     request's device bytes (cov_slot_bytes) fit in free HBM less a reserve
     (and under an optional byte budget); a request that does not fit waits
     for retirements -- later, smaller requests may pass it;
  2. advance every admitted request by up to `chunk` moves in one launch per
     cluster size, the launches side by side; each slot stops at exactly its
     own budget (its "it_limit"), so a request's result never depends on
     which others share the GPU or where step boundaries fall;
  3. retire requests whose budget is spent or whose code covers: read back
     the best code, check its uncovered count with the GPU verifier
     (cov_verify, the count of cov/verify_cov.py), free the slot.

Between steps the cluster sizes are rebalanced: while the GPU has CTAs to
spare (few requests active), the requests with the most work per move get
wider clusters.  Requests that arrive while a step runs join at the next
step.  Latency is
completion minus arrival; throughput is the moves of all requests over the
wall time.
"""
import math
import time

import numpy as np

from . import verify
from .batch import elastic_clusters, resident_ctas, size_class
from .engine import Pool, device_memory, slot_bytes
from .workloads import uniform_code


def default_cluster(q, n, R, M):
    """CTAs per request by its per-move work S' = C(n-1,R)(q-1)^R."""
    sp = math.comb(n - 1, R) * (q - 1) ** R if R <= n - 1 else 1
    if sp < 1 << 12:
        return 1
    if sp < 1 << 15:
        return 2
    if sp < 1 << 17:
        return 4
    return 8


def _work_per_move(r):
    return math.comb(r["n"] - 1, r["R"]) * (r["q"] - 1) ** r["R"] if r["R"] <= r["n"] - 1 else 1


class Server:
    def __init__(self, max_slots=256, chunk=256, reserve_bytes=8 << 30, budget_bytes=None, clusters=None,
                 verify_results=True, budget_s=120.0, elastic=True, ctas=None):
        self.pool = Pool(max_slots, cluster=1, budget_s=budget_s)
        self.max_slots = max_slots
        self.chunk = chunk
        self.reserve = reserve_bytes
        self.budget = budget_bytes
        self.clusters = clusters
        self.verify_results = verify_results
        self.waiting = []          # requests not yet admitted, in arrival order
        self.active = {}           # slot -> request
        self.done = []
        self.resident = 0          # device bytes of admitted requests
        self.moves = 0
        self.steps = 0
        self.elastic = elastic
        self.ctas = resident_ctas() if ctas is None else ctas

    def _cluster(self, r):
        if isinstance(self.clusters, dict):
            c = self.clusters.get(size_class(r["q"], r["n"], r["R"], r["M"]))
            if c:
                return c
        elif callable(self.clusters):
            return self.clusters(r["q"], r["n"], r["R"], r["M"])
        return default_cluster(r["q"], r["n"], r["R"], r["M"])

    def submit(self, req, now=None):
        req = dict(req)
        req.setdefault("arrival", now if now is not None else time.monotonic())
        req["bytes"] = slot_bytes(req["q"], req["n"], req["R"], req["M"], tabu=req.get("tabu", 0),
                                  wide=req.get("wide", False))
        if req["bytes"] == 0:
            raise ValueError("request outside the engine's domain: %r" % (req,))
        self.waiting.append(req)

    def _fits(self, req, free):
        if len(self.active) >= self.max_slots:
            return False
        if self.budget is not None and self.resident + req["bytes"] > self.budget:
            return False
        return req["bytes"] + self.reserve <= free

    def admit(self, now):
        if not self.waiting or len(self.active) >= self.max_slots:
            return 0
        free, _ = device_memory()
        n = 0
        keep = []
        for r in self.waiting:
            if self._fits(r, free):
                code = r.get("code")
                if code is None:
                    code = uniform_code(r["q"], r["n"], r["M"], r["seed"])
                s = self.pool.add(r["q"], r["n"], r["R"], r["M"], code=code, seed=r["seed"],
                                  tabu=r.get("tabu", 0), wide=r.get("wide", False))
                r["cluster"] = self._cluster(r)
                self.pool.set_slot_param(s, "cluster", r["cluster"])
                r["cur_cluster"] = r["cluster"]
                self.pool.set_slot_param(s, "it_limit", r["moves"])
                r["admitted"] = now
                r["slot"] = s
                self.active[s] = r
                self.resident += r["bytes"]
                free -= r["bytes"]
                n += 1
            else:
                keep.append(r)
        self.waiting = keep
        return n

    def _rebalance(self):
        """Elastic cluster sizes: start from each request's own size; while
        the GPU has CTAs to spare, double the cluster of the request with
        the most work per move (up to 16).  Cluster size never changes a
        trajectory, only how fast each request advances."""
        base = {s: r["cluster"] for s, r in self.active.items()}
        want = elastic_clusters(base, {s: _work_per_move(r) for s, r in self.active.items()}, self.ctas) \
            if self.elastic else base
        for s, c in want.items():
            if self.active[s].get("cur_cluster") != c:
                self.pool.set_slot_param(s, "cluster", c)
                self.active[s]["cur_cluster"] = c

    def step(self):
        """One launch over every admitted request; retire the finished."""
        if not self.active:
            return []
        self._rebalance()
        self.pool.run(self.chunk)
        self.steps += 1
        st = self.pool.status_all(self.max_slots)
        out = []
        now = time.monotonic()
        for s in list(self.active):
            r = self.active[s]
            d = st[s]
            if d["status"] != 0:
                raise RuntimeError("request %r: engine status %d" % (r.get("id"), d["status"]))
            if d["it"] >= r["moves"] or d["finished"]:
                best = self.pool.best(s)
                res = dict(uncovered=int(d["best"]), iters=int(d["it"]), kicks=int(d["kicks"]))
                if self.verify_results:
                    unc, _ = verify.verify(best, r["n"], r["q"], r["R"], want_witness=False)
                    if unc != res["uncovered"]:
                        raise RuntimeError("request %r: verifier counts %d uncovered, engine %d"
                                           % (r.get("id"), unc, res["uncovered"]))
                    res["verified"] = True
                r["result"] = res
                r["best"] = best
                r["done"] = now
                self.moves += res["iters"]
                self.pool.remove(s)
                del self.active[s]
                self.resident -= r["bytes"]
                self.done.append(r)
                out.append(r)
        return out

    def serve(self, requests, t0=None, time_limit=None):
        """Open loop: each request is submitted at t0 + its 'arrival' offset
        (seconds); returns when all are done (or the time limit passes)."""
        pending = sorted(requests, key=lambda r: r["arrival"])
        t0 = time.monotonic() if t0 is None else t0
        i = 0
        while i < len(pending) or self.waiting or self.active:
            now = time.monotonic()
            if time_limit is not None and now - t0 > time_limit:
                break
            while i < len(pending) and t0 + pending[i]["arrival"] <= now:
                r = dict(pending[i])
                r["arrival"] = t0 + pending[i]["arrival"]
                self.submit(r)
                i += 1
            self.admit(now)
            if self.active:
                self.step()
            elif i < len(pending):
                time.sleep(max(0.0, min(0.01, t0 + pending[i]["arrival"] - time.monotonic())))
            elif self.waiting:
                raise RuntimeError("request needs more device memory than the server may use: %r"
                                   % ({k: self.waiting[0][k] for k in ("q", "n", "R", "M", "bytes")},))
        wall = time.monotonic() - t0
        return self.report(wall)

    def report(self, wall):
        lat = np.array([r["done"] - r["arrival"] for r in self.done]) if self.done else np.zeros(0)
        return dict(requests=len(self.done), moves=int(self.moves), wall_s=wall,
                    moves_per_s=self.moves / wall if wall > 0 else 0.0,
                    p50_s=float(np.percentile(lat, 50)) if lat.size else None,
                    p99_s=float(np.percentile(lat, 99)) if lat.size else None,
                    steps=self.steps, chunk=self.chunk)

    def close(self):
        self.pool.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def main(argv=None):
    """Open-loop sweep: python -m coldcase_gb300.serve --lam 10 50 100 500"""
    import argparse
    import json
    from .batch import tune_batch
    from .workloads import serve_requests
    ap = argparse.ArgumentParser(description="continuous-batching solve server, Poisson load sweep")
    ap.add_argument("--lam", type=float, nargs="+", default=[10.0, 50.0, 100.0, 500.0])
    ap.add_argument("--requests", type=int, default=100)
    ap.add_argument("--chunk", type=int, default=256)
    ap.add_argument("--seed", type=int, default=2027)
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--no-elastic", action="store_true")
    a = ap.parse_args(argv)
    plan = None
    if not a.no_tune:
        plan, _, _ = tune_batch(serve_requests(a.requests, lam=a.lam[0], seed=a.seed))
    for lam in a.lam:
        reqs = serve_requests(a.requests, lam=lam, seed=a.seed)
        with Server(chunk=a.chunk, clusters=plan, elastic=not a.no_elastic) as srv:
            rep = srv.serve(reqs)
        rep["lam_per_s"] = lam
        print(json.dumps(rep), flush=True)


if __name__ == "__main__":
    main()
