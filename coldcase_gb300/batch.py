"""Batched heterogeneous instances and the cluster-size autotuner.

A Batch advances many independent covsearch2e searches of uneven
(q, n, R, M) together: every instance is one slot of a single Pool, each slot
stops at its own move budget (the per-slot "it_limit"), and a whole batch is
one graph launch in which the slots of each cluster size form one persistent
kernel, the kernels side by side.  This is the GPU form of running one
`covsearch2e --iters K` process per cell (cov/engine/covsearch2e.c:1304-1580)
or one chain per block (chain_run, cov/gemm2/chainsolve.cu:370-375).

The cluster size -- how many CTAs share one instance's commit, sphere walks
and list passes -- is the schedule knob.  Larger clusters cut an instance's
per-move latency but occupy more SMs.  Tuner measures the per-move latency
of each size class at every cluster size on a short sample run, then picks
per class the sizes that minimise the estimated batch time:
    max(critical path, total CTA time / resident CTAs),
starting from 1 CTA per instance and widening the class on the critical
path while the estimate improves.  Cluster size never changes a trajectory,
so tuning changes only speed.
"""
import json
import math
import os
import time

import numpy as np

from .engine import Pool
from .workloads import uniform_code

CLUSTERS = (1, 2, 4, 8, 16)


def resident_ctas():
    """Engine CTAs resident at once: one per SM (an engine CTA's shared
    memory fills an SM), so the current device's SM count."""
    try:
        import torch
        if torch.cuda.is_available():
            return int(torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count)
    except Exception:
        pass
    return 152      # GB300 (planning only; nothing runs without a device)


def size_class(q, n, R, M):
    """Instances whose per-move work is alike: S' = C(n-1,R)(q-1)^R patterns
    per commit and C(n,R)(q-1)^R words per sphere, by powers of two."""
    sp = math.comb(n - 1, R) * (q - 1) ** R if R <= n - 1 else 1
    return "s%02d" % int(math.log2(max(1, sp)))


def _cache_path():
    base = os.environ.get("COLDCASE_GB300_CACHE") or os.path.join(os.path.expanduser("~"), ".cache",
                                                                  "coldcase_gb300")
    return os.path.join(base, "tune.json")


def _device_key():
    try:
        import torch
        if torch.cuda.is_available():
            p = torch.cuda.get_device_properties(0)
            return "%s/%d" % (p.name, p.multi_processor_count)
    except Exception:
        pass
    return "device0"


class Tuner:
    """Per-move latency of each size class at each cluster size, measured on
    sample instances and cached per device."""

    def __init__(self, moves=120, warm=30, sample=2, clusters=CLUSTERS, cache=True):
        self.moves, self.warm, self.sample = moves, warm, sample
        self.clusters = tuple(clusters)
        self.cache = cache
        self.table = {}
        self.path = _cache_path()
        self.dev = _device_key()
        if cache and os.path.exists(self.path):
            try:
                with open(self.path) as f:
                    self.table = json.load(f).get(self.dev, {})
            except (OSError, ValueError):
                self.table = {}

    def _save(self):
        """Best effort: the cache only saves re-measuring."""
        if not self.cache:
            return
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            data = {}
            if os.path.exists(self.path):
                try:
                    with open(self.path) as f:
                        data = json.load(f)
                except (OSError, ValueError):
                    data = {}
            data[self.dev] = self.table
            tmp = "%s.%d.tmp" % (self.path, os.getpid())
            with open(tmp, "w") as f:
                json.dump(data, f, indent=1, sort_keys=True)
            os.replace(tmp, self.path)
        except OSError:
            pass

    def measure(self, key, specs):
        """Seconds per move of class `key` at every cluster size (sample of
        `specs`, all advancing together as in the batch)."""
        if key in self.table:
            return {int(c): v for c, v in self.table[key].items()}
        sample = specs[: self.sample]
        lat = {}
        for c in self.clusters:
            pool = Pool(len(sample), cluster=c, budget_s=60.0)
            try:
                for sp in sample:
                    pool.add(sp["q"], sp["n"], sp["R"], sp["M"], code=uniform_code(sp["q"], sp["n"], sp["M"],
                                                                                    sp["seed"]),
                             seed=sp["seed"], tabu=sp.get("tabu", 0), wide=sp.get("wide", False))
                pool.run(self.warm)
                t0 = time.perf_counter()
                pool.run(self.moves)
                lat[c] = (time.perf_counter() - t0) / self.moves
            finally:
                pool.close()
        self.table[key] = {str(c): v for c, v in lat.items()}
        self._save()
        return lat

    @staticmethod
    def plan(classes, budget, resident=None):
        """classes: {key: (count, {cluster: seconds per move})}; budget: moves
        per instance.  Returns ({key: cluster}, estimated seconds)."""
        if resident is None:
            resident = resident_ctas()
        choice = {k: min(lat) for k, (cnt, lat) in classes.items()}

        def estimate(ch):
            cp = max(classes[k][1][ch[k]] * budget for k in ch)
            work = sum(classes[k][0] * ch[k] * classes[k][1][ch[k]] * budget for k in ch)
            return max(cp, work / resident)

        best = estimate(choice)
        while True:
            crit = max(choice, key=lambda k: classes[k][1][choice[k]])
            wider = [c for c in sorted(classes[crit][1]) if c > choice[crit]]
            if not wider:
                break
            trial = dict(choice)
            trial[crit] = wider[0]
            t = estimate(trial)
            if t >= best:
                break
            choice, best = trial, t
        return choice, best


def elastic_clusters(base, work, ctas=None):
    """Cluster size per instance: its base size, doubled round by round for
    the instances with the most work per move while the total stays within
    `ctas` resident CTAs (default: one per SM; at most 16 per instance)."""
    if ctas is None:
        ctas = resident_ctas()
    want = dict(base)
    used = sum(want.values())
    order = sorted(want, key=lambda s: -work[s])
    grown = True
    while grown:
        grown = False
        for s in order:
            c = want[s]
            if c < 16 and used + c <= ctas:
                want[s] = 2 * c
                used += c
                grown = True
    return want


def work_per_move(q, n, R):
    """S' = C(n-1,R)(q-1)^R, the patterns of one commit."""
    return math.comb(n - 1, R) * (q - 1) ** R if R <= n - 1 else 1


class Batch:
    """Many instances in one pool; each runs exactly its own move budget.

    specs: dicts with q, n, R, M, seed, moves and optionally tabu, code, wide.
    clusters: {size class: cluster size} (e.g. from Tuner.plan) or an int.
    """

    def __init__(self, specs, clusters=1, budget_s=600.0):
        self.specs = list(specs)
        self.pool = Pool(len(self.specs), cluster=1, budget_s=budget_s)
        self.slots = []
        self.cluster_of = []
        for sp in self.specs:
            code = sp.get("code")
            if code is None:
                code = uniform_code(sp["q"], sp["n"], sp["M"], sp["seed"])
            s = self.pool.add(sp["q"], sp["n"], sp["R"], sp["M"], code=code, seed=sp["seed"],
                              tabu=sp.get("tabu", 0), wide=sp.get("wide", False))
            c = clusters if isinstance(clusters, int) else clusters.get(size_class(sp["q"], sp["n"], sp["R"],
                                                                                     sp["M"]), 1)
            self.pool.set_slot_param(s, "cluster", c)
            self.pool.set_slot_param(s, "it_limit", sp["moves"])
            self.slots.append(s)
            self.cluster_of.append(c)
        self.max_moves = max(sp["moves"] for sp in self.specs) if self.specs else 0

    def run_async(self, graph=True):
        """The whole batch as one launch per cluster size (one graph)."""
        if graph:
            self.pool.graph_run(self.max_moves, 1)
        else:
            self.pool.run_async(self.max_moves)

    def run(self, graph=True, segment=None):
        """Run every instance to its budget.  With `segment` moves, the batch
        runs in launches of that many moves and, between them, the clusters
        of the instances still running are widened while SMs are spare
        (elastic_clusters) -- small cells finish early and their SMs go to
        the large ones."""
        if not segment:
            self.run_async(graph)
            self.pool.sync()
            return
        base = dict(zip(self.slots, self.cluster_of))
        cur = dict(base)
        work = {s: work_per_move(sp["q"], sp["n"], sp["R"]) for s, sp in zip(self.slots, self.specs)}
        while True:
            st = self.pool.status_all(max(self.slots) + 1)
            live = [s for s, sp in zip(self.slots, self.specs)
                    if st[s]["it"] < sp["moves"] and not st[s]["finished"] and st[s]["status"] == 0]
            if not live:
                return
            want = elastic_clusters({s: base[s] for s in live}, work)
            for s in live:
                if want[s] != cur[s]:
                    self.pool.set_slot_param(s, "cluster", want[s])
                    cur[s] = want[s]
            self.pool.run(segment)

    def results(self):
        st = self.pool.status_all(max(self.slots) + 1 if self.slots else 0)
        out = []
        for sp, s in zip(self.specs, self.slots):
            d = st[s]
            out.append(dict(uncovered=d["best"], iters=d["it"], kicks=d["kicks"], status=d["status"],
                            finished=d["finished"]))
        return out

    def best(self, i):
        return self.pool.best(self.slots[i])

    def close(self):
        self.pool.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def tune_batch(specs, tuner=None):
    """Cluster size per size class for this batch: (plan, estimate, table)."""
    tuner = tuner or Tuner()
    groups = {}
    for sp in specs:
        groups.setdefault(size_class(sp["q"], sp["n"], sp["R"], sp["M"]), []).append(sp)
    classes = {}
    for key, members in groups.items():
        classes[key] = (len(members), tuner.measure(key, members))
    budget = max(sp["moves"] for sp in specs)
    choice, est = Tuner.plan(classes, budget)
    return choice, est, classes
