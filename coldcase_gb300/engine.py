"""Host side of the tabu engine: the covsearch2e search behind the C ABI.

Search is one instance (what one `covsearch2e --preset p5b` process does,
cov/engine/covsearch2e.c:1023-1621); Pool holds many instances that advance
together in one launch (batched restarts, uneven cells, served requests).
"""
import ctypes

import numpy as np

from . import lib as L

DEFAULTS = dict(seed=12345, tabu=0, kick=2, stall=5000, cand=100000)


SA_DEFAULTS = (0.6, 0.999999, 0.02)     # --t0 --cool --tmin (covsearch2e.c:1035)


def make_params(q, n, R, M, seed=12345, tabu=0, kick=2, stall=5000, cand=100000,
                trace=0, trace_cap=0, wide=False, fix0=False, sa=None, noise=0):
    """sa: None, or (t0, cool, tmin) for --sa; noise: --noise PERMILLE."""
    t0, cool, tmin = SA_DEFAULTS if sa is None else sa
    return L.CovParams(q=q, n=n, R=R, M=M, seed=seed, tabu=tabu, kick=kick, cand=cand,
                       trace=1 if trace else 0, stall=stall, trace_cap=trace_cap if trace else 0,
                       wide=1 if wide else 0, fix0=1 if fix0 else 0, sa=0 if sa is None else 1,
                       noise=int(noise), t0=float(t0), cool=float(cool), tmin=float(tmin))


def slot_bytes(q, n, R, M, **kw):
    lib = L.load()
    p = make_params(q, n, R, M, **kw)
    return int(lib.cov_slot_bytes(ctypes.byref(p)))


def device_memory():
    """(free, total) bytes of the current device."""
    lib = L.load()
    f, t = ctypes.c_int64(), ctypes.c_int64()
    L.check(lib.cov_device_memory(ctypes.byref(f), ctypes.byref(t)), "cov_device_memory")
    return f.value, t.value


class Pool:
    """Up to `max_slots` independent searches, one thread-block cluster of
    `cluster` CTAs each, advanced together by run()."""

    def __init__(self, max_slots, cluster=1, budget_s=30.0):
        self.lib = L.load()
        h = ctypes.c_void_p()
        L.check(self.lib.cov_pool_create(int(max_slots), int(cluster), ctypes.byref(h)), "cov_pool_create")
        self.h = h
        self.cluster = cluster
        self.meta = {}
        L.check(self.lib.cov_pool_set_budget(self.h, float(budget_s)), "cov_pool_set_budget")

    def set_param(self, name, value):
        L.check(self.lib.cov_pool_set_param(self.h, name.encode(), int(value)), "cov_pool_set_param")

    def set_slot_param(self, slot, name, value):
        """Per-slot setting: "cluster", "neg_cluster_pairs" or "it_limit"."""
        L.check(self.lib.cov_pool_set_slot_param(self.h, int(slot), name.encode(), int(value)),
                "cov_pool_set_slot_param")

    def add(self, q, n, R, M, code=None, random_init=False, seed=12345, tabu=0, kick=2,
            stall=5000, cand=100000, trace=0, trace_cap=0, wide=False, fix0=False, sa=None, noise=0):
        """Create an instance from `code` (m x n digits; m may be <, = or > M).
        `wide`, `fix0` and `noise` are covsearch2e's --wide, --fix0 and
        --noise; `sa` = (t0, cool, tmin) is --sa --t0 --cool --tmin."""
        p = make_params(q, n, R, M, seed=seed, tabu=tabu, kick=kick, stall=stall, cand=cand,
                        trace=trace, trace_cap=trace_cap, wide=wide, fix0=fix0, sa=sa, noise=noise)
        if code is None:
            arr = np.zeros((0, n), dtype=np.uint8)
        else:
            arr = L.as_code(code, q, n)
        slot = ctypes.c_int32(-1)
        ptr = L.u8ptr(arr) if arr.size else None
        L.check(self.lib.cov_pool_add(self.h, ctypes.byref(p), ptr, int(arr.shape[0]),
                                      1 if random_init else 0, ctypes.byref(slot)), "cov_pool_add")
        self.meta[slot.value] = (q, n, R, M)
        return slot.value

    def load(self, slot, code=None, seed=12345, random_init=False):
        """Re-initialise a slot with a new seed and code, keeping its storage."""
        q, n, R, M = self.meta[slot]
        arr = np.zeros((0, n), dtype=np.uint8) if code is None else L.as_code(code, q, n)
        L.check(self.lib.cov_pool_load(self.h, int(slot), int(seed), L.u8ptr(arr) if arr.size else None,
                                       int(arr.shape[0]), 1 if random_init else 0), "cov_pool_load")

    def run(self, moves, target=-1):
        L.check(self.lib.cov_pool_run(self.h, int(moves), int(target)), "cov_pool_run")

    def run_async(self, moves, target=-1):
        L.check(self.lib.cov_pool_run_async(self.h, int(moves), int(target)), "cov_pool_run_async")

    def graph_run(self, moves, steps, target=-1):
        L.check(self.lib.cov_pool_graph_run(self.h, int(moves), int(target), int(steps)), "cov_pool_graph_run")

    def sync(self):
        L.check(self.lib.cov_pool_sync(self.h), "cov_pool_sync")

    def set_stream(self, stream_handle):
        """Queue work on an external cudaStream_t (int handle, e.g.
        torch.cuda.Stream().cuda_stream); None returns to the pool's own."""
        L.check(self.lib.cov_pool_set_stream(self.h, ctypes.c_void_p(stream_handle) if stream_handle else None),
                "cov_pool_set_stream")

    def status_all(self, n):
        arr = (L.CovStatus * n)()
        L.check(self.lib.cov_pool_status_all(self.h, arr, int(n)), "cov_pool_status_all")
        return [{k: getattr(a, k) for k, _ in L.CovStatus._fields_} for a in arr]

    def status(self, slot):
        st = L.CovStatus()
        L.check(self.lib.cov_pool_status(self.h, int(slot), ctypes.byref(st)), "cov_pool_status")
        return {k: getattr(st, k) for k, _ in L.CovStatus._fields_}

    def _digits(self, fn, slot):
        q, n, R, M = self.meta[slot]
        out = np.zeros((M, n), dtype=np.uint8)
        L.check(fn(self.h, int(slot), L.u8ptr(out)), fn.__name__)
        return out

    def code(self, slot):
        return self._digits(self.lib.cov_pool_get_code, slot)

    def best(self, slot):
        return self._digits(self.lib.cov_pool_get_best, slot)

    def cnt(self, slot):
        q, n, R, M = self.meta[slot]
        out = np.zeros(q ** n, dtype=np.uint16)
        L.check(self.lib.cov_pool_get_cnt(self.h, int(slot),
                                          out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16))),
                "cov_pool_get_cnt")
        return out

    def private(self, slot):
        q, n, R, M = self.meta[slot]
        out = np.zeros((M, n + 1), dtype=np.int32)
        L.check(self.lib.cov_pool_get_private(self.h, int(slot), out.ctypes.data_as(L._PI32)),
                "cov_pool_get_private")
        return out

    def tabu(self, slot):
        q, n, R, M = self.meta[slot]
        out = np.zeros(M * n * q, dtype=np.int32)
        L.check(self.lib.cov_pool_get_tabu(self.h, int(slot), out.ctypes.data_as(L._PI32)),
                "cov_pool_get_tabu")
        return out

    def rng(self, slot):
        out = np.zeros(4, dtype=np.uint64)
        L.check(self.lib.cov_pool_get_rng(self.h, int(slot),
                                          out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))),
                "cov_pool_get_rng")
        return out

    PROF_NAMES = ("pick", "candidates", "entering", "select", "move", "finish", "compact", "other")

    def prof(self, slot):
        """Leader phase cycle counts and the list-pair counter."""
        out = np.zeros(25, dtype=np.uint64)
        L.check(self.lib.cov_pool_get_prof(self.h, int(slot),
                                           out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))),
                "cov_pool_get_prof")
        d = {k: int(v) for k, v in zip(self.PROF_NAMES, out[:8])}
        for k in range(8, 20):
            d["sub%d" % k] = int(out[k])
        d["sum_ncw"], d["sum_ul_n"], d["planned_moves"] = int(out[20]), int(out[21]), int(out[22])
        d["ul_pairs"] = int(out[24])
        return d

    def trace(self, slot):
        n = ctypes.c_int64(0)
        L.check(self.lib.cov_pool_get_trace(self.h, int(slot), None, 0, ctypes.byref(n)), "cov_pool_get_trace")
        out = np.zeros(n.value, dtype=L.MOVE_DTYPE)
        if n.value:
            L.check(self.lib.cov_pool_get_trace(self.h, int(slot),
                                                out.ctypes.data_as(ctypes.POINTER(L.CovMoveRec)),
                                                n.value, ctypes.byref(n)), "cov_pool_get_trace")
        return out

    def set_budget(self, seconds):
        """Wall-clock budget of each launch; a slot that reaches it stops
        between moves with status COV_ETIMEOUT (see resume)."""
        L.check(self.lib.cov_pool_set_budget(self.h, float(seconds)), "cov_pool_set_budget")

    def resume(self, slot):
        """Clear a deadline stop so the slot continues its trajectory."""
        L.check(self.lib.cov_pool_resume(self.h, int(slot)), "cov_pool_resume")

    def remove(self, slot):
        L.check(self.lib.cov_pool_remove(self.h, int(slot)), "cov_pool_remove")
        self.meta.pop(slot, None)

    def close(self):
        if self.h:
            self.lib.cov_pool_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Search:
    """One covsearch2e instance on the GPU (a pool with a single slot).

    Parameters are covsearch2e's: -q -n -R -M -s --tabu --kick --stall --cand --wide --fix0,
    --noise, and --sa --t0 --cool --tmin as sa=(t0, cool, tmin).
    """

    def __init__(self, q, n, R, M, seed=12345, tabu=0, kick=2, stall=5000, cand=100000,
                 cluster=8, trace=0, trace_cap=0, budget_s=30.0, wide=False, fix0=False, sa=None, noise=0):
        self.q, self.n, self.R, self.M = q, n, R, M
        self.kw = dict(seed=seed, tabu=tabu, kick=kick, stall=stall, cand=cand,
                       trace=trace, trace_cap=trace_cap, wide=wide, fix0=fix0, sa=sa, noise=noise)
        self.pool = Pool(1, cluster=cluster, budget_s=budget_s)
        self.slot = None

    def load(self, code=None, random_init=False):
        """Initial code as covsearch2e builds it from --in (see Pool.add)."""
        self.slot = self.pool.add(self.q, self.n, self.R, self.M, code=code,
                                  random_init=random_init, **self.kw)
        return self.status()["uncovered"]

    def run(self, moves, target=-1):
        self.pool.run(moves, target)
        return self.status()

    def status(self):
        return self.pool.status(self.slot)

    def code(self):
        return self.pool.code(self.slot)

    def best(self):
        return self.pool.best(self.slot)

    def cnt(self):
        return self.pool.cnt(self.slot)

    def trace(self):
        return self.pool.trace(self.slot)

    def close(self):
        self.pool.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
