"""The quotient search (cov/engine/symsearch.c) on the GPU.

A code invariant under the diagonal translation x -> x + 1^n is a union of
orbits {(j, e + j) : j in Z_q}; SymPool searches over the orbit
representatives e in Z_q^(n-1) with the reference's trajectory.  Each
instance is one slot of the pool; a run advances every slot in one launch
per cluster size.
"""
import ctypes

import numpy as np

from . import lib as L

DIG = "0123456789abcdefghijklmnopqrstuvwxyz"


def make_params(q, n, R, M, orbits=0, seed=12345, kick=2, stall=3000, cand=100000, trace=0, trace_cap=0):
    return L.CovSymParams(q=q, n=n, R=R, M=M, orbits=orbits, kick=kick, seed=seed, stall=stall, cand=cand,
                          trace=1 if trace else 0, trace_cap=trace_cap if trace else 0)


def orbits_of(q, n, R, M, orbits=0):
    """Orbit count, or the CovError symsearch's exit 2 / 3 corresponds to."""
    lib = L.load()
    p = make_params(q, n, R, M, orbits=orbits)
    rc = lib.cov_sym_orbits(ctypes.byref(p))
    L.check(min(rc, 0), "cov_sym_orbits")
    return rc


def expand(reps, q):
    """The q words (j, e + j) of every orbit, orbit by orbit: the code."""
    reps = np.asarray(reps, dtype=np.int64)
    j = np.arange(q, dtype=np.int64)
    words = np.concatenate([np.broadcast_to(j[None, :, None], (len(reps), q, 1)),
                            (reps[:, None, :] + j[None, :, None]) % q], axis=2)
    return words.reshape(-1, reps.shape[1] + 1).astype(np.uint8)


def format_code(reps, q):
    """symsearch's --out text (symsearch.c:250-266)."""
    return "".join(DIG[j] + "".join(DIG[(int(x) + j) % q] for x in e) + "\n" for e in reps for j in range(q))


class SymPool:
    """Quotient-search instances on one GPU (cov_sym_* in include/covgpu.h)."""

    def __init__(self, max_slots=1, cluster=1, budget_s=30.0, grid_eval=False):
        """grid_eval: with one live instance, spread each move's estimates over
        the whole GPU instead of the instance's cluster."""
        self.lib = L.load()
        h = ctypes.c_void_p()
        L.check(self.lib.cov_sym_create(int(max_slots), int(cluster), ctypes.byref(h)), "cov_sym_create")
        self.h = h
        self.meta = {}
        if budget_s:
            L.check(self.lib.cov_sym_set_budget(self.h, float(budget_s)), "cov_sym_set_budget")
        if grid_eval:
            L.check(self.lib.cov_sym_set_param(self.h, b"grid_eval", 1), "cov_sym_set_param")

    def add(self, q, n, R, M, orbits=0, seed=12345, kick=2, stall=3000, cand=100000, trace=0, trace_cap=0):
        """Create an instance; its orbits are placed greedily on the device."""
        p = make_params(q, n, R, M, orbits=orbits, seed=seed, kick=kick, stall=stall, cand=cand, trace=trace,
                        trace_cap=trace_cap)
        norb = self.lib.cov_sym_orbits(ctypes.byref(p))
        L.check(min(norb, 0), "cov_sym_orbits")
        slot = ctypes.c_int32(-1)
        L.check(self.lib.cov_sym_add(self.h, ctypes.byref(p), ctypes.byref(slot)), "cov_sym_add")
        self.meta[slot.value] = (q, n, R, M, norb)
        return slot.value

    def set_slot_param(self, slot, name, value):
        L.check(self.lib.cov_sym_set_slot_param(self.h, int(slot), name.encode(), int(value)),
                "cov_sym_set_slot_param")

    def run(self, moves):
        L.check(self.lib.cov_sym_run(self.h, int(moves)), "cov_sym_run")

    def status(self, slot):
        st = L.CovStatus()
        L.check(self.lib.cov_sym_status(self.h, int(slot), ctypes.byref(st)), "cov_sym_status")
        return {k: getattr(st, k) for k, _ in L.CovStatus._fields_ if k not in ("ul_valid", "ul_n")}

    def resume(self, slot):
        L.check(self.lib.cov_sym_resume(self.h, int(slot)), "cov_sym_resume")

    def _reps(self, fn, slot):
        q, n, R, M, norb = self.meta[slot]
        out = np.zeros((norb, n - 1), dtype=np.uint8)
        L.check(fn(self.h, int(slot), L.u8ptr(out)), fn.__name__)
        return out

    def rep(self, slot):
        return self._reps(self.lib.cov_sym_get_rep, slot)

    def best(self, slot):
        """Best representatives (orbits x (n-1) digits)."""
        return self._reps(self.lib.cov_sym_get_best, slot)

    def cnt(self, slot):
        q, n = self.meta[slot][:2]
        out = np.zeros(q ** (n - 1), dtype=np.uint16)
        L.check(self.lib.cov_sym_get_cnt(self.h, int(slot), out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16))),
                "cov_sym_get_cnt")
        return out

    def rng(self, slot):
        out = np.zeros(4, dtype=np.uint64)
        L.check(self.lib.cov_sym_get_rng(self.h, int(slot), out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))),
                "cov_sym_get_rng")
        return out

    def prof(self, slot):
        """Leader cycles per move by phase (diagnostics)."""
        out = np.zeros(9, dtype=np.uint64)
        L.check(self.lib.cov_sym_get_prof(self.h, int(slot), out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))),
                "cov_sym_get_prof")
        moves = max(1, int(out[8]))
        names = ("pick", "candidates", "sample", "estimate", "select", "commit", "orbit", "other")
        return {k: float(out[i]) / moves for i, k in enumerate(names)}, int(out[8])

    def trace(self, slot):
        n = ctypes.c_int64(0)
        L.check(self.lib.cov_sym_get_trace(self.h, int(slot), None, 0, ctypes.byref(n)), "cov_sym_get_trace")
        out = np.zeros(n.value, dtype=L.MOVE_DTYPE)
        if n.value:
            L.check(self.lib.cov_sym_get_trace(self.h, int(slot), out.ctypes.data_as(ctypes.POINTER(L.CovMoveRec)),
                                               n.value, ctypes.byref(n)), "cov_sym_get_trace")
        return out

    def remove(self, slot):
        L.check(self.lib.cov_sym_remove(self.h, int(slot)), "cov_sym_remove")
        self.meta.pop(slot, None)

    def close(self):
        if self.h:
            self.lib.cov_sym_destroy(self.h)
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
