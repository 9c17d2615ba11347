"""GPU verifier with the reference verifiers' interface.

verify(code, n, q, R) -> (n_uncovered, witnesses) mirrors
cov/verify_cov.py:109-152 / :169-230; mindist() mirrors the run_mindist
report of cov/verify_independent.py:144-186 (per-word distance, histogram,
covering radius); dilate() the covering decision of run_dilate (:128-141);
count() the coverage multiplicity cnt[] of covsearch2e.c:958-967.
All of it runs in libcovgpu.so; there is no CPU path.
"""
import ctypes

import numpy as np

from . import lib as L


def _code(code, q, n):
    a = L.as_code(code, q, n) if len(code) else np.zeros((0, n), dtype=np.uint8)
    return a


def mindist(code, q, n, want_dist=True):
    """(dist uint8[q^n] or None, hist int64[n+2], covering radius)."""
    lib = L.load()
    a = _code(code, q, n)
    dist = np.zeros(q ** n, dtype=np.uint8) if want_dist else None
    hist = np.zeros(n + 2, dtype=np.int64)
    rad = ctypes.c_int32(0)
    L.check(lib.cov_mindist(q, n, L.u8ptr(a) if a.size else None, int(a.shape[0]),
                            L.u8ptr(dist) if dist is not None else None,
                            hist.ctypes.data_as(L._PI64), ctypes.byref(rad)), "cov_mindist")
    return dist, hist, rad.value


def verify(code, n, q, R, want_witness=True, max_witness=5):
    """Exact uncovered count and the first uncovered words (index order)."""
    if not want_witness:
        lib = L.load()
        a = _code(code, q, n)
        u = ctypes.c_int64(0)
        L.check(lib.cov_verify(q, n, R, L.u8ptr(a) if a.size else None, int(a.shape[0]),
                               ctypes.byref(u)), "cov_verify")
        return int(u.value), []
    dist, hist, _ = mindist(code, q, n)
    unc = int(hist[R + 1:].sum()) if R + 1 <= n + 1 else 0
    wit = []
    if unc:
        idx = np.flatnonzero(dist > R)[:max_witness]
        pw = q ** np.arange(n - 1, -1, -1, dtype=np.int64)
        for x in idx.tolist():
            wit.append(tuple(int((x // p) % q) for p in pw))
    return unc, wit


def covering_radius(code, n, q):
    return mindist(code, q, n, want_dist=False)[2]


def dilate(code, q, n, R):
    """Covering decision and the covered map (D <= R)."""
    dist, hist, _ = mindist(code, q, n)
    cov = dist <= R
    return bool(cov.all()), cov


def count(code, q, n, R):
    """Coverage multiplicity of every word (uint16) and the uncovered count."""
    lib = L.load()
    a = _code(code, q, n)
    cnt = np.zeros(q ** n, dtype=np.uint16)
    u = ctypes.c_int64(0)
    L.check(lib.cov_count(q, n, R, L.u8ptr(a) if a.size else None, int(a.shape[0]),
                          cnt.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16)), ctypes.byref(u)),
            "cov_count")
    return cnt, int(u.value)


def finish(code, q, n, R, M, fast=False):
    """covcount's finisher (cov/engine/covcount.c): (M distinct words,
    uncovered count or -1 with fast).  The top-up and the recount run on the
    GPU; with fast only the de-duplication and counting-order top-up."""
    lib = L.load()
    a = _code(code, q, n)
    out = np.zeros((M, n), dtype=np.uint8)
    words = ctypes.c_int32(0)
    unc = ctypes.c_int64(0)
    L.check(lib.cov_finish(q, n, R, M, L.u8ptr(a) if a.size else None, int(a.shape[0]), 1 if fast else 0,
                           L.u8ptr(out), ctypes.byref(words), ctypes.byref(unc)), "cov_finish")
    return out, int(unc.value)
