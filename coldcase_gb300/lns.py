"""Transform-engine LNS: ruin-and-recreate over exact full-grid maps.

The GPU form of cov/gemm2/gpuchain.py (Engine, :94-410).  One cell is
resident on the device (cov_lns_* in libcovgpu.so); every decision reads an
exact map:

  * recreate (greedy_fill, gpuchain.py:193-279): lazy greedy placement.  A
    gain map gives, for every word at once, how many uncovered words a
    codeword there would cover.  Gains only fall as codewords are added, so
    stale gains bound the true ones: candidates are popped best-first in
    batches, re-evaluated exactly by ball gathers, and the best is placed
    when it still beats the next bound.  The map is refreshed after a number
    of placements, or when the bounds run out.
  * ruin (:281-323): remove k codewords -- the lowest exact private coverage
    (loss map) with exponential jitter, a random subset, a cluster around a
    random codeword, or a cluster around a high-gain word (a hole).
  * peel (:325-364): remove codewords of zero loss (a cover stays a cover),
    pairwise far apart so that removals do not create private words for
    each other.
  * lns (:367-410): at fixed M, rounds of ruin + recreate; a round that
    ends worse is undone with probability 0.9.

Words are MSB-first indices (x = sum_j w_j q^(n-1-j)); extraction returns
positions in index order, so a run is reproducible from its seed.
"""
import ctypes
import heapq
import os
import time

import numpy as np

from . import lib as L


class TransformEngine:
    """The device state of one (q, n, R) cell: coverage counts and a map."""

    def __init__(self, q, n, R):
        self.q, self.n, self.R = q, n, R
        self.N = q ** n
        self.pw = np.array([q ** (n - 1 - j) for j in range(n)], dtype=np.int64)
        self.lib = L.load()
        h = ctypes.c_void_p()
        L.check(self.lib.cov_lns_create(q, n, R, ctypes.byref(h)), "cov_lns_create")
        self.h = h
        self.extract_cap = 1 << 22

    def close(self):
        if self.h:
            self.lib.cov_lns_destroy(self.h)
            self.h = None

    @staticmethod
    def _u32(idx):
        a = np.ascontiguousarray(np.atleast_1d(idx), dtype=np.uint32)
        return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))

    def word_index(self, words):
        return np.asarray(words, dtype=np.int64) @ self.pw

    def index_word(self, idx):
        idx = np.asarray(idx, dtype=np.int64).ravel()
        return ((idx[:, None] // self.pw[None, :]) % self.q).astype(np.uint8)

    def recount(self, idx):
        a, p = self._u32(idx)
        L.check(self.lib.cov_lns_recount(self.h, p if a.size else None, int(a.size)), "cov_lns_recount")

    def gain_map(self):
        L.check(self.lib.cov_lns_map(self.h, 0), "cov_lns_map")

    def loss_map(self):
        L.check(self.lib.cov_lns_map(self.h, 1), "cov_lns_map")

    def map_max(self):
        v = ctypes.c_int32(0)
        L.check(self.lib.cov_lns_map_max(self.h, ctypes.byref(v)), "cov_lns_map_max")
        return int(v.value)

    def map_hist(self, nbins, vmax):
        out = np.zeros(nbins, dtype=np.int64)
        L.check(self.lib.cov_lns_map_hist(self.h, int(nbins), int(vmax),
                                          out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))), "cov_lns_map_hist")
        return out

    def map_extract(self, thr, cap):
        idx = np.zeros(max(cap, 1), dtype=np.uint32)
        val = np.zeros(max(cap, 1), dtype=np.int32)
        found = ctypes.c_int64(0)
        L.check(self.lib.cov_lns_map_extract(self.h, int(thr), int(cap),
                                             idx.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                             val.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                             ctypes.byref(found)), "cov_lns_map_extract")
        k = min(int(found.value), cap)
        return idx[:k].astype(np.int64), val[:k].astype(np.int64), int(found.value)

    def map_read(self, idx):
        a, p = self._u32(idx)
        out = np.zeros(a.size, dtype=np.int32)
        if a.size:
            L.check(self.lib.cov_lns_map_read(self.h, p, int(a.size), out.ctypes.data_as(L._PI32)),
                    "cov_lns_map_read")
        return out.astype(np.int64)

    def ball_count(self, idx, target):
        """#{y in the ball of each idx : cnt[y] == target} (0: gain, 1: loss)."""
        a, p = self._u32(idx)
        out = np.zeros(a.size, dtype=np.int32)
        if a.size:
            L.check(self.lib.cov_lns_ball(self.h, p, int(a.size), 0, int(target), out.ctypes.data_as(L._PI32)),
                    "cov_lns_ball")
        return out.astype(np.int64)

    def ball_update(self, idx, delta):
        a, p = self._u32(idx)
        if a.size:
            L.check(self.lib.cov_lns_ball(self.h, p, int(a.size), 1, int(delta), None), "cov_lns_ball")

    def count(self, target=0):
        v = ctypes.c_int64(0)
        L.check(self.lib.cov_lns_count(self.h, int(target), ctypes.byref(v)), "cov_lns_count")
        return int(v.value)

    def cnt(self):
        out = np.zeros(self.N, dtype=np.uint16)
        L.check(self.lib.cov_lns_get_cnt(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16))),
                "cov_lns_get_cnt")
        return out

    def map(self):
        out = np.zeros(self.N, dtype=np.int32)
        L.check(self.lib.cov_lns_get_map(self.h, out.ctypes.data_as(L._PI32)), "cov_lns_get_map")
        return out


def write_code_atomic(path, words):
    digits = "0123456789abcdefghijklmnopqrstuvwxyz"
    body = "".join("".join(digits[int(v)] for v in w) + "\n" for w in words)
    tmp = path + ".part"
    with open(tmp, "w") as f:
        f.write(body)
    os.replace(tmp, path)


class LNS:
    """Ruin-and-recreate search for one cell; codewords kept as sorted word
    indices (distinct)."""

    RUIN_MODES = ("low", "hole", "hole", "cluster", "random")

    def __init__(self, q, n, R, seed=1, out=None, log=None, deadline=None, bound_cap=1 << 14):
        self.q, self.n, self.R = q, n, R
        self.bound_cap = bound_cap      # most stale bounds kept per refresh of the gain map
        self.rng = np.random.default_rng(seed * 1000003 + 12345)
        self.out = out
        self.log = log or (lambda *a: None)
        self.deadline = deadline
        self.eng = TransformEngine(q, n, R)
        self.code = np.zeros(0, dtype=np.int64)
        self.uncov = None
        self.best_code = None
        self.best_uncov = None
        self._last_pub = 0.0
        self.stats = dict(transforms=0, placements=0, removals=0, rounds=0, recounts=0)

    def close(self):
        self.eng.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def time_left(self):
        return float("inf") if self.deadline is None else self.deadline - time.time()

    # ------------------------------------------------------------ state
    def load(self, code):
        """Word indices (1-D) or digits (m, n); repeats are dropped."""
        a = np.asarray(code)
        if a.ndim == 2:
            a = self.eng.word_index(a)
        self.code = np.unique(a.astype(np.int64)) if a.size else np.zeros(0, dtype=np.int64)
        self._recount()
        self._keep_best()

    def _recount(self):
        self.eng.recount(self.code)
        self.stats["transforms"] += 1
        self.uncov = self.eng.count(0)

    def _keep_best(self):
        better = (self.best_uncov is None or self.uncov < self.best_uncov or
                  (self.uncov == self.best_uncov and len(self.code) < len(self.best_code)))
        if better:
            self.best_uncov = self.uncov
            self.best_code = self.code.copy()
            self.publish()

    def publish(self, force=False):
        if self.out is None or self.best_code is None or not len(self.best_code):
            return
        now = time.time()
        if not force and now - self._last_pub < 1.0:
            return
        self._last_pub = now
        write_code_atomic(self.out, self.eng.index_word(self.best_code))

    def recount_from_scratch(self):
        self._recount()
        self.stats["recounts"] += 1
        return self.uncov

    # ------------------------------------------------------------ recreate
    def _refresh_bounds(self, codeset):
        """Gain map -> heap of (-gain, word) above a threshold that keeps the
        extraction bounded; returns (heap, threshold)."""
        eng = self.eng
        eng.gain_map()
        self.stats["transforms"] += 1
        top = eng.map_max()
        if top <= 0:
            return [], 0
        cap = min(eng.extract_cap, self.bound_cap)
        thr = 1
        if top > 1:
            hist = eng.map_hist(1024, top)
            above = np.cumsum(hist[::-1])[::-1]           # words with gain in bin b or higher
            ok = np.flatnonzero(above <= cap * 0.9)
            b = int(ok[0]) if len(ok) else 1023
            thr = max(1, b * top // 1024 + 1)
        idx, val, found = eng.map_extract(thr, cap)
        while found > cap and thr < top:
            thr = min(top, thr + max(1, (top - thr) // 2))
            idx, val, found = eng.map_extract(thr, cap)
        heap = [(-int(v), int(i)) for v, i in zip(val.tolist(), idx.tolist()) if int(i) not in codeset]
        heapq.heapify(heap)
        return heap, thr

    def greedy_fill(self, target_m, batch=64, refresh_every=512):
        """Exact lazy greedy placement until covered, target_m codewords, or
        the deadline; returns the uncovered count."""
        eng = self.eng
        codeset = set(self.code.tolist())
        heap, thr = [], 1
        since = refresh_every
        while self.uncov > 0 and len(codeset) < target_m and self.time_left() >= 5:
            if since >= refresh_every or not heap:
                heap, thr = self._refresh_bounds(codeset)
                since = 0
                if not heap:
                    if thr > 1:
                        since = refresh_every
                        continue
                    break
            cand = []
            while heap and len(cand) < batch:
                v, i = heapq.heappop(heap)
                if i not in codeset:
                    cand.append(i)
            if not cand:
                since = refresh_every
                continue
            exact = eng.ball_count(np.array(cand, dtype=np.int64), 0)
            bi = int(np.argmax(exact))
            best = int(exact[bi])
            bound = -heap[0][0] if heap else 0
            if best < 1:
                since = refresh_every
                continue
            placed = None
            if best >= bound and best >= thr:
                placed = cand[bi]
                eng.ball_update(np.array([placed], dtype=np.int64), +1)
                codeset.add(placed)
                self.uncov -= best
                self.stats["placements"] += 1
                since += 1
            elif best < thr:
                since = refresh_every              # below the extracted range: refresh to stay exact
            for k, i in enumerate(cand):
                if i != placed and exact[k] > 0:
                    heapq.heappush(heap, (-int(exact[k]), i))
        self.code = np.array(sorted(codeset), dtype=np.int64)
        return self.uncov

    # ------------------------------------------------------------ ruin
    def losses(self):
        self.eng.loss_map()
        self.stats["transforms"] += 1
        return self.eng.map_read(self.code)

    def _nearest(self, centre_digits, k):
        digs = self.eng.index_word(self.code).astype(np.int16)
        d = (digs != centre_digits[None, :]).sum(axis=1)
        return np.argsort(d + self.rng.random(len(self.code)))[:k]

    def ruin(self, k, mode="low"):
        """Remove k codewords (mode: low, random, cluster, hole); returns them."""
        m = len(self.code)
        k = min(k, m - 1)
        if k <= 0:
            return np.zeros(0, dtype=np.int64)
        if mode == "random":
            pick = self.rng.choice(m, size=k, replace=False)
        elif mode == "cluster":
            centre = self.eng.index_word(self.code[self.rng.integers(m)])[0].astype(np.int16)
            pick = self._nearest(centre, k)
        elif mode == "hole":
            self.eng.gain_map()
            self.stats["transforms"] += 1
            top = self.eng.map_max()
            if top <= 0:
                return self.ruin(k, "low")
            hi, _, _ = self.eng.map_extract(max(1, top // 2), 4096)
            if not len(hi):
                return self.ruin(k, "low")
            centre = self.eng.index_word(np.array([int(hi[self.rng.integers(len(hi))])]))[0].astype(np.int16)
            pick = self._nearest(centre, k)
        else:
            lo = self.losses().astype(np.float64)
            jitter = self.rng.exponential(scale=max(1.0, lo.mean() * 0.15), size=m)
            pick = np.argsort(lo + jitter)[:k]
        removed = self.code[pick]
        self.eng.ball_update(removed, -1)
        self.code = np.delete(self.code, pick)
        self.uncov = self.eng.count(0)
        self.stats["removals"] += int(k)
        return removed

    # ------------------------------------------------------------ peel
    def peel(self):
        """Remove zero-loss codewords until none is left; returns how many."""
        total = 0
        while self.time_left() >= 5:
            zeros = np.flatnonzero(self.losses() == 0)
            if not len(zeros):
                break
            zeros = zeros[self.eng.ball_count(self.code[zeros], 1) == 0]
            if not len(zeros):
                break
            self.rng.shuffle(zeros)
            if 2 * self.R < self.n:
                digs = self.eng.index_word(self.code[zeros]).astype(np.int16)
                keep = []
                for i in range(len(zeros)):
                    if all((digs[j] != digs[i]).sum() > 2 * self.R for j in keep):
                        keep.append(i)
                pick = zeros[np.array(keep)]
            else:
                pick = zeros[:1]
            self.eng.ball_update(self.code[pick], -1)
            mask = np.ones(len(self.code), dtype=bool)
            mask[pick] = False
            self.code = self.code[mask]
            total += len(pick)
            self.stats["removals"] += len(pick)
        if total:
            self.uncov = self.eng.count(0)
        return total

    # ------------------------------------------------------------ LNS
    def lns(self, M, budget_s, kmin=8, kmax=None, log_every=20, max_rounds=None):
        """Rounds of ruin + recreate at M codewords until covered, the
        budget or max_rounds; returns the uncovered count of the best code."""
        t0 = time.time()
        kmax = kmax or max(kmin + 1, M // 20)
        self.best_uncov = None
        self.best_code = None
        if len(self.code) < M:
            self.greedy_fill(M)
        self._keep_best()
        r = 0
        while self.uncov > 0:
            if time.time() - t0 > budget_s or self.time_left() < 10:
                break
            if max_rounds is not None and r >= max_rounds:
                break
            before = self.uncov
            k = int(self.rng.integers(kmin, kmax + 1))
            mode = self.RUIN_MODES[int(self.rng.integers(len(self.RUIN_MODES)))]
            self.ruin(k, mode)
            self.greedy_fill(M)
            self.stats["rounds"] += 1
            r += 1
            if self.uncov > before and self.rng.random() > 0.10:
                self.code = self.best_code.copy()
                self._recount()
            else:
                self._keep_best()
            if r % log_every == 0:
                self.log("  lns M=%d round=%d uncov=%d best=%d k=%d (%.0fs)"
                         % (M, r, self.uncov, self.best_uncov, k, time.time() - t0))
            if r % 50 == 0:
                inc = self.uncov
                if self.recount_from_scratch() != inc:
                    self.log("  drift: incremental %d, recount %d" % (inc, self.uncov))
        if self.uncov == 0:
            self._keep_best()
        elif self.best_code is not None and self.best_uncov < self.uncov:
            self.code = self.best_code.copy()
            self._recount()
        return self.uncov
