"""Transform-engine search: ruin and recreate over exact maps of one cell.

Capability of cov/gemm2/gpuchain.py (its Engine, :94-410): a code of M words
is improved by removing some codewords and placing new ones greedily, with
every decision read off exact counts kept on the device (cov_lns_* in
libcovgpu.so).  The search here is its own design:

  * recreate -- cov_lns_greedy: the lazy greedy placement runs on the device
    (a persistent cluster kernel re-counts the best gain bound exactly until
    it is current, then places it), so a placement costs no host round trip;
    the host only asks for it.  Each placed word covers as many uncovered
    words as any word can (ties to the lower index).
  * ruin -- k codewords leave, chosen by one of four rules drawn with fixed
    weights: a soft minimum of their exact losses (Gumbel top-k: codewords
    that cover few words alone leave first, with randomness set by a
    temperature), the codewords nearest a random uncovered word, the
    codewords nearest a random codeword, or a uniform draw.  k follows a
    truncated geometric law between kmin and kmax (small ruins are common).
  * acceptance -- late acceptance (LAHC, Burke and Bykov): a round is kept
    when its uncovered count is no worse than the current one or than the
    count kept `history` rounds earlier; otherwise it is undone exactly by
    the opposite balls of the words it placed and removed.
  * peel -- cov_lns_peel: codewords in a random order leave while each
    covers no word alone (one exact pass on the device is complete: a
    removal never lowers another codeword's private count).

Words are MSB-first indices (x = sum_j w_j q^(n-1-j)); every device result is
deterministic, and the host draws come from one seeded generator, so a run
is reproducible from its seed.
"""
import ctypes
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

    def apply(self, idx, sign):
        """Add sign (+1/-1) over the ball of each word in turn; returns the
        uncovered count afterwards."""
        a, p = self._u32(idx)
        u = ctypes.c_int64(0)
        L.check(self.lib.cov_lns_apply(self.h, p if a.size else None, int(a.size), int(sign), ctypes.byref(u)),
                "cov_lns_apply")
        return int(u.value)

    def ball_update(self, idx, delta):
        self.apply(idx, delta)

    def greedy(self, room, cand_cap=1 << 16):
        """Place up to `room` best words (device lazy greedy); returns
        (placed indices in order, uncovered, refreshes, exact counts)."""
        out = np.zeros(max(room, 1), dtype=np.uint32)
        k = ctypes.c_int32(0)
        u = ctypes.c_int64(0)
        st = np.zeros(2, dtype=np.int64)
        L.check(self.lib.cov_lns_greedy(self.h, int(room), int(cand_cap),
                                        out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), ctypes.byref(k),
                                        ctypes.byref(u), st.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))),
                "cov_lns_greedy")
        return out[:k.value].astype(np.int64), int(u.value), int(st[0]), int(st[1])

    def peel(self, order):
        """Exact peel of the listed codewords in this order; returns (mask of
        the removed, uncovered)."""
        a, p = self._u32(order)
        flags = np.zeros(max(a.size, 1), dtype=np.uint8)
        k = ctypes.c_int32(0)
        u = ctypes.c_int64(0)
        L.check(self.lib.cov_lns_peel(self.h, p if a.size else None, int(a.size),
                                      flags.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), ctypes.byref(k),
                                      ctypes.byref(u)), "cov_lns_peel")
        return flags[:a.size].astype(bool), int(u.value)

    def uncovered_words(self, cap):
        idx = np.zeros(max(cap, 1), dtype=np.uint32)
        found = ctypes.c_int64(0)
        L.check(self.lib.cov_lns_uncovered(self.h, int(cap), idx.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                           ctypes.byref(found)), "cov_lns_uncovered")
        return idx[:min(cap, int(found.value))].astype(np.int64), int(found.value)

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
    """Ruin-and-recreate search for one cell; the code is kept as a sorted
    array of distinct word indices."""

    RUIN_RULES = ("soft", "near_uncovered", "cluster", "random")
    RUIN_WEIGHTS = (0.45, 0.30, 0.15, 0.10)

    def __init__(self, q, n, R, seed=1, out=None, log=None, deadline=None, cand_cap=1 << 16, history=16,
                 temperature=0.25):
        self.q, self.n, self.R = q, n, R
        self.rng = np.random.default_rng([int(seed), q, n, R])
        self.out = out
        self.log = log or (lambda *a: None)
        self.deadline = deadline
        self.cand_cap = cand_cap
        self.history = history
        self.temperature = temperature
        self.eng = TransformEngine(q, n, R)
        self.code = np.zeros(0, dtype=np.int64)
        self.uncov = None
        self.best_code = None
        self.best_uncov = None
        self._last_pub = 0.0
        self.stats = dict(transforms=0, placements=0, removals=0, rounds=0, recounts=0, refreshes=0,
                          exact_counts=0, accepted=0)

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
            a = self.eng.word_index(a) if a.size else np.zeros(0, dtype=np.int64)
        self.code = np.unique(a.astype(np.int64)) if a.size else np.zeros(0, dtype=np.int64)
        self.recount_from_scratch()
        self.stats["recounts"] = 0
        self._remember()

    def recount_from_scratch(self):
        self.eng.recount(self.code)
        self.stats["transforms"] += 1
        self.stats["recounts"] += 1
        self.uncov = self.eng.count(0)
        return self.uncov

    def _remember(self):
        """Keep the best code (fewest uncovered, then fewest words)."""
        if (self.best_uncov is None or self.uncov < self.best_uncov or
                (self.uncov == self.best_uncov and len(self.code) < len(self.best_code))):
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

    # ------------------------------------------------------------ moves
    def recreate(self, M):
        """Greedy placement up to M words; returns the placed words."""
        room = M - len(self.code)
        if room <= 0 or self.uncov == 0:
            return np.zeros(0, dtype=np.int64)
        placed, self.uncov, refr, ev = self.eng.greedy(room, self.cand_cap)
        self.stats["refreshes"] += refr
        self.stats["transforms"] += refr
        self.stats["exact_counts"] += ev
        self.stats["placements"] += len(placed)
        if len(placed):
            self.code = np.union1d(self.code, placed)
        return placed

    def greedy_fill(self, M):
        self.recreate(M)
        return self.uncov

    def losses(self):
        """Exact private coverage of every codeword (the loss map read at
        the code)."""
        self.eng.loss_map()
        self.stats["transforms"] += 1
        return self.eng.map_read(self.code)

    def _nearest(self, centre, k):
        """Indices (into self.code) of the k codewords nearest `centre`
        (digits), ties in random order."""
        digs = self.eng.index_word(self.code)
        d = (digs != centre[None, :]).sum(axis=1).astype(np.float64)
        return np.argsort(d + self.rng.random(len(self.code)), kind="stable")[:k]

    def choose_ruin(self, k, rule):
        m = len(self.code)
        if rule == "random":
            return self.rng.choice(m, size=k, replace=False)
        if rule == "cluster":
            return self._nearest(self.eng.index_word(self.code[self.rng.integers(m)])[0], k)
        if rule == "near_uncovered":
            words, found = self.eng.uncovered_words(4096)
            if found == 0:
                return self.choose_ruin(k, "soft")
            u = words[self.rng.integers(len(words))]
            return self._nearest(self.eng.index_word(np.array([u]))[0], k)
        # soft minimum of the losses: Gumbel top-k of -loss / tau
        loss = self.losses().astype(np.float64)
        tau = max(1.0, self.temperature * float(loss.mean()))
        g = -loss / tau + self.rng.gumbel(size=m)
        return np.argsort(-g, kind="stable")[:k]

    def ruin(self, k, rule="soft"):
        """Remove k codewords chosen by `rule`; returns them."""
        m = len(self.code)
        k = min(k, m - 1)
        if k <= 0:
            return np.zeros(0, dtype=np.int64)
        pick = self.choose_ruin(k, rule)
        removed = self.code[pick]
        self.uncov = self.eng.apply(removed, -1)
        self.code = np.delete(self.code, pick)
        self.stats["removals"] += int(k)
        return removed

    def peel(self):
        """Remove, in a random order, every codeword that covers no word
        alone; returns how many left."""
        if not len(self.code):
            return 0
        order = self.code[self.rng.permutation(len(self.code))]
        gone, self.uncov = self.eng.peel(order)
        keep = np.setdiff1d(self.code, order[gone])
        removed = len(self.code) - len(keep)
        self.code = keep
        self.stats["removals"] += removed
        return removed

    def _k(self, kmin, kmax):
        """Ruin size: kmin plus a geometric draw of mean (kmax - kmin) / 4,
        truncated at kmax."""
        if kmax <= kmin:
            return kmin
        p = 1.0 / (1.0 + (kmax - kmin) / 4.0)
        return int(min(kmax, kmin + self.rng.geometric(p) - 1))

    # ------------------------------------------------------------ search
    def lns(self, M, budget_s, kmin=8, kmax=None, log_every=20, max_rounds=None):
        """Rounds of ruin + recreate at M codewords until covered, the
        budget or max_rounds; returns the uncovered count of the best code."""
        t0 = time.time()
        kmax = kmax or max(kmin + 1, M // 20)
        self.best_uncov = None
        self.best_code = None
        if len(self.code) < M:
            self.recreate(M)
        self._remember()
        hist = [self.uncov] * max(1, self.history)
        r = 0
        while self.uncov > 0:
            if time.time() - t0 > budget_s or self.time_left() < 5:
                break
            if max_rounds is not None and r >= max_rounds:
                break
            before = self.uncov
            rule = self.RUIN_RULES[int(self.rng.choice(len(self.RUIN_RULES), p=self.RUIN_WEIGHTS))]
            removed = self.ruin(self._k(kmin, kmax), rule)
            placed = self.recreate(M)
            self.stats["rounds"] += 1
            v = r % len(hist)
            r += 1
            if self.uncov <= before or self.uncov <= hist[v]:
                self.stats["accepted"] += 1
                self._remember()
            else:
                # undo exactly: the placed words leave, the removed return
                self.eng.apply(placed, -1)
                self.uncov = self.eng.apply(removed, +1)
                self.code = np.union1d(np.setdiff1d(self.code, placed), removed)
            hist[v] = self.uncov
            if r % log_every == 0:
                self.log("  lns M=%d round=%d uncov=%d best=%d (%.1fs)" % (M, r, self.uncov, self.best_uncov,
                                                                          time.time() - t0))
        if self.best_code is not None and (self.uncov > self.best_uncov or
                                           (self.uncov == self.best_uncov and len(self.code) > len(self.best_code))):
            self.code = self.best_code.copy()
            self.recount_from_scratch()
        return self.uncov
