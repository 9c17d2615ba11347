"""ctypes wrapper of liboracle.so (test infrastructure only; see oracle.h)."""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None


class MoveRec(ctypes.Structure):
    _fields_ = [("it", ctypes.c_int64), ("u", ctypes.c_int64), ("delta", ctypes.c_int64),
                ("unc", ctypes.c_int64), ("unc_end", ctypes.c_int64), ("best", ctypes.c_int64),
                ("ncand", ctypes.c_int32), ("ncw", ctypes.c_int32), ("i", ctypes.c_int32),
                ("p", ctypes.c_int32), ("v", ctypes.c_int32), ("kicked", ctypes.c_int32)]


MOVE_DTYPE = np.dtype([("it", "<i8"), ("u", "<i8"), ("delta", "<i8"), ("unc", "<i8"),
                       ("unc_end", "<i8"), ("best", "<i8"), ("ncand", "<i4"), ("ncw", "<i4"),
                       ("i", "<i4"), ("p", "<i4"), ("v", "<i4"), ("kicked", "<i4")])


def build():
    """make -C oracle (the restatement; `ref` also when the reference tree exists)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return os.path.join(HERE, "liboracle.so")


def load():
    global _lib
    if _lib is not None:
        return _lib
    path = os.path.join(HERE, "liboracle.so")
    srcs = [os.path.join(HERE, f) for f in ("covoracle.c", "dtoracle.c", "oracle.h")]
    if not os.path.exists(path) or any(os.path.getmtime(s) > os.path.getmtime(path) for s in srcs):
        build()
    lib = ctypes.CDLL(path)
    P = ctypes.c_void_p
    u8p = ctypes.POINTER(ctypes.c_uint8)
    lib.orc_create.restype = P
    lib.orc_create.argtypes = [ctypes.c_int] * 4 + [ctypes.c_uint64, ctypes.c_int, ctypes.c_int,
                                                   ctypes.c_longlong, ctypes.c_int, ctypes.c_int]
    lib.orc_destroy.argtypes = [P]
    lib.orc_init.restype = ctypes.c_longlong
    lib.orc_init.argtypes = [P, u8p, ctypes.c_int, ctypes.c_int]
    lib.orc_run.restype = ctypes.c_longlong
    lib.orc_run.argtypes = [P, ctypes.c_longlong, ctypes.c_longlong, ctypes.POINTER(MoveRec)]
    for f in ("orc_uncovered", "orc_best_uncovered", "orc_iters", "orc_kicks"):
        getattr(lib, f).restype = ctypes.c_longlong
        getattr(lib, f).argtypes = [P]
    lib.orc_get_code.argtypes = [P, u8p]
    lib.orc_get_best.argtypes = [P, u8p]
    lib.orc_get_cnt.argtypes = [P, ctypes.POINTER(ctypes.c_uint16)]
    lib.orc_get_tabu.argtypes = [P, ctypes.POINTER(ctypes.c_int32)]
    lib.orc_get_rng.argtypes = [P, ctypes.POINTER(ctypes.c_uint64)]
    lib.orc_eval_codeword.argtypes = [P, ctypes.c_int, ctypes.POINTER(ctypes.c_longlong)]
    lib.orc_set_fix0.restype = ctypes.c_int
    lib.orc_set_fix0.argtypes = [P, ctypes.c_int]
    lib.orc_set_sa.restype = ctypes.c_int
    lib.orc_set_sa.argtypes = [P, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double]
    lib.orc_set_noise.restype = ctypes.c_int
    lib.orc_set_noise.argtypes = [P, ctypes.c_int]
    lib.orc_set_pick.restype = ctypes.c_int
    lib.orc_set_pick.argtypes = [P, ctypes.c_int, ctypes.c_int]
    lib.orc_set_wide.restype = ctypes.c_int
    lib.orc_set_wide.argtypes = [P, ctypes.c_int]
    lib.orc_ul_state.argtypes = [P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    lib.sym_create.restype = P
    lib.sym_create.argtypes = [ctypes.c_int] * 5 + [ctypes.c_uint64, ctypes.c_int, ctypes.c_longlong,
                                                    ctypes.c_int]
    lib.sym_destroy.argtypes = [P]
    lib.sym_init.restype = ctypes.c_longlong
    lib.sym_init.argtypes = [P]
    lib.sym_run.restype = ctypes.c_longlong
    lib.sym_run.argtypes = [P, ctypes.c_longlong, ctypes.POINTER(MoveRec)]
    for f in ("sym_uncovered", "sym_best_uncovered", "sym_iters", "sym_kicks"):
        getattr(lib, f).restype = ctypes.c_longlong
        getattr(lib, f).argtypes = [P]
    lib.sym_set_threads.argtypes = [P, ctypes.c_int]
    lib.sym_orbits.restype = ctypes.c_int
    lib.sym_orbits.argtypes = [P]
    lib.sym_get_rep.argtypes = [P, u8p]
    lib.sym_get_best.argtypes = [P, u8p]
    lib.sym_get_cnt.argtypes = [P, ctypes.POINTER(ctypes.c_uint16)]
    lib.sym_get_rng.argtypes = [P, ctypes.POINTER(ctypes.c_uint64)]
    lib.orc_distinct_code.restype = ctypes.c_int
    lib.orc_distinct_code.argtypes = [ctypes.c_int] * 3 + [u8p, ctypes.c_int, u8p]
    lib.orc_cover_count.restype = ctypes.c_int
    lib.orc_cover_count.argtypes = [ctypes.c_int] * 3 + [u8p, ctypes.c_int, ctypes.POINTER(ctypes.c_uint16)]
    lib.orc_verify_pure.restype = ctypes.c_longlong
    lib.orc_verify_pure.argtypes = [ctypes.c_int] * 3 + [u8p, ctypes.c_int]
    lib.orc_mindist.restype = ctypes.c_int
    lib.orc_mindist.argtypes = [ctypes.c_int, ctypes.c_int, u8p, ctypes.c_int, u8p, ctypes.c_int]
    lib.orc_linemin.restype = ctypes.c_int
    lib.orc_linemin.argtypes = [ctypes.c_int, ctypes.c_int, u8p, ctypes.c_int, u8p, ctypes.c_int]
    lib.orc_dilate.restype = ctypes.c_int
    lib.orc_dilate.argtypes = [ctypes.c_int] * 3 + [u8p, ctypes.c_int, u8p]
    _lib = lib
    return lib


def _u8(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))


class Oracle:
    """One restated covsearch2e p5b search (covsearch2e.c:1023-1621)."""

    def __init__(self, q, n, R, M, seed=12345, tabu=0, kick=2, stall=5000, cand=100000, threads=1,
                 wide=False, fix0=False, sa=None, noise=0, upick=False, ucache=False):
        """sa: None, or (t0, cool, tmin) for --sa --t0 --cool --tmin;
        noise: --noise PERMILLE; upick / ucache: --upick / --ucache."""
        self.lib = load()
        self.q, self.n, self.R, self.M = q, n, R, M
        self.h = self.lib.orc_create(q, n, R, M, seed, tabu, kick, stall, cand, threads)
        if not self.h:
            raise ValueError("oracle: bad parameters")
        if wide and self.lib.orc_set_wide(self.h, 1) != 0:
            self.close()
            raise MemoryError("oracle: no memory for the wide candidate set")
        if fix0 and self.lib.orc_set_fix0(self.h, 1) != 0:
            self.close()
            raise ValueError("oracle: --fix0 needs M >= 2")
        if sa is not None:
            self.lib.orc_set_sa(self.h, 1, float(sa[0]), float(sa[1]), float(sa[2]))
        if noise and self.lib.orc_set_noise(self.h, int(noise)) != 0:
            self.close()
            raise ValueError("oracle: bad --noise")
        if upick or ucache:
            self.lib.orc_set_pick(self.h, 1 if upick else 0, 1 if ucache else 0)

    def init(self, code=None, random_init=False):
        a = np.zeros((0, self.n), dtype=np.uint8) if code is None else \
            np.ascontiguousarray(np.asarray(code, dtype=np.uint8).reshape(-1, self.n))
        return self.lib.orc_init(self.h, _u8(a) if a.size else None, a.shape[0], 1 if random_init else 0)

    def run(self, moves, target=-1, trace=False):
        tr = (MoveRec * max(1, int(moves)))() if trace else None
        made = self.lib.orc_run(self.h, int(moves), int(target), tr)
        if not trace:
            return made
        buf = np.frombuffer(tr, dtype=MOVE_DTYPE, count=max(1, int(moves)))[:made].copy()
        return buf

    def uncovered(self):
        return self.lib.orc_uncovered(self.h)

    def best_uncovered(self):
        return self.lib.orc_best_uncovered(self.h)

    def iters(self):
        return self.lib.orc_iters(self.h)

    def kicks(self):
        return self.lib.orc_kicks(self.h)

    def ul_state(self):
        """(valid, length) of the uncovered-word list."""
        v, n = ctypes.c_int(), ctypes.c_int()
        self.lib.orc_ul_state(self.h, ctypes.byref(v), ctypes.byref(n))
        return v.value, n.value

    def code(self):
        out = np.zeros((self.M, self.n), dtype=np.uint8)
        self.lib.orc_get_code(self.h, _u8(out))
        return out

    def best(self):
        out = np.zeros((self.M, self.n), dtype=np.uint8)
        self.lib.orc_get_best(self.h, _u8(out))
        return out

    def cnt(self):
        out = np.zeros(self.q ** self.n, dtype=np.uint16)
        self.lib.orc_get_cnt(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16)))
        return out

    def tabu(self):
        out = np.zeros(self.M * self.n * self.q, dtype=np.int32)
        self.lib.orc_get_tabu(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
        return out

    def rng(self):
        out = np.zeros(4, dtype=np.uint64)
        self.lib.orc_get_rng(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)))
        return out

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def distinct_code(code, q, n, M):
    lib = load()
    a = np.ascontiguousarray(np.asarray(code, dtype=np.uint8).reshape(-1, n))
    out = np.zeros((M, n), dtype=np.uint8)
    m = lib.orc_distinct_code(q, n, M, _u8(a), a.shape[0], _u8(out))
    return out[:m]


def cover_count(code, q, n, R):
    lib = load()
    a = np.ascontiguousarray(np.asarray(code, dtype=np.uint8).reshape(-1, n))
    out = np.zeros(q ** n, dtype=np.uint16)
    lib.orc_cover_count(q, n, R, _u8(a), a.shape[0], out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16)))
    return out


def verify_pure(code, q, n, R):
    lib = load()
    a = np.ascontiguousarray(np.asarray(code, dtype=np.uint8).reshape(-1, n))
    return int(lib.orc_verify_pure(q, n, R, _u8(a), a.shape[0]))


def mindist(code, q, n, threads=1):
    lib = load()
    a = np.ascontiguousarray(np.asarray(code, dtype=np.uint8).reshape(-1, n))
    out = np.zeros(q ** n, dtype=np.uint8)
    lib.orc_mindist(q, n, _u8(a) if a.size else None, a.shape[0], _u8(out), threads)
    return out


def linemin(code, q, n, threads=1):
    """Per-word minimum distance by n axis line-min passes (orc_linemin)."""
    lib = load()
    a = np.ascontiguousarray(np.asarray(code, dtype=np.uint8).reshape(-1, n))
    out = np.zeros(q ** n, dtype=np.uint8)
    lib.orc_linemin(q, n, _u8(a) if a.size else None, a.shape[0], _u8(out), threads)
    return out


def dilate(code, q, n, R):
    lib = load()
    a = np.ascontiguousarray(np.asarray(code, dtype=np.uint8).reshape(-1, n))
    cov = np.zeros(q ** n, dtype=np.uint8)
    ok = lib.orc_dilate(q, n, R, _u8(a), a.shape[0], _u8(cov))
    return bool(ok), cov.astype(bool)


# ---------------------------------------------------------------- finisher --
# Restatement of the reference finisher cov/engine/covcount.c: read at most
# M well-formed words (:94-118), drop repeats keeping first occurrences
# (:120-131), top up to M distinct words -- in base-q counting order with
# --fast (:133-160), else on still-uncovered words found by 64 xorshift64
# probes, then a linear scan, then any unused word (:163-195) -- marking each
# added word's ball, and count the uncovered words (:197-199).  Pure Python:
# small cases only.
_DIG = "0123456789abcdefghijklmnopqrstuvwxyz"


def finish_read(text, q, n, M):
    import re
    out = []
    for line in text.splitlines(True):
        if len(out) >= M:
            break
        line = line.split("#")[0]
        if any(ch in line for ch in " ,\t"):
            toks = [t for t in re.split(r"[ ,\t\r\n]+", line) if t][:n]
            w = []
            for t in toks:
                m = re.match(r"[+-]?\d+", t)
                w.append((int(m.group(0)) if m else 0) & 0xff)
        else:
            w = [_DIG.index(ch) for ch in line.rstrip("\r\n") if ch in _DIG][:n]
        if len(w) != n or any(v >= q for v in w):
            continue
        out.append(w)
    return out


def finish(text, q, n, R, M, fast=False):
    """(words as lists, uncovered or -1, exit status) of covcount."""
    N = q ** n
    pw = [q ** (n - 1 - j) for j in range(n)]
    code = []
    seen = set()
    for w in finish_read(text, q, n, M):
        t = tuple(w)
        if t not in seen:
            seen.add(t)
            code.append(list(w))
    digits = lambda x: [(x // pw[j]) % q for j in range(n)]
    if fast:
        x = 0
        while len(code) < M:
            t = tuple(digits(x))
            x += 1
            if t in seen:
                continue
            seen.add(t)
            code.append(list(t))
        return code, -1, 1
    cov = np.zeros(N, dtype=bool)

    def mark(c):
        cov[cover_count(np.array([c], dtype=np.uint8), q, n, R) > 0] = True

    for c in code:
        mark(c)
    mask = (1 << 64) - 1
    rs = 88172645463325252 ^ len(code)

    def step(r):
        r ^= (r << 13) & mask
        r ^= r >> 7
        r ^= (r << 17) & mask
        return r

    scan = 0
    while len(code) < M:
        w = -1
        for _ in range(64):
            rs = step(rs)
            c2 = rs % N
            if not cov[c2]:
                w = c2
                break
        if w < 0:
            while scan < N and cov[scan]:
                scan += 1
            if scan < N:
                w = scan
        if w < 0:
            while True:
                rs = step(rs)
                cand = digits(rs % N)
                if tuple(cand) not in seen:
                    break
            new = cand
        else:
            new = digits(w)
        seen.add(tuple(new))
        code.append(new)
        mark(new)
    unc = int((~cov).sum())
    return code, unc, 0 if unc == 0 else 1


class SymOracle:
    """One restated symsearch run (cov/engine/symsearch.c:282-491)."""

    def __init__(self, q, n, R, M, orbits=0, seed=12345, kick=2, stall=3000, cand=100000, threads=1):
        self.lib = load()
        self.q, self.n, self.R, self.M = q, n, R, M
        self.h = self.lib.sym_create(q, n, R, M, orbits, seed, kick, stall, cand)
        if not self.h:
            raise ValueError("symsearch oracle: bad parameters")
        if threads > 1:
            self.lib.sym_set_threads(self.h, int(threads))
        self.orbits = self.lib.sym_orbits(self.h)

    def init(self):
        return self.lib.sym_init(self.h)

    def run(self, moves, trace=False):
        tr = (MoveRec * max(1, int(moves)))() if trace else None
        made = self.lib.sym_run(self.h, int(moves), tr)
        if not trace:
            return made
        return np.frombuffer(tr, dtype=MOVE_DTYPE, count=max(1, int(moves)))[:made].copy()

    def uncovered(self):
        return self.lib.sym_uncovered(self.h)

    def best_uncovered(self):
        return self.lib.sym_best_uncovered(self.h)

    def iters(self):
        return self.lib.sym_iters(self.h)

    def kicks(self):
        return self.lib.sym_kicks(self.h)

    def _reps(self, fn):
        out = np.zeros((self.orbits, self.n - 1), dtype=np.uint8)
        fn(self.h, _u8(out))
        return out

    def rep(self):
        return self._reps(self.lib.sym_get_rep)

    def best(self):
        return self._reps(self.lib.sym_get_best)

    def cnt(self):
        out = np.zeros(self.q ** (self.n - 1), dtype=np.uint16)
        self.lib.sym_get_cnt(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16)))
        return out

    def rng(self):
        out = np.zeros(4, dtype=np.uint64)
        self.lib.sym_get_rng(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)))
        return out

    def close(self):
        if self.h:
            self.lib.sym_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()
