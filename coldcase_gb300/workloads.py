"""Synthetic workloads with the shapes of the five benchmark configurations.

Codes are numpy.random.default_rng(seed).integers(0, q, (M, n), uint8):
uniform i.i.d. digits, the convention used to seed the reference engine
through --in for every measurement.  Restart / instance seeds follow the
covengine convention base*1000003 + i*7919 (cov/engine/covengine:557).
"""
import math

import numpy as np


def uniform_code(q, n, M, seed):
    return np.random.default_rng(seed).integers(0, q, (M, n), dtype=np.uint8)


def ball_volume(q, n, R):
    return sum(math.comb(n, i) * (q - 1) ** i for i in range(0, min(R, n) + 1))


def instance_seed(base, i):
    return base * 1000003 + i * 7919


PLAIN_CPU = dict(name="plain q4 n6 R1 M420 tenure10", q=4, n=6, R=1, M=420, tabu=10, moves=10 ** 4)
PLAIN_GPU = dict(name="plain q6 n9 R4 M700 tenure20", q=6, n=9, R=4, M=700, tabu=20, moves=10 ** 5)
BATCHED = dict(name="batched 64x q7 n9 R4 M1500 tenure20", q=7, n=9, R=4, M=1500, tabu=20,
               moves=10 ** 5, restarts=64)


def hetero_cells(count=256, seed=2026, max_words=43_000_000, max_m=65535, rejected=None):
    """Uneven (q,n,R,M) cells: q in {5..8}, n in {6..9} with q^n <= 4.3e7,
    R in {1..4}, M = ceil(1.3 q^n / |B(n,R)|).  Cells whose M exceeds 65535
    lie outside the reference engine's domain (covsearch2e.c:1117) and this
    engine's (16-bit coverer ids): they are redrawn, and each one drawn is
    appended to `rejected` when a list is given."""
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < count:
        q = int(rng.integers(5, 9))
        n = int(rng.integers(6, 10))
        R = int(rng.integers(1, 5))
        if q ** n > max_words:
            continue
        M = math.ceil(1.3 * q ** n / ball_volume(q, n, R))
        if M > max_m:
            if rejected is not None:
                rejected.append(dict(q=q, n=n, R=R, M=M))
            continue
        out.append(dict(q=q, n=n, R=R, M=M, seed=instance_seed(seed, len(out))))
    return out


def serve_requests(count=200, lam=100.0, seed=2027, max_words=60_500_000, max_m=65535, rejected=None):
    """Open-loop Poisson stream of solve requests: q in {5,6,7}, n in
    {6..10} with q^n <= 6.05e7, R in {1..4}, M = ceil(1.3 q^n / |B(n,R)|),
    move budget log-uniform in [1e3, 1e5], arrivals with exponential gaps of
    mean 1/lam seconds.  Requests with M above 65535 (outside the reference
    engine's domain and this engine's) are redrawn and, when a list is
    given, appended to `rejected`."""
    rng = np.random.default_rng(seed)
    out = []
    t = 0.0
    while len(out) < count:
        q = int(rng.integers(5, 8))
        n = int(rng.integers(6, 11))
        R = int(rng.integers(1, 5))
        if q ** n > max_words:
            continue
        M = math.ceil(1.3 * q ** n / ball_volume(q, n, R))
        if M > max_m:
            if rejected is not None:
                rejected.append(dict(q=q, n=n, R=R, M=M))
            continue
        moves = int(round(10 ** rng.uniform(3, 5)))
        t += float(rng.exponential(1.0 / lam))
        out.append(dict(id=len(out), q=q, n=n, R=R, M=M, seed=instance_seed(seed, len(out)), moves=moves,
                        arrival=t))
    return out
