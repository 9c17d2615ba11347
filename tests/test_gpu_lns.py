"""Transform-engine primitives against brute force on small cells and
against the oracle's ball marking on a cell whose transform takes several
shared-memory sweeps; the device greedy and peel against plain CPU
restatements; the search's written codes against the verifier."""
import itertools
import os
import re
import subprocess
import sys
import tempfile

import numpy as np
import pytest

from coldcase_gb300 import codefile, verify
from coldcase_gb300.lns import LNS, TransformEngine
from coldcase_gb300.workloads import uniform_code

pytestmark = pytest.mark.gpu
REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def brute(q, n, R, code_idx):
    N = q ** n
    words = np.array(list(itertools.product(range(q), repeat=n)), dtype=np.int64)   # MSB-first order
    D = (words[:, None, :] != words[None, :, :]).sum(2)
    cnt = np.zeros(N, dtype=np.int64)
    for c in code_idx:
        cnt += D[c] <= R
    gain = ((D <= R) & (cnt == 0)[None, :]).sum(1)
    loss = ((D <= R) & (cnt == 1)[None, :]).sum(1)
    return cnt, gain, loss, D


@pytest.mark.parametrize("q,n,R,m", [(3, 4, 1, 6), (4, 4, 2, 5), (2, 7, 2, 9), (5, 3, 1, 7), (3, 5, 0, 20),
                                     (6, 4, 3, 2)])
def test_primitives_exact(covlib, q, n, R, m):
    rng = np.random.default_rng(q * 100 + n)
    N = q ** n
    code = rng.integers(0, N, m)
    code[1] = code[0]                      # a repeat counts twice
    cnt, gain, loss, D = brute(q, n, R, code)
    e = TransformEngine(q, n, R)
    try:
        e.recount(code)
        assert (e.cnt() == cnt).all()
        assert e.count(0) == int((cnt == 0).sum())
        e.gain_map()
        assert (e.map() == gain).all()
        assert e.map_max() == int(gain.max())
        thr = max(1, int(gain.max()) // 2)
        idx, val, found = e.map_extract(thr, 1 << 20)
        want = np.flatnonzero(gain >= thr)
        assert found == len(want) and (idx == want).all() and (val == gain[want]).all()
        v = gain[gain >= 1].astype(np.int64)
        # 32-bit binning, and the 64-bit one where (vmax-1) * nbins passes 2^32
        for nb, vmax in ((8, int(gain.max()) or 1), (1024, 3), (8192, 600000)):
            hist = e.map_hist(nb, vmax)
            assert (hist == np.bincount((np.minimum(v, vmax) - 1) * nb // vmax, minlength=nb)).all(), (nb, vmax)
        probe = rng.integers(0, N, 9)
        assert (e.ball_count(probe, 0) == gain[probe]).all()
        e.loss_map()
        assert (e.map() == loss).all()
        assert (e.map_read(code) == loss[code]).all()
        assert (e.ball_count(probe, 1) == loss[probe]).all()
        add = rng.integers(0, N, 3)
        e.ball_update(add, +1)
        assert (e.cnt() == cnt + sum((D[a] <= R).astype(np.int64) for a in add)).all()
        e.ball_update(add, -1)
        assert (e.cnt() == cnt).all()
    finally:
        e.close()


def test_lns_finds_cover_and_writes_it(covlib):
    q, n, R, M = 3, 5, 1, 30
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "best.txt")
        with LNS(q, n, R, seed=3, out=out) as e:
            e.load(np.zeros(0, dtype=np.int64))
            unc = e.lns(M, budget_s=60, max_rounds=400)
            e.publish(force=True)
            assert unc == 0 and e.recount_from_scratch() == 0
        code = codefile.read_code(out, n)
        assert len(code) <= M and len({tuple(w) for w in code.tolist()}) == len(code)
        assert verify.verify(code, n, q, R, want_witness=False)[0] == 0


def test_lns_improves_a_random_seed(covlib):
    q, n, R, M = 4, 6, 2, 60
    code = uniform_code(q, n, 80, 5)
    with LNS(q, n, R, seed=7) as e:
        e.load(code)
        e.ruin(len(e.code) - M, "soft")
        start = e.uncov
        unc = e.lns(M, budget_s=60, max_rounds=60)
        assert len(e.code) <= M and unc <= start
        assert verify.verify(e.eng.index_word(e.code), n, q, R, want_witness=False)[0] == unc


def test_gpuchain_cli(covlib):
    cli = os.path.join(REPO, "coldcase_gb300", "bin", "gpuchain_gpu")
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "out.txt")
        p = subprocess.run([sys.executable, cli, "-q", "3", "-n", "5", "-R", "1", "-M", "30", "-t", "60", "-s", "2",
                            "--out", out, "--quiet", "--rounds", "300"], capture_output=True, text=True, timeout=300)
        assert p.returncode == 0, p.stderr
        m = re.search(r"RESULT q=3 n=5 R=1 M=(\d+) uncovered=(\d+) iters=(\d+)", p.stdout)
        assert m, p.stdout
        code = codefile.read_code(out, 5)
        assert verify.verify(code, 5, 3, 1, want_witness=False)[0] == int(m.group(2))


@pytest.mark.parametrize("q,n,R,M", [(6, 9, 5, 250), (7, 7, 3, 300), (8, 7, 4, 137), (5, 9, 2, 6000),
                                     (9, 6, 2, 2500), (4, 10, 3, 1500)])
def test_layered_maps_multi_sweep(covlib, q, n, R, M):
    """Low tiles and strip sweeps for the alphabets with their own map
    kernels (q = 5..8) and the generic one (q = 4, 9); q6 n9 R5 needs a low
    tile and two strip sweeps.  cnt, the gain map and the loss map equal the
    oracle's ball marking of the code, of the uncovered words and of the
    words covered once."""
    from oracle import pyoracle as po
    code = uniform_code(q, n, M, 41)
    e = TransformEngine(q, n, R)
    try:
        idx = e.word_index(code)
        e.recount(idx)
        cnt = e.cnt()
        assert (cnt == po.cover_count(code, q, n, R)).all()
        for target in (0, 1):
            marked = np.flatnonzero(cnt == target)
            assert 0 < len(marked)
            want = po.cover_count(e.index_word(marked), q, n, R)
            e.gain_map() if target == 0 else e.loss_map()
            assert (e.map() == want).all(), target
    finally:
        e.close()


def cpu_greedy(q, n, R, code_idx, room):
    """Plain greedy: repeatedly the word covering most uncovered words
    (lowest index on ties), until room is used, all is covered or nothing
    gains."""
    N = q ** n
    words = np.array(list(itertools.product(range(q), repeat=n)), dtype=np.int64)
    B = (words[:, None, :] != words[None, :, :]).sum(2) <= R
    cov = np.zeros(N, dtype=np.int64)
    for c in code_idx:
        cov += B[c]
    out = []
    while len(out) < room and (cov == 0).any():
        gain = (B & (cov == 0)[None, :]).sum(1)
        x = int(np.argmax(gain))            # first index of the maximum
        if gain[x] <= 0:
            break
        out.append(x)
        cov += B[x]
    return out, int((cov == 0).sum())


@pytest.mark.parametrize("q,n,R,m0,room,cap", [(4, 6, 1, 40, 300, 1 << 16), (3, 7, 2, 5, 200, 1 << 16),
                                               (4, 6, 1, 40, 300, 16), (5, 5, 2, 3, 60, 4)])
def test_device_greedy_is_the_plain_greedy(covlib, q, n, R, m0, room, cap):
    rng = np.random.default_rng(q * 31 + n)
    start = np.unique(rng.integers(0, q ** n, m0))
    want, unc = cpu_greedy(q, n, R, start, room)
    e = TransformEngine(q, n, R)
    try:
        e.recount(start)
        placed, u, refreshes, _ = e.greedy(room, cand_cap=cap)
        assert placed.tolist() == want and u == unc and e.count(0) == unc
        if cap < 64:
            assert refreshes > 1
    finally:
        e.close()


def test_device_peel_and_apply(covlib):
    """The peel removes, in the given order, each codeword that covers no
    word alone at its turn; apply's +-1 balls leave the exact counts."""
    q, n, R = 4, 6, 1
    N = q ** n
    words = np.array(list(itertools.product(range(q), repeat=n)), dtype=np.int64)
    B = (words[:, None, :] != words[None, :, :]).sum(2) <= R
    rng = np.random.default_rng(9)
    code = np.unique(rng.integers(0, N, 900))
    order = code[rng.permutation(len(code))]
    cov = B[code].sum(0)
    gone = []
    for c in order:
        if not ((cov == 1) & B[c]).any():
            cov -= B[c]
            gone.append(True)
        else:
            gone.append(False)
    e = TransformEngine(q, n, R)
    try:
        e.recount(code)
        mask, u = e.peel(order)
        assert mask.tolist() == gone and u == int((cov == 0).sum())
        assert (e.cnt() == cov).all()
        extra = rng.integers(0, N, 7)
        u2 = e.apply(extra, +1)
        assert u2 == int((cov + B[extra].sum(0) == 0).sum())
        assert e.apply(extra, -1) == u and (e.cnt() == cov).all()
    finally:
        e.close()


def test_lns_rounds_undo_exactly(covlib):
    """Rejected rounds are undone by opposite balls: the device counts
    equal a fresh count of the code the search holds after every round."""
    q, n, R, M = 5, 6, 2, 110
    with LNS(q, n, R, seed=4, history=1) as e:
        e.load(uniform_code(q, n, M, 8))
        for _ in range(6):
            e.lns(M, budget_s=60, max_rounds=5, kmin=4, kmax=12)
            cnt = e.eng.cnt().copy()
            u = e.uncov
            assert e.recount_from_scratch() == u and (e.eng.cnt() == cnt).all()
            if u == 0:
                break
