"""Transform-engine primitives against brute force on small cells, and the
LNS solver's written codes against the verifier."""
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
        hist = e.map_hist(8, int(gain.max()) or 1)
        v = gain[gain >= 1]
        assert (hist == np.bincount((np.minimum(v, max(1, gain.max())) - 1) * 8 // max(1, gain.max()),
                                    minlength=8)).all()
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
        e.ruin(len(e.code) - M, "low")
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
