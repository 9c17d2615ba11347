"""CUDA distance transform / coverage count vs the reference verifiers'
golden values and the oracle."""
import numpy as np
import pytest

from coldcase_gb300 import verify
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def test_golden_verify_cases(covlib, golden):
    _, cases = golden
    for c in cases:
        code = np.array(c["code"], dtype=np.uint8)
        q, n, R = c["q"], c["n"], c["R"]
        unc, wit = verify.verify(code, n, q, R)
        assert unc == c["uncovered"], c["src"]
        assert verify.verify(code, n, q, R, want_witness=False)[0] == unc
        dist, hist, rad = verify.mindist(code, q, n)
        if c["hist"] is not None:
            assert hist.tolist() == c["hist"], c["src"]
            assert rad == c["radius"]
        for w in wit:
            x = int(np.dot(w, q ** np.arange(n - 1, -1, -1)))
            assert dist[x] > R
        cnt, u2 = verify.count(code, q, n, R)
        assert u2 == c["uncovered"]
        if q ** n <= 5_000_000:
            assert (cnt == po.cover_count(code, q, n, R)).all(), c["src"]
            assert (dist == po.mindist(code, q, n, threads=8)).all(), c["src"]


@pytest.mark.parametrize("q,n,R,M", [(4, 6, 1, 420), (6, 9, 4, 700), (7, 9, 4, 1500), (6, 10, 4, 1500),
                                     (5, 10, 3, 900), (8, 8, 4, 300), (2, 16, 3, 700), (16, 4, 1, 100),
                                     (3, 1, 0, 2), (7, 2, 1, 1)])
def test_transform_properties(covlib, q, n, R, M):
    from coldcase_gb300.workloads import uniform_code
    code = uniform_code(q, n, M, 7)
    dist, hist, rad = verify.mindist(code, q, n)
    cnt, unc = verify.count(code, q, n, R)
    # size-independent properties: D <= R exactly where cnt > 0; D == 0 on the code
    assert ((dist <= R) == (cnt > 0)).all()
    pw = q ** np.arange(n - 1, -1, -1, dtype=np.int64)
    idx = code.astype(np.int64) @ pw
    assert (dist[idx] == 0).all()
    assert hist.sum() == q ** n and unc == int(hist[R + 1:].sum())
    # spot check D against brute force on sampled words
    rng = np.random.default_rng(1)
    xs = rng.integers(0, q ** n, 2000)
    dig = (xs[:, None] // pw[None, :]) % q
    brute = (dig[:, None, :] != code[None, :, :]).sum(axis=2).min(axis=1)
    assert (dist[xs] == brute).all()
    if q ** n <= 50_000_000 and M * sum(1 for _ in range(1)) and q ** n * 2 < 2 ** 31:
        ref = po.cover_count(code, q, n, R)
        assert (cnt == ref).all()


def test_empty_code(covlib):
    dist, hist, rad = verify.mindist(np.zeros((0, 5), np.uint8), 3, 5)
    assert (dist == 6).all() and rad == 6 and hist[6] == 3 ** 5
    assert verify.verify(np.zeros((0, 5), np.uint8), 5, 3, 2, want_witness=False)[0] == 3 ** 5


@pytest.mark.parametrize("q,n,M", [(5, 9, 300), (3, 13, 200), (7, 8, 400), (6, 8, 90), (2, 16, 500)])
def test_transform_into_unaligned_output(covlib, q, n, M):
    """cov_mindist_dev writing its words at byte offsets 0..3 of a device
    buffer (rows of every pass start at any byte; the kernels move them as
    aligned words plus edge bytes): every word equals the oracle's, and the
    bytes around the output stay untouched."""
    import torch
    from coldcase_gb300.workloads import uniform_code
    code = uniform_code(q, n, M, 5)
    want = torch.from_numpy(po.mindist(code, q, n, threads=8))
    dev = torch.device("cuda", 0)
    d_code = torch.from_numpy(code).to(dev)
    N = q ** n
    buf = torch.empty(N + 8, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for off in range(4):
        buf.fill_(0xA5)
        assert covlib.cov_mindist_dev(q, n, d_code.data_ptr(), M, buf.data_ptr() + off, stream) == 0
        torch.cuda.synchronize()
        h = buf.cpu()
        assert torch.equal(h[off:off + N], want), off
        assert (h[:off] == 0xA5).all() and (h[off + N:] == 0xA5).all(), off
