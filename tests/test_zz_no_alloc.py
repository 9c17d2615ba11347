"""The allocation-free distance transform (cov_mindist_dev_static).

It exists for callers that may not allocate device memory themselves, for
example because their device memory belongs to another allocator; its only
scratch buffer is a fixed device array.  Called through the C ABI, its output
must equal, word for word, both the oracle's line-min transform and the
allocating entry point cov_mindist_dev, on two calls in a row (the second
call finds the scratch holding the first call's contents); the largest
accepted size (q^n = 2^26, where the bitmap fills the whole array) must run,
and a size beyond its limit must be refused.

The file name makes pytest collect it last.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _threads():
    import os
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


@pytest.mark.parametrize("q,n,M", [(4, 6, 420), (6, 9, 700), (7, 9, 1500), (5, 3, 2), (4, 13, 3000)])
def test_static_scratch_matches_oracle_and_allocating_transform(covlib, q, n, M):
    import torch
    from oracle import pyoracle as po
    from coldcase_gb300.workloads import uniform_code
    code = uniform_code(q, n, M, 11)
    oracle = torch.from_numpy(po.mindist(code, q, n, threads=_threads()))
    dev = torch.device("cuda", 0)
    d_code = torch.from_numpy(code).to(dev)
    want = torch.empty(q ** n, dtype=torch.uint8, device=dev)
    got = torch.empty(q ** n, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    assert covlib.cov_mindist_dev(q, n, d_code.data_ptr(), M, want.data_ptr(), stream) == 0
    torch.cuda.synchronize()
    assert torch.equal(want.cpu(), oracle)
    for _ in range(2):
        got.fill_(255)
        assert covlib.cov_mindist_dev_static(q, n, d_code.data_ptr(), M, got.data_ptr(), stream) == 0
        torch.cuda.synchronize()
        assert torch.equal(got, want)
        assert torch.equal(got.cpu(), oracle)


def test_static_scratch_refuses_oversized(covlib):
    import torch
    dev = torch.device("cuda", 0)
    buf = torch.empty(16, dtype=torch.uint8, device=dev)
    # 8^9 = 134,217,728 words: beyond the 2^26-word limit
    rc = covlib.cov_mindist_dev_static(8, 9, buf.data_ptr(), 1, buf.data_ptr(),
                                       torch.cuda.current_stream(dev).cuda_stream)
    assert rc == -7
