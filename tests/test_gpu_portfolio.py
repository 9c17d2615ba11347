"""The reference's campaign driver (cov/campaign.py, run_batch :54-86,
record :88-145; its copy under baseline/_ref) launching the covsearch_gpu
drop-in on the GPU through COVSEARCH_BIN: campaign's parse of the RESULT
lines and the --out files equal what it gets from the reference engine
binary (built from the same copy) on the same seeds, and a cover passes
campaign's own verifier and is recorded."""
import os

import pytest

from tests.test_portfolio import REPO, batch, load_campaign

pytestmark = pytest.mark.gpu

GPU_BIN = os.path.join(REPO, "coldcase_gb300", "bin", "covsearch_gpu")
COPY = os.path.join(REPO, "baseline", "_ref")


@pytest.mark.parametrize("M,iters", [(420, 400), (380, 300)])
def test_campaign_drives_the_gpu_drop_in(covlib, tmp_path, M, iters):
    campaign = load_campaign(os.path.join(COPY, "cov"))
    ref_bin = os.path.join(COPY, "bin", "covsearch2e")
    if not os.path.exists(ref_bin):
        pytest.skip("the reference engine is not built from its copy on this host")
    q, n, R = 4, 6, 1
    b_ref, _, out_ref = batch(campaign, ref_bin, str(tmp_path / "ref"), q, n, R, M, iters)
    b_us, path, out_us = batch(campaign, GPU_BIN, str(tmp_path / "gpu"), q, n, R, M, iters)
    assert b_us == b_ref and out_us == out_ref
    if b_us == 0:
        campaign.RESULTS = str(tmp_path / "results")
        assert campaign.record(q, n, R, M, path, "covsearch_gpu drop-in")
