"""Portfolio integration: the reference's campaign driver (cov/campaign.py,
run_batch :54-86 and record :88-145) launches the covsearch_gpu drop-in
through COVSEARCH_BIN exactly as it launches the reference engine.

On this CPU host the drop-in's command line runs with the oracle standing in
for the GPU (tests/portfolio_stub.py); campaign's parse of its RESULT lines
and its --out files must equal what campaign gets from the reference engine
binary on the same seeds, and a cover must pass campaign's own verifier and
be recorded.  (tests/test_gpu_portfolio.py does the same with the GPU.)
"""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("COLDCASE_REF", "/root/reference")
STUB = os.path.join(REPO, "tests", "portfolio_stub.py")
REF_BIN = os.path.join(REPO, "oracle", "_ref", "covsearch2e")


def load_campaign(cov_dir):
    if not os.path.exists(os.path.join(cov_dir, "campaign.py")):
        pytest.skip("no copy of the reference's campaign driver on this host")
    sys.dont_write_bytecode = True
    if cov_dir not in sys.path:
        sys.path.insert(0, cov_dir)
    import campaign
    return campaign


def batch(campaign, binary, tmp, q, n, R, M, iters, workers=3):
    campaign.BIN = binary
    os.makedirs(tmp, exist_ok=True)
    best, path = campaign.run_batch(q, n, R, M, workers, 60.0, 1, 1, ["--iters", str(iters)], None, tmp,
                                    verbose=False)
    outs = []
    for w in range(workers):
        with open(os.path.join(tmp, "w%03d.txt" % w)) as f:
            outs.append(f.read())
    return best, path, outs


@pytest.mark.parametrize("M,iters", [(420, 400), (380, 300)])
def test_campaign_drives_the_drop_in(tmp_path, M, iters):
    campaign = load_campaign(os.path.join(REF, "cov"))
    if not os.path.exists(REF_BIN):
        pytest.skip("the reference engine is not built on this host (make -C oracle ref)")
    q, n, R = 4, 6, 1
    b_ref, _, out_ref = batch(campaign, REF_BIN, str(tmp_path / "ref"), q, n, R, M, iters)
    b_us, path, out_us = batch(campaign, STUB, str(tmp_path / "us"), q, n, R, M, iters)
    assert b_us == b_ref and out_us == out_ref
    if b_us == 0:
        campaign.RESULTS = str(tmp_path / "results")
        dest = campaign.record(q, n, R, M, path, "covsearch_gpu drop-in")
        assert dest and os.path.exists(dest) and os.path.exists(dest.replace(".txt", ".json"))
