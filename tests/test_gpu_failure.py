"""Failure detection without a GPU fault: every launch is bounded by a
deadline; a slot that reaches it stops between moves with COV_ETIMEOUT, the
host reads the status, the context stays usable, and after resume the slot
continues on exactly the trajectory of an uninterrupted run.  Bad requests
are refused on the host with COV_E* codes."""
import numpy as np
import pytest

from coldcase_gb300 import lib as L
from coldcase_gb300.engine import Pool
from coldcase_gb300.workloads import uniform_code

pytestmark = pytest.mark.gpu


def test_deadline_stop_resume_same_trajectory(covlib):
    q, n, R, M, moves = 6, 7, 3, 74, 1500
    code = uniform_code(q, n, M, 9)
    ref = Pool(1, cluster=2)
    a = ref.add(q, n, R, M, code=code, seed=9, trace=1, trace_cap=moves)
    ref.run(moves)
    want = ref.trace(a)
    ref.close()

    pool = Pool(1, cluster=2)
    s = pool.add(q, n, R, M, code=code, seed=9, trace=1, trace_cap=moves)
    pool.set_budget(1e-6)                 # the deadline passes at once
    pool.run(moves)
    st = pool.status(s)
    assert st["status"] == -4 and st["it"] < moves      # COV_ETIMEOUT, read on the host
    with pytest.raises(L.CovError):
        L.check(st["status"], "run")
    # the context is usable: another instance runs normally meanwhile
    other = Pool(1, cluster=1)
    o = other.add(4, 6, 1, 420, code=uniform_code(4, 6, 420, 1), seed=1)
    other.run(50)
    assert other.status(o)["status"] == 0
    other.close()
    pool.resume(s)
    pool.set_budget(30.0)
    pool.run(moves - st["it"])
    assert pool.status(s)["status"] == 0
    got = pool.trace(s)
    assert got.tobytes() == want.tobytes()
    pool.close()


def test_host_side_refusals(covlib):
    pool = Pool(2, cluster=1)
    with pytest.raises(L.CovError) as e:
        pool.add(17, 6, 1, 10)              # q > 16
    assert e.value.rc == -1
    with pytest.raises(L.CovError):
        pool.add(4, 6, 1, 70000)            # M > 65535 (covsearch2e.c:1117)
    with pytest.raises(L.CovError):
        pool.set_slot_param(5, "cluster", 2)
    s = pool.add(4, 6, 1, 50, code=uniform_code(4, 6, 50, 2), seed=2)
    with pytest.raises(L.CovError):
        pool.set_slot_param(s, "cluster", 17)
    with pytest.raises(L.CovError):
        pool.set_slot_param(s, "no_such_knob", 1)
    pool.add(4, 6, 1, 50, code=uniform_code(4, 6, 50, 3), seed=3)
    with pytest.raises(L.CovError) as e:
        pool.add(4, 6, 1, 50)               # pool full
    assert e.value.rc == -7
    pool.close()


def test_grid_help_wait_runs_out(covlib):
    """The leader's wait for its helper clusters is bounded: with the helpers
    told to leave at once (a test setting), the wait runs out one second past
    the launch budget, the slot reports COV_EDRIFT on the host (its state may
    lack a share of a move), and the context stays usable."""
    import time
    q, n, R, M = 6, 7, 3, 74
    pool = Pool(1, cluster=2, budget_s=0.05)
    pool.set_param("grid_help", 64)
    pool.set_param("grid_help_absent", 1)
    s = pool.add(q, n, R, M, code=uniform_code(q, n, M, 9), seed=9)
    t0 = time.monotonic()
    pool.run(100)
    st = pool.status(s)
    assert st["status"] == -5 and st["it"] <= 1                 # COV_EDRIFT, after the first move
    assert time.monotonic() - t0 < 30
    pool.close()
    other = Pool(1, cluster=2)
    other.set_param("grid_help", 64)
    o = other.add(q, n, R, M, code=uniform_code(q, n, M, 9), seed=9)
    other.run(100)
    assert other.status(o)["status"] == 0 and other.status(o)["it"] == 100
    other.close()
