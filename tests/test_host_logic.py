"""Host-side logic that needs no GPU: workload generators, size classes,
the autotuner's plan."""
import math

from coldcase_gb300 import workloads
from coldcase_gb300.batch import Tuner, size_class
from coldcase_gb300.batch import elastic_clusters
from coldcase_gb300.serve import default_cluster


def test_hetero_cells_domain():
    cells = workloads.hetero_cells()
    assert len(cells) == 256
    for c in cells:
        assert c["q"] in (5, 6, 7, 8) and 6 <= c["n"] <= 9 and 1 <= c["R"] <= 4
        assert c["q"] ** c["n"] <= 43_000_000
        assert c["M"] == math.ceil(1.3 * c["q"] ** c["n"] / workloads.ball_volume(c["q"], c["n"], c["R"]))
        assert c["M"] <= 65535
    assert len({c["seed"] for c in cells}) == 256


def test_serve_requests_domain():
    reqs = workloads.serve_requests(300, lam=50.0)
    arr = [r["arrival"] for r in reqs]
    assert arr == sorted(arr)
    for r in reqs:
        assert r["q"] in (5, 6, 7) and 6 <= r["n"] <= 10 and r["q"] ** r["n"] <= 60_500_000
        assert 1000 <= r["moves"] <= 100000 and r["M"] <= 65535
    gaps = [b - a for a, b in zip([0.0] + arr[:-1], arr)]
    assert 0.5 / 50 < sum(gaps) / len(gaps) < 2.0 / 50


def test_size_class_orders_by_work():
    assert size_class(4, 6, 1, 420) < size_class(7, 9, 4, 1500)
    assert size_class(7, 9, 4, 1500) == "s16"
    assert default_cluster(4, 6, 1, 420) == 1 and default_cluster(7, 9, 4, 1500) == 4


def test_tuner_plan_widens_critical_class():
    classes = {"small": (200, {1: 1e-5, 2: 0.8e-5, 4: 0.7e-5}),
               "big": (10, {1: 300e-6, 2: 170e-6, 4: 90e-6, 8: 50e-6, 16: 35e-6})}
    choice, est = Tuner.plan(classes, 20000, resident=152)
    assert choice["small"] == 1
    assert choice["big"] == 8          # 16 would cost more SM time than it saves
    assert abs(est - 1.0) < 1e-9


def test_tuner_plan_keeps_narrow_when_saturated():
    # many big instances: the GPU is full, wider clusters only add CTA time
    classes = {"big": (1000, {1: 300e-6, 2: 170e-6, 4: 90e-6})}
    choice, _ = Tuner.plan(classes, 20000, resident=152)
    assert choice["big"] == 1


def test_elastic_clusters():
    # few requests: everyone widened, the heaviest first, within the CTAs
    w = elastic_clusters({1: 1, 2: 2, 3: 1}, {1: 10, 2: 90000, 3: 500}, 152)
    assert w == {1: 16, 2: 16, 3: 16}
    w = elastic_clusters({1: 1, 2: 2, 3: 1}, {1: 10, 2: 90000, 3: 500}, 20)
    assert sum(w.values()) <= 20 and w[2] >= w[3] >= w[1]
    # saturated: nothing changes
    base = {k: 1 for k in range(200)}
    assert elastic_clusters(base, {k: k for k in range(200)}, 152) == base


def test_tuner_cache_unwritable(tmp_path, monkeypatch):
    """An unwritable cache location does not break tuning."""
    import os
    from coldcase_gb300 import batch
    ro = tmp_path / "ro"
    ro.mkdir()
    os.chmod(ro, 0o500)
    monkeypatch.setenv("COLDCASE_GB300_CACHE", str(ro / "sub"))
    t = batch.Tuner()
    t.table["s04"] = {"1": 1e-5}
    t._save()                       # must not raise
    os.chmod(ro, 0o700)
