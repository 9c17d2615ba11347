"""bench.py's reference arm (the reference engine, built from its copy under
baseline/_ref, on the host cores; the oracle port where this host has no
copy) runs and prints one JSON line with the contract's keys, and the CPU
baselines of uneven cells are modelled from per-shape samples."""
import json
import os
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)


def test_reference_arm_line():
    out = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0", "--ref-moves", "2"], capture_output=True, text=True, timeout=600,
                         cwd=REPO)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "config", "cpu_baseline", "e2e"):
        assert k in line
    assert line["impl"] == "reference" and line["value"] > 0
    import bench
    want = "reference" if bench.ref_exe() else "port"
    assert line["cpu_baseline"]["kind"] == want and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    assert "window" in line["config"]


def test_cell_baseline_model():
    import bench
    if not bench.ref_exe():
        import pytest
        pytest.skip("no copy of the reference engine on this host")
    cells = [dict(q=6, n=6, R=2, M=20, moves=100), dict(q=5, n=6, R=2, M=90, moves=500),
             dict(q=6, n=6, R=2, M=20, moves=300)]
    r = bench.ref_cells_measure(cells, 20, cores=2)
    assert r["shapes"] == 2 and r["value"] > 0 and len(r["per_cell_s"]) == 3
    # the same shape costs in proportion to its budget (plus the same init)
    a, _, c = r["per_cell_s"]
    assert c > a


def test_dt_pass_bytes():
    import bench
    # 7^9: bitmap + the low tile pass + one strip pass over the high axes
    assert bench.dt_pass_bytes(7, 9) == 7 ** 9 // 8 + 7 ** 9 + 2 * 7 ** 9
    # 8^10: two strip passes
    assert bench.dt_pass_bytes(8, 10) == 8 ** 10 // 8 + 8 ** 10 + 4 * 8 ** 10
