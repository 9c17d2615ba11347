#!/usr/bin/env python3
"""Headline benchmark: tabu moves/s and coverage words/s at q=7, n=9, R=4.

Workload (one "step"): 64 independent restarts of the q7 n9 R4 M1500
search (tenure 20, uniform random codes from per-restart seeds), each
advanced by --moves moves in one launch of the batched engine.  The state
of the 64 restarts (64 x 40.35M-word counter arrays, ~11 GB) is far larger
than L2, so no flush is needed between steps.

Printed (rank 0, one JSON line):
  value        aggregate tabu moves/s of the batched engine, device-timed with
               CUDA events on the engine's stream over K steps, state resident
  plain        the same search as one instance on one wide cluster, same GPU
  coverage     words/s of the uint8 distance transform and of the coverage
               count over the 7^9 words
  hetero       256 uneven (q,n,R,M) cells, 2e4 moves each, as one graph
               launch with autotuned cluster sizes per size class
  served       a Poisson stream of solve requests through the continuous-
               batching server: aggregate moves/s and p50/p99 latency
  e2e          moves/s through the public Python API with host buffers: each
               step re-seeds every restart from a pinned host code (H2D),
               builds its state, runs --moves moves and reads every best code
               back (D2H)
  roofline     the batched kernel's algorithmic bytes (the reference
               algorithm's per-move bytes with the measured candidate and
               list counts) / its time vs the measured HBM copy bandwidth;
               `design` gives the same for the bytes this engine touches
  cpu_baseline the oracle restatement of the reference engine timed on this
               host's cores (independent restarts, one per core)
--impl reference times that CPU path alone (the reference arm).
"""
import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "tabu moves/s & coverage words/s (q7,n9,R4); batched/served vs plain, same GPU"
Q, N_, R_, M_, TENURE, RESTARTS = 7, 9, 4, 1500, 20, 64
BASE_SEED = 1


def workload_name(restarts, moves):
    return "batched %d restarts q7 n9 R4 M1500 tenure20, %d moves per restart per step" % (restarts, moves)


# ------------------------------------------------------------------ CPU ----
REF_DIR = os.path.join(HERE, "baseline", "_ref")
WARM_NPZ = os.path.join(HERE, "tests", "golden", "warm_q7n9.npz")
WARM_JSON = os.path.join(HERE, "tests", "golden", "warm_q7n9.json")


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def ref_exe():
    """The reference engine (cov/engine/covsearch2e.c, unchanged), built from
    its copy under baseline/_ref by oracle/Makefile's refbin recipe; None
    when this host has no copy."""
    exe = os.path.join(REF_DIR, "bin", "covsearch2e")
    if not os.path.exists(exe) and os.path.exists(os.path.join(REF_DIR, "cov", "engine", "covsearch2e.c")):
        subprocess.run(["make", "-s", "-C", os.path.join(HERE, "oracle"), exe], capture_output=True)
    return exe if os.path.exists(exe) else None


def warm_state():
    """The restarts' codes at the start of the timed window: the oracle's
    codes of restarts 0..15 after `moves` moves (tests/golden/make_warm.py)."""
    import numpy as np
    d = np.load(WARM_NPZ)
    with open(WARM_JSON) as f:
        moves = json.load(f)["moves"]
    return d["codes"], [int(x) for x in d["seeds"]], moves


def _code_file(d, name, code, q):
    from coldcase_gb300 import codefile
    path = os.path.join(d, name)
    with open(path, "w") as f:
        f.write(codefile.format_code(code, q))
    return path


def ref_processes(exe, jobs, tlimit=600.0):
    """Run one reference process per job concurrently (single-threaded, as
    covengine runs its chains): job = (q, n, R, M, code file, seed, tabu,
    iters).  Returns [(iters, seconds after init, wall seconds)], from each
    process's own RESULT line (covsearch2e.c:1582-1589); the seconds are its
    CPU seconds (printed to the millisecond) when its wall time after init,
    printed to 10 ms, is too short to be precise."""
    import re
    rx = re.compile(r"RESULT .* iters=(\d+) .*time=([0-9.]+) rate=\S+ cpu=([0-9.]+) ")
    procs = []
    for (q, n, R, M, path, seed, tabu, iters) in jobs:
        cmd = [exe, "-q", str(q), "-n", str(n), "-R", str(R), "-M", str(M), "--preset", "p5b", "--in", path,
               "-s", str(seed), "--tabu", str(tabu), "--iters", str(iters), "--threads", "1", "-t", str(tlimit),
               "--quiet"]
        procs.append((time.monotonic(), subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                                         text=True)))
    out = []
    for t0, p in procs:
        txt, _ = p.communicate()
        wall = time.monotonic() - t0
        m = rx.search(txt or "")
        if not m:
            raise RuntimeError("reference engine printed no RESULT line (rc %s)" % p.returncode)
        t, cpu = float(m.group(2)), float(m.group(3))
        out.append((int(m.group(1)), t if t >= 0.5 else max(t, cpu), wall))
    return out


def ref_measure(warmup, steps, moves, cores=None):
    """The reference engine on this host's cores: `cores` concurrent
    single-thread processes, restart i started from its code at the start of
    the GPU's timed window (warm_state), `moves` moves per step.  The rate of
    a step is the sum of the processes' own rates (moves / seconds after
    init); the value is the mean over the timed steps."""
    exe = ref_exe()
    if exe is None:
        return None
    codes, seeds, at = warm_state()
    cores = min(cores or host_cores(), len(codes))
    rates, walls = [], []
    with tempfile.TemporaryDirectory() as d:
        files = [_code_file(d, "w%02d.txt" % i, codes[i], Q) for i in range(cores)]
        for k in range(warmup + steps):
            t0 = time.monotonic()
            res = ref_processes(exe, [(Q, N_, R_, M_, files[i], seeds[i] + k, TENURE, moves) for i in range(cores)])
            if k >= warmup:
                rates.append(sum(it / t for it, t, _ in res if t > 0))
                walls.append(time.monotonic() - t0)
    return dict(value=statistics.mean(rates), cores=cores, kind="reference", seconds=sum(walls),
                sample="%d concurrent single-thread covsearch2e --preset p5b processes x %d moves x %d steps, "
                       "restart i from its code after %d moves (the GPU's timed window), rate after init"
                       % (cores, moves, steps, at))


def _cpu_worker(args):
    """One restart on the oracle (single thread) from its warm code:
    untimed init, then the timed steps; each step starts at a shared
    barrier."""
    idx, steps, moves, barrier = args
    sys.path.insert(0, HERE)
    from oracle.pyoracle import Oracle
    codes, seeds, _ = warm_state()
    o = Oracle(Q, N_, R_, M_, seed=seeds[idx], tabu=TENURE, threads=1)
    o.init(codes[idx])
    out = []
    for _ in range(steps):
        barrier.wait()
        t0 = time.monotonic()
        made = o.run(moves)
        out.append((made, t0, time.monotonic()))
    o.close()
    return out


def cpu_measure(warmup, steps, moves, cores=None):
    """The oracle port: aggregate moves/s of `cores` concurrent single-thread
    restarts from the same warm codes as ref_measure."""
    codes, _, at = warm_state()
    cores = min(cores or host_cores(), len(codes))
    subprocess.run(["make", "-s", "-C", os.path.join(HERE, "oracle")], check=True)
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    barrier = mgr.Barrier(cores)
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_worker, [(i, warmup + steps, moves, barrier) for i in range(cores)])
    mgr.shutdown()
    total_m, total_t = 0, 0.0
    for k in range(warmup, warmup + steps):
        total_m += sum(r[k][0] for r in res)
        total_t += max(r[k][2] for r in res) - min(r[k][1] for r in res)
    return dict(value=total_m / total_t, cores=cores, moves=total_m, seconds=total_t, kind="port",
                sample="%d concurrent oracle restarts x %d moves x %d steps from their codes after %d moves "
                       "(after untimed init)" % (cores, moves, steps, at))


def ref_cells_measure(cells, moves, tlimit=600.0, cores=None, min_s=0.3):
    """CPU baseline of a set of independent cells (the uneven batch, the
    served requests): every distinct (q, n, R, M) shape once on the
    reference engine from a uniform code, up to `cores` processes at a time;
    a shape is re-run with ten times the moves while its run took under
    `min_s` seconds after init (and did not cover), so that its rate is
    timed precisely.  Returns per shape (rate after init, init seconds) and
    the batch's modelled CPU time: each cell costs init + its own move budget
    / its shape's rate on one core, the cores share the cells perfectly."""
    from coldcase_gb300.workloads import uniform_code
    exe = ref_exe()
    if exe is None:
        return None
    cores = cores or host_cores()
    shapes = sorted({(c["q"], c["n"], c["R"], c["M"]) for c in cells})
    rate = {}
    iters = {sh: moves for sh in shapes}
    with tempfile.TemporaryDirectory() as d:
        files = {sh: _code_file(d, "c%d.txt" % j, uniform_code(sh[0], sh[1], sh[3], 4242 + j), sh[0])
                 for j, sh in enumerate(shapes)}
        pending = list(shapes)
        for _ in range(4):
            if not pending:
                break
            again = []
            for b in range(0, len(pending), cores):
                part = pending[b:b + cores]
                jobs = [(q, n, R, M, files[(q, n, R, M)], 4242, 0, iters[(q, n, R, M)]) for (q, n, R, M) in part]
                for sh, (it, t, wall) in zip(part, ref_processes(exe, jobs, tlimit)):
                    # a run that stops short of its moves has covered: the cell's
                    # search would stop there too
                    rate[sh] = (it / t if t > 0 and it > 0 else None, max(0.0, wall - t),
                                it if it < iters[sh] else None)
                    if t < min_s and it >= iters[sh]:
                        iters[sh] *= 10
                        again.append(sh)
            pending = again
    per_cell, total_moves = [], 0
    for c in cells:
        r, init, cover = rate[(c["q"], c["n"], c["R"], c["M"])]
        mv = c["moves"] if cover is None else min(c["moves"], cover)
        per_cell.append(init + (mv / r if r else 0.0))
        total_moves += mv
    cpu_s = sum(per_cell) / cores
    return dict(value=total_moves / cpu_s, unit="moves/s", cores=cores, kind="reference", per_cell_s=per_cell,
                shapes=len(shapes),
                sample="each of %d distinct (q,n,R,M) shapes on covsearch2e --preset p5b from a uniform code, "
                       ">= %d moves (more until >= %.1f s after init); every cell costs init + its move budget "
                       "(or the moves its shape's sample needed to cover) at its shape's rate on one core, %d "
                       "cores shared perfectly"
                       % (len(shapes), moves, min_s, cores))



def cells_cpu_measure(args, world):
    """CPU baselines of the uneven-cells and served legs (one reference
    process per cell or request, concurrent up to the host's cores),
    sampled per distinct shape (ref_cells_measure)."""
    import numpy as np
    from coldcase_gb300 import workloads
    out = {}
    if not args.no_hetero:
        cells = workloads.hetero_cells(count=args.cells * world)
        for c in cells:
            c["moves"] = args.cell_moves
        r = ref_cells_measure(cells, args.cell_cpu_moves)
        if r:
            r.pop("per_cell_s")
            out["hetero"] = r
    if not args.no_serve:
        reqs = workloads.serve_requests(args.requests * world, lam=args.lam * world, seed=2027)
        r = ref_cells_measure(reqs, args.cell_cpu_moves)
        if r:
            svc = np.array(r.pop("per_cell_s"))
            r["p50_s"] = float(np.percentile(svc, 50))
            r["p99_s"] = float(np.percentile(svc, 99))
            r["latency_note"] = "service time of each request alone on one core (init + budget / rate), no queueing"
            out["served"] = r
    return out


# --------------------------------------------------------------- clocks ----
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None
        self.idx = gpu_index

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.FIELDS,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return dict(sm_mhz=None, sm_max_mhz=None, reasons=["nvidia-smi unavailable"])
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return dict(sm_mhz=None, sm_max_mhz=None, reasons=["no samples"])
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return dict(sm_mhz=statistics.median(sm) if sm else None, sm_max_mhz=max(mx) if mx else None,
                    reasons=reasons, samples=len(rows))


def measured_peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic():
    """Per-move DRAM bytes of the batched kernel from the committed ncu
    summary, when one exists (profiles/engine_batched_q7n9.json)."""
    p = os.path.join(HERE, "profiles", "engine_batched_q7n9.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    return d.get("dram_bytes_per_move")


def algo_bytes_per_move(q, n, R, M, ncw, ul_n, b_r=1, b_c=2):
    """Algorithmic bytes of one tabu move of the reference algorithm (p5b,
    uncovered list on):
        ncw * S_R * b_r      every candidate codeword's radius-R sphere read
                             once (covsearch2e.c:592-654)
      + U_n * (n + b_c)      the uncovered list: digits and count of each entry
                             (covsearch2e.c:720-734)
      + 2 * S' * 2 * b_c     commit: the leaving and the entering word read
                             and written (covsearch2e.c:450-493)
      + M * n                the distance scan over the code
    S_R = C(n,R)(q-1)^R, S' = C(n-1,R)(q-1)^R; ncw and U_n are the measured
    means per move; b_r = 1 (the 1-byte shadow the reference reads), b_c = 2
    (its uint16 counts)."""
    Sp = math.comb(n - 1, R) * (q - 1) ** R
    SR = math.comb(n, R) * (q - 1) ** R
    return ncw * SR * b_r + ul_n * (n + b_c) + 2 * Sp * 2 * b_c + M * n


def design_bytes_per_move(q, n, R, M, ul_n):
    """Bytes one move of this engine touches at word granularity: the commit
    reads and writes 2 S' 4-byte counters, the moved codeword's sphere
    change reads 2 C(n-1,R-1)(q-1)^(R-1) counters, the list pass reads U_n
    entries of 12 bytes and the distance scan M packed codewords."""
    Sp = math.comb(n - 1, R) * (q - 1) ** R
    X = math.comb(n - 1, R - 1) * (q - 1) ** (R - 1) if R >= 1 else 0
    return 2 * Sp * 8 + 2 * X * 4 + ul_n * 12 + M * 8


# ------------------------------------------------------------------ GPU ----
def sym_cpu_measure(moves):
    """The quotient-search oracle (a port of symsearch.c, its estimates
    OpenMP-parallel as the reference's are) on all host cores:
    K_8(9,4)@940 from its greedy start, `moves` moves timed."""
    from oracle.pyoracle import SymOracle
    try:
        cores = len(os.sched_getaffinity(0))
    except AttributeError:
        cores = os.cpu_count() or 1
    o = SymOracle(8, 9, 4, 940, seed=1000, threads=cores)
    o.init()
    o.run(1)
    t0 = time.perf_counter()
    o.run(moves)
    dt = time.perf_counter() - t0
    return dict(value=moves / dt, unit="moves/s", cores=cores, kind="port",
                sample="K_8(9,4)@940 seed 1000: %d moves after init and one untimed move" % moves)


def dt_pass_bytes(q, n):
    """HBM bytes the distance transform's kernels must move per launch: the
    code bitmap read (N/8), the low-axes tile pass writing every word once
    (N), and one read + write of every word per high-axes strip pass (the
    same grouping of axes as cov_verify.cu's dt_run)."""
    N = q ** n
    q4 = (q + 3) // 4 * 4

    def sweeps(k):
        passes, j0 = 0, k
        while j0 < n:
            g = 0
            while j0 + g < n and q ** (g + 1) * 32 <= 98304:
                g += 1
            j0 += max(g, 1)
            passes += 1
        return passes

    def low(cap):
        k = 1
        while k < n and q ** (k + 1) // q * q4 <= cap:
            k += 1
        return k
    passes = min(sweeps(low(65536)), sweeps(low(200 * 1024)))
    return N // 8 + N + 2 * N * passes


COVERAGE_CELLS = (   # (q, n, R, M): the headline cell and the reference's published transform sizes
    (7, 9, 4, 1500),
    (7, 10, 5, 163),     # M = ceil(1.3 q^n / |B|)
    (8, 10, 4, 2549),
)


def coverage_bench(args, code79, dev):
    """Words/s of the distance transform (cov_mindist_dev) and of the
    coverage count (cov_count_dev) at 7^9 (the headline code) and at 7^10 /
    8^10 (HBM-resident), each with its roofline, plus the CPU baselines at
    7^9: the oracle's line-min transform on all host cores and the
    reference's own verifiers (verify_cov.py --method numpy,
    verify_independent.py --method dilate) as processes."""
    import numpy as np
    import torch
    from coldcase_gb300 import lib as L
    from coldcase_gb300.workloads import uniform_code
    lib = L.load()
    peak, kind = measured_peaks()
    out = {}
    for (q, n, R, M) in COVERAGE_CELLS:
        code = code79 if (q, n, M) == (Q, N_, M_) else uniform_code(q, n, M, 77)
        Nw = q ** n
        code_d = torch.from_numpy(np.ascontiguousarray(code)).to(dev)
        dist_d = torch.empty(Nw, dtype=torch.uint8, device=dev)
        cnt_d = torch.empty(Nw + 1, dtype=torch.int16, device=dev)
        st = torch.cuda.Stream(device=dev)
        cs = st.cuda_stream
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(st):
            for _ in range(3):
                L.check(lib.cov_mindist_dev(q, n, code_d.data_ptr(), M, dist_d.data_ptr(), cs))
            reps = max(5, args.steps) if Nw < 1e8 else 5
            a.record(st)
            for _ in range(reps):
                L.check(lib.cov_mindist_dev(q, n, code_d.data_ptr(), M, dist_d.data_ptr(), cs))
            b.record(st)
            st.synchronize()
            dt_ms = a.elapsed_time(b) / reps
            for _ in range(2):
                L.check(lib.cov_count_dev(q, n, R, code_d.data_ptr(), M, cnt_d.data_ptr(), cs))
            st.synchronize()
            a.record(st)
            for _ in range(3):
                L.check(lib.cov_count_dev(q, n, R, code_d.data_ptr(), M, cnt_d.data_ptr(), cs))
            b.record(st)
            st.synchronize()
            ct_ms = a.elapsed_time(b) / 3
        unc_dt = int((dist_d > R).sum())
        unc_ct = int((cnt_d[:Nw] == 0).sum())
        if unc_dt != unc_ct:
            raise RuntimeError("distance transform and count disagree at %d^%d: %d vs %d" % (q, n, unc_dt, unc_ct))
        algo = 2 * n * Nw                       # n per-axis uint8 read+write sweeps
        need = dt_pass_bytes(q, n)
        cbytes = 2 * 2 * M * sum(math.comb(n, i) * (q - 1) ** i for i in range(R + 1))
        key = "q%dn%d" % (q, n)
        out[key] = dict(
            q=q, n=n, R=R, M=M, words=Nw, uncovered=unc_dt,
            l2="resident (%.0f MB uint8 array)" % (Nw / 1e6) if Nw < 1.2e8 else
               "HBM-resident (%.0f MB uint8 array > L2)" % (Nw / 1e6),
            dt=dict(ms=dt_ms, words_s=Nw / (dt_ms / 1e3),
                    roofline=dict(bound="hbm", achieved=algo / (dt_ms / 1e3) / 1e9, peak=peak, unit="GB/s",
                                  frac=algo / (dt_ms / 1e3) / 1e9 / peak, algorithmic_bytes=algo,
                                  pass_bytes=need, pass_frac=need / (dt_ms / 1e3) / 1e9 / peak,
                                  peak_source=kind + " (MEASURED_PEAKS.json hbm_gbs)",
                                  note="algorithmic bytes = 2 n N (n axis passes, uint8 read + write); "
                                       "the kernels fuse the passes into %d HBM sweeps, pass_bytes" % (
                                           1 + (need - Nw // 8 - Nw) // (2 * Nw)))),
            count=dict(ms=ct_ms, words_s=Nw / (ct_ms / 1e3),
                       roofline=dict(bound="hbm", achieved=cbytes / (ct_ms / 1e3) / 1e9, peak=peak, unit="GB/s",
                                     frac=cbytes / (ct_ms / 1e3) / 1e9 / peak, algorithmic_bytes=cbytes,
                                     written_bytes=2 * Nw,
                                     note="algorithmic bytes = 2 b_c M V (ball marking RMW, b_c = 2); the "
                                          "tiles mark in shared memory and write each count once (2 N)")))
        del code_d, dist_d, cnt_d
        torch.cuda.empty_cache()
    # CPU baselines of the 7^9 transform / count
    cpu = {}
    try:
        from oracle import pyoracle as po
        cores = host_cores()
        po.linemin(code79[:4], Q, N_, threads=cores)     # warm the library
        t0 = time.perf_counter()
        d_cpu = po.linemin(code79, Q, N_, threads=cores)
        t1 = time.perf_counter()
        cpu["line_min_port"] = dict(value=Q ** N_ / (t1 - t0), unit="words/s", seconds=t1 - t0, cores=cores,
                                    kind="port", sample="the whole 7^9 transform: n uint8 axis line-min passes "
                                                        "(oracle/dtoracle.c orc_linemin), OpenMP over lines")
        if int((d_cpu > R_).sum()) != out["q7n9"]["uncovered"]:
            raise RuntimeError("CPU and GPU transforms disagree")
    except (OSError, ImportError) as e:
        cpu["line_min_port"] = dict(unavailable=str(e))
    vdir = os.path.join(REF_DIR, "cov")
    if os.path.exists(os.path.join(vdir, "verify_cov.py")):
        with tempfile.TemporaryDirectory() as d:
            path = _code_file(d, "c.txt", code79, Q)
            for name, cmd in (("verify_numpy", [sys.executable, os.path.join(vdir, "verify_cov.py"), path, "-q",
                                                 str(Q), "-n", str(N_), "-R", str(R_), "--method", "numpy"]),
                              ("dilate", [sys.executable, os.path.join(vdir, "verify_independent.py"), path, "-q",
                                          str(Q), "-n", str(N_), "-R", str(R_), "--method", "dilate"])):
                t0 = time.perf_counter()
                p = subprocess.run(cmd, capture_output=True, text=True)
                t1 = time.perf_counter()
                cpu[name] = dict(value=Q ** N_ / (t1 - t0), unit="words/s", seconds=t1 - t0, cores=1,
                                 kind="reference", rc=p.returncode,
                                 sample="process wall time, the whole 7^9 verification of the headline code")
    out["cpu_baseline"] = cpu
    return out


CHAIN_CELLS = (   # (label, q, n, R, M, iters per chain): the reference's idle benchmark cells
    ("K6(6,3)@41", 6, 6, 3, 41, 2000),
    ("K6(8,4)@169", 6, 8, 4, 169, 300),
    ("K8(9,4)@2944", 8, 9, 4, 2944, 40),
)
DCT_CELLS = ((7, 9, 4, 1500), (7, 10, 5, 163))

_REF_CHAIN = r"""
import json, sys, time
import numpy as np
sys.path.insert(0, sys.argv[1])
from chain import run, random_code
q, n, R, M, chains, iters, seed = map(int, sys.argv[2:9])
code = random_code(q, n, M, np.random.default_rng(seed))
t0 = time.perf_counter()
r = run(q, n, R, code, nchains=chains, iters=iters, seed=seed)
dt = time.perf_counter() - t0
print(json.dumps(dict(wall_s=dt, iters=int(r["iters"].sum()), best_u_median=float(np.median(r["best_u"])),
                      solved=int(r["solved"].sum()))))
"""

_REF_DCT = r"""
import json, sys, time
import numpy as np
sys.path.insert(0, sys.argv[1])
from dctlib import DCT
q, n, R, M, seed = map(int, sys.argv[2:7])
code = np.random.default_rng(seed).integers(0, q, (M, n), dtype=np.uint8)
e = DCT(q, n, R)
idx = e.word_index(code)
e.recount(idx)
out = {}
for name, fn in (("count", lambda: e.recount(idx)), ("gain_map", e.gain_map)):
    fn()
    t0 = time.perf_counter()
    for _ in range(3):
        fn()
    out[name + "_ms"] = (time.perf_counter() - t0) / 3 * 1e3
e.recount(idx)
out["uncovered"] = e.uncovered()
e.close()
print(json.dumps(out))
"""


def gpu_comparators(args, dev):
    """The reference's own GPU kernels, rebuilt for sm_103a from their copy
    and driven through their own ctypes drivers (cov/gemm2/chain.py,
    cov/gemm2/dctlib.py) in a child process, beside this engine's entry
    points on the same cells and inputs:
      chain      chain_run (chainsolve.cu:370-375) vs cov_chain_run (the same
                 C ABI), 256 chains from one uniform code, wall time of the
                 whole call as the reference's idle benchmark takes it;
      transform  dct_transform code -> cnt (dct.cu:360-411, OUT=2) and the
                 gain map ([cnt==0] -> sum, OUT=1) vs cov_count_dev and
                 cov_lns_map(0).
    chain_kernel's 32-bit atomics on 16-bit counter pairs are misaligned for
    a chain whose counter array starts at an odd word (odd q^n and odd chain
    index), so it is only run on the reference's own even-q cells."""
    import ctypes
    import numpy as np
    import torch
    from coldcase_gb300 import lib as L
    gem = os.path.join(REF_DIR, "cov", "gemm2")
    libs = [os.path.join(gem, f) for f in ("libchain.so", "libdct.so")]
    if not all(os.path.exists(x) for x in libs) and os.path.exists(os.path.join(gem, "chainsolve.cu")):
        subprocess.run(["make", "-s", "-C", os.path.join(HERE, "oracle")] + libs, capture_output=True)
    if not all(os.path.exists(x) for x in libs):
        return dict(unavailable="the reference's GPU sources are not on this host (baseline/_ref)")
    lib = L.load()
    out = dict(chain={}, transform={}, chains=args.comp_chains,
               note="reference kernels compiled here with nvcc -O3 -gencode arch=compute_103a,code=sm_103a")
    for label, q, n, R, M, iters in CHAIN_CELLS:
        seed = 23
        p = subprocess.run([sys.executable, "-c", _REF_CHAIN, gem, str(q), str(n), str(R), str(M),
                            str(args.comp_chains), str(iters), str(seed)], capture_output=True, text=True)
        if p.returncode != 0:
            out["chain"][label] = dict(error=(p.stderr or p.stdout)[-300:])
            continue
        ref = json.loads(p.stdout.strip().splitlines()[-1])
        code = np.random.default_rng(seed).integers(0, q, size=(M, n), dtype=np.uint8)
        rows = np.zeros((args.comp_chains, M, 16), dtype=np.uint8)
        rows[:, :, :n] = code
        best = np.zeros_like(rows)
        bu = np.zeros(args.comp_chains, np.int32)
        sv = np.zeros(args.comp_chains, np.int32)
        io = np.zeros(args.comp_chains, np.int64)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rc = lib.cov_chain_run(q, n, R, M, args.comp_chains, ctypes.c_longlong(iters), ctypes.c_ulonglong(seed),
                               256, L.u8ptr(rows), L.u8ptr(best), bu.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                               sv.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                               io.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
        dt = time.perf_counter() - t0
        L.check(rc, "cov_chain_run")
        ours = dict(wall_s=dt, iters=int(io.sum()), best_u_median=float(np.median(bu)), solved=int(sv.sum()))
        out["chain"][label] = dict(
            iters_per_chain=iters,
            reference=dict(ref, agg_moves_s=ref["iters"] / ref["wall_s"]),
            ours=dict(ours, agg_moves_s=ours["iters"] / ours["wall_s"]),
            speedup=(ours["iters"] / ours["wall_s"]) / (ref["iters"] / ref["wall_s"]))
    for (q, n, R, M) in DCT_CELLS:
        seed = 91
        p = subprocess.run([sys.executable, "-c", _REF_DCT, gem, str(q), str(n), str(R), str(M), str(seed)],
                           capture_output=True, text=True)
        key = "q%dn%dR%d" % (q, n, R)
        if p.returncode != 0:
            out["transform"][key] = dict(error=(p.stderr or p.stdout)[-300:])
            continue
        ref = json.loads(p.stdout.strip().splitlines()[-1])
        code = np.random.default_rng(seed).integers(0, q, (M, n), dtype=np.uint8)
        code_d = torch.from_numpy(code).to(dev)
        cnt_d = torch.empty(q ** n + 1, dtype=torch.int16, device=dev)
        st = torch.cuda.current_stream(dev).cuda_stream
        L.check(lib.cov_count_dev(q, n, R, code_d.data_ptr(), M, cnt_d.data_ptr(), st))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(3):
            L.check(lib.cov_count_dev(q, n, R, code_d.data_ptr(), M, cnt_d.data_ptr(), st))
        torch.cuda.synchronize()
        c_ms = (time.perf_counter() - t0) / 3 * 1e3
        unc = int((cnt_d[: q ** n] == 0).sum())
        del cnt_d, code_d
        from coldcase_gb300.lns import TransformEngine
        te = TransformEngine(q, n, R)
        te.recount(te.word_index(code))
        te.gain_map()
        t0 = time.perf_counter()
        for _ in range(3):
            te.gain_map()
        g_ms = (time.perf_counter() - t0) / 3 * 1e3
        te.close()
        torch.cuda.empty_cache()
        out["transform"][key] = dict(
            M=M, reference=ref, ours=dict(count_ms=c_ms, gain_map_ms=g_ms, uncovered=unc),
            count_speedup=ref["count_ms"] / c_ms, gain_map_speedup=ref["gain_map_ms"] / g_ms,
            note="wall time of each call after a warm-up; the reference's dct_transform ends in "
                 "cudaDeviceSynchronize, cov_count_dev in a stream synchronize")
        if ref["uncovered"] != unc:
            out["transform"][key]["mismatch"] = "uncovered %d (reference) vs %d" % (ref["uncovered"], unc)
    return out


LNS_CELLS = ((7, 9, 4, 1500, 30), (8, 9, 4, 2944, 10))   # (q, n, R, M, rounds)


def lns_bench(args):
    """The transform-engine search (coldcase_gb300.lns) on the big cells.
    fill: the device greedy from no codeword up to M (placements/s, and how
    many words it needed when it covers below M).  rounds: a fixed number
    of ruin-and-recreate rounds at M, or, when the greedy already covers
    with fewer words, at 95% of that count, from the greedy code ruined to
    that size; rounds/s and the uncovered count, the best code checked by
    the GPU verifier (cov_verify)."""
    import numpy as np
    import torch
    from coldcase_gb300 import verify
    from coldcase_gb300.lns import LNS
    out = {}
    for (q, n, R, M, rounds) in LNS_CELLS:
        rounds = args.lns_rounds if args.lns_rounds else rounds
        with LNS(q, n, R, seed=1) as e:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            e.load(np.zeros(0, dtype=np.int64))
            e.recreate(M)
            t1 = time.perf_counter()
            fill = dict(M=M, placements=len(e.code), uncovered=int(e.uncov), seconds=t1 - t0,
                        placements_s=len(e.code) / max(t1 - t0, 1e-9), refreshes=e.stats["refreshes"],
                        exact_counts=e.stats["exact_counts"],
                        covered_with=len(e.code) if e.uncov == 0 else None)
            Mr = M if e.uncov > 0 else int(0.95 * len(e.code))
            if len(e.code) > Mr:
                e.ruin(len(e.code) - Mr, "soft")
            start = int(e.uncov)
            s0 = dict(e.stats)
            t2 = time.perf_counter()
            e.lns(Mr, budget_s=300.0, max_rounds=rounds)
            t3 = time.perf_counter()
            best = e.eng.index_word(e.best_code if e.best_code is not None else e.code)
            unc_v, _ = verify.verify(best, n, q, R, want_witness=False)
            st = e.stats
            out["q%dn%dR%dM%d" % (q, n, R, M)] = dict(
                fill=fill,
                rounds=dict(M=Mr, rounds=st["rounds"], seconds=t3 - t2, rounds_s=st["rounds"] / max(t3 - t2, 1e-9),
                            placements_s=(st["placements"] - s0["placements"]) / max(t3 - t2, 1e-9),
                            uncovered_start=start, uncovered=int(e.best_uncov), verifier_uncovered=int(unc_v),
                            verified=int(unc_v) == int(e.best_uncov), accepted=st["accepted"]))
    return out


def portfolio_bench(args):
    """A portfolio of N chains two ways, on the q6 n9 R4 M700 cell with the
    flags campaign.py passes: N covsearch_gpu processes started together
    (each its own CUDA context, taking turns on the GPU; the sum of their
    own RESULT rates), and the same N chains as one Pool in this process
    (the seeds campaign would give them)."""
    import re
    import torch
    from coldcase_gb300.engine import Pool
    from coldcase_gb300.workloads import uniform_code
    q, n, R, M, N, T = 6, 9, 4, 700, args.portfolio_chains, args.portfolio_s
    cli = os.path.join(HERE, "coldcase_gb300", "bin", "covsearch_gpu")
    rx = re.compile(r"RESULT .* iters=(\d+) .*time=([0-9.]+) ")
    with tempfile.TemporaryDirectory() as d:
        code = uniform_code(q, n, M, 5)
        path = _code_file(d, "seed.txt", code, q)
        procs = [subprocess.Popen([sys.executable, cli, "-q", str(q), "-n", str(n), "-R", str(R), "-M", str(M),
                                   "-t", str(T), "-s", str(1 + w), "--threads", "1", "--in", path,
                                   "--out", os.path.join(d, "w%d.txt" % w), "--quiet"],
                                  stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True) for w in range(N)]
        rates, iters = [], 0
        for p in procs:
            txt, _ = p.communicate()
            m = rx.search(txt or "")
            if m and float(m.group(2)) > 0:
                rates.append(int(m.group(1)) / float(m.group(2)))
                iters += int(m.group(1))
    pool = Pool(N, cluster=8, budget_s=120.0)
    slots = [pool.add(q, n, R, M, code=code, seed=1 + w) for w in range(N)]
    pool.run(50)
    it0 = sum(pool.status(s)["it"] for s in slots)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < min(T, 5.0):
        pool.run(200)
    dt = time.perf_counter() - t0
    moves = sum(pool.status(s)["it"] for s in slots) - it0
    pool.close()
    one = moves / dt
    procs_rate = sum(rates)
    return dict(cell="q6 n9 R4 M700, campaign's flags, one seed code", chains=N,
                processes=dict(moves_s=procs_rate, finished=len(rates), seconds=T,
                               note="sum of each process's RESULT rate (its moves after init / its search time)"),
                one_pool=dict(moves_s=one, cluster=8, seconds=dt),
                pool_over_processes=one / procs_rate if procs_rate else None)


def ctypes_sizeof_status():
    from coldcase_gb300 import lib as L
    import ctypes
    return ctypes.sizeof(L.CovStatus)


def gpu_bench(args, rank, world, dist):
    import numpy as np
    import torch
    from coldcase_gb300 import lib as L
    from coldcase_gb300.engine import Pool, Search
    from coldcase_gb300 import replicas
    from coldcase_gb300.workloads import uniform_code

    L.load(build_if_missing=True)
    dev = torch.device("cuda", torch.cuda.current_device())
    S = args.moves
    seeds = replicas.rank_seeds(BASE_SEED, rank, args.restarts)
    codes = [uniform_code(Q, N_, M_, sd) for sd in seeds]

    # ---------------- batched: device-resident state, events on its stream
    pool = Pool(args.restarts, cluster=args.cluster, budget_s=120.0)
    stream = torch.cuda.Stream(device=dev)
    pool.set_stream(stream.cuda_stream)
    slots = [pool.add(Q, N_, R_, M_, code=codes[i], seed=seeds[i], tabu=TENURE) for i in range(args.restarts)]
    for _ in range(args.warmup):
        pool.run(S)
    it0 = sum(s["it"] for s in pool.status_all(args.restarts))
    prof0 = [pool.prof(sl) for sl in slots]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clk = ClockSampler(torch.cuda.current_device())
    clk.start()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    e_all0, e_all1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e_all0.record(stream)
    for k in range(args.steps):
        evs[k][0].record(stream)
        if args.graph:
            pool.graph_run(S, 1)
        else:
            pool.run_async(S)
        evs[k][1].record(stream)
    e_all1.record(stream)
    stream.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = clk.stop()
    st = pool.status_all(args.restarts)
    moves = sum(s["it"] for s in st) - it0
    errs = [s["status"] for s in st if s["status"] != 0]
    if errs:
        raise RuntimeError("engine status %s" % errs[:4])
    ms = e_all0.elapsed_time(e_all1)
    step_ms = [a.elapsed_time(b) for a, b in evs]
    ms_max, moves_all = replicas.combine(dist, ms, moves, device=dev)
    value = moves_all / (ms_max / 1e3)
    finished = sum(1 for s in st if s["finished"])
    best_unc = [s["best"] for s in st]
    prof1 = [pool.prof(sl) for sl in slots]
    pm = sum(b["planned_moves"] - a["planned_moves"] for a, b in zip(prof0, prof1))
    work = dict(ncw=sum(b["sum_ncw"] - a["sum_ncw"] for a, b in zip(prof0, prof1)) / max(1, pm),
                ul_n=sum(b["sum_ul_n"] - a["sum_ul_n"] for a, b in zip(prof0, prof1)) / max(1, pm))

    # ---------------- e2e: host buffers through the public API.  The host
    # holds the search state between steps as a caller of the covsearch2e
    # CLI does (its --in / --out codes): every step uploads each restart's
    # code from pinned host memory, rebuilds its state on the device, runs
    # --moves moves and reads the current code back (it seeds the next step)
    # with the restarts' status.  The warm-up steps bring the codes to the
    # same phase of the search as the device-timed window.
    e2e = None
    if not args.no_e2e:
        pinned = [torch.from_numpy(c.copy()).pin_memory() for c in codes]
        e_moves, e_t = 0, 0.0
        t_load = t_run = t_read = 0.0
        h2d = sum(int(c.numel()) for c in pinned)
        d2h = args.restarts * M_ * N_ + args.restarts * ctypes_sizeof_status()
        for k in range(args.warmup + args.e2e_steps):
            torch.cuda.synchronize()
            t0 = time.monotonic()
            for i, sl in enumerate(slots):
                pool.load(sl, code=pinned[i].numpy(), seed=seeds[i] + 1 + k)
            t1 = time.monotonic()
            pool.run(S)
            t2 = time.monotonic()
            stt = pool.status_all(args.restarts)
            for i, sl in enumerate(slots):
                pinned[i].numpy()[:] = pool.code(sl)
            t3 = time.monotonic()
            if k < args.warmup:
                continue
            e_t += t3 - t0
            t_load += t1 - t0
            t_run += t2 - t1
            t_read += t3 - t2
            e_moves += sum(x["it"] for x in stt)
        e_t, e_moves = replicas.combine(dist, e_t, e_moves, device=dev)     # slowest rank, all moves
        e2e = dict(value=e_moves / e_t, unit="moves/s", h2d_bytes_per_step=h2d, d2h_bytes_per_step=d2h,
                   note="per step: %d restarts re-seeded from pinned host codes (state build included), %d moves "
                        "each, every current code read back for the next step; %d untimed warm-up steps, then %d "
                        "timed" % (args.restarts, S, args.warmup, args.e2e_steps),
                   ms_per_step=dict(load=1e3 * t_load / args.e2e_steps, run=1e3 * t_run / args.e2e_steps,
                                    read=1e3 * t_read / args.e2e_steps))
    pool.close()

    # ---------------- plain: one instance on the GPU: its cluster, with the
    # commits of its moves shared by helper CTAs on the other SMs (grid help),
    # and its cluster alone
    plain = None
    if not args.no_plain and rank == 0:
        runs = {}
        for help_ in ((args.plain_help, 0) if args.plain_help else (0,)):
            eng = Search(Q, N_, R_, M_, seed=seeds[0], tabu=TENURE, cluster=args.plain_cluster, budget_s=120.0)
            if help_:
                eng.pool.set_param("grid_help", help_)
            eng.load(codes[0])
            ps = torch.cuda.Stream(device=dev)
            eng.pool.set_stream(ps.cuda_stream)
            for _ in range(args.warmup):
                eng.pool.run(args.plain_moves)
            i0 = eng.status()["it"]
            p0 = eng.pool.prof(eng.slot)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(ps)
            for _ in range(args.steps):
                eng.pool.run_async(args.plain_moves)
            b.record(ps)
            ps.synchronize()
            st = eng.status()
            if st["status"] != 0:
                raise RuntimeError("plain engine status %d" % st["status"])
            pm = st["it"] - i0
            p1 = eng.pool.prof(eng.slot)
            # the phase counters are SM cycles: at the clock sampled under the batched leg
            mhz = (clocks.get("sm_mhz") or 2070.0) if isinstance(clocks, dict) else 2070.0
            us = {k: round((p1[k] - p0[k]) / (mhz * pm), 2) for k in eng.pool.PROF_NAMES if p1[k] > p0[k]}
            runs[help_] = dict(value=pm / (a.elapsed_time(b) / 1e3), unit="moves/s", cluster=args.plain_cluster,
                               grid_help=help_, moves=pm, us_per_move=us)
            eng.close()
        plain = dict(runs[args.plain_help])
        if args.plain_help:
            plain["cluster_only"] = runs[0]
            plain["note"] = ("one instance: the leader's serial steps on its cluster, each move's commit shared "
                             "with helper CTAs on the SMs the cluster leaves free")

    # ---------------- the other plain configurations (one instance each)
    plain_cfgs = None
    if not args.no_plain and rank == 0:
        from coldcase_gb300 import workloads
        plain_cfgs = {}
        loose = dict(name="plain q3 n11 R4 M81 tenure0", q=3, n=11, R=4, M=81, tabu=0)
        loose_wide = dict(loose, name="plain q3 n11 R4 M81 tenure0 --wide", wide=True)
        for key, w, cl, mv in (("q6n9_M700", workloads.PLAIN_GPU, 16, 2000),
                               ("q4n6_M420", workloads.PLAIN_CPU, 1, 2000),
                               ("q3n11_M81", loose, 4, 2000),
                               ("q3n11_M81_wide", loose_wide, 4, 2000)):
            eng = Search(w["q"], w["n"], w["R"], w["M"], seed=1, tabu=w["tabu"], cluster=cl, budget_s=120.0,
                         wide=w.get("wide", False))
            eng.load(uniform_code(w["q"], w["n"], w["M"], 1))
            ps = torch.cuda.Stream(device=dev)
            eng.pool.set_stream(ps.cuda_stream)
            eng.pool.run(200)
            i0 = eng.status()["it"]
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(ps)
            eng.pool.run_async(mv)
            b.record(ps)
            ps.synchronize()
            m = eng.status()["it"] - i0
            plain_cfgs[key] = dict(value=m / (a.elapsed_time(b) / 1e3) if m else None, unit="moves/s", moves=m,
                                   cluster=cl, workload=w["name"],
                                   note=None if m == mv else "the search covered after %d moves" % m)
            eng.close()

    # ---------------- coverage words/s: distance transform and count
    cov = None
    if rank == 0 and not args.no_cov:
        cov = coverage_bench(args, codes[0], dev)
    # ---------------- heterogeneous cells: one tuned graph launch
    hetero = None
    if not args.no_hetero:
        from coldcase_gb300 import workloads
        from coldcase_gb300.batch import Batch, tune_batch
        h_rej = []
        cells = replicas.shard(workloads.hetero_cells(count=args.cells * world, rejected=h_rej), rank, world)
        for c in cells:
            c["moves"] = args.cell_moves
        t0 = time.monotonic()
        plan, est, classes = tune_batch(cells)
        t_tune = time.monotonic() - t0
        with Batch(cells, clusters=plan) as b:
            hs = torch.cuda.Stream(device=dev)
            b.pool.set_stream(hs.cuda_stream)
            a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            if dist:
                dist.barrier()
            a0.record(hs)
            if args.cell_segment:
                b.run(segment=args.cell_segment)
            else:
                b.run_async(graph=True)
            a1.record(hs)
            hs.synchronize()
            hms = a0.elapsed_time(a1)
            res = b.results()
            if any(x["status"] != 0 for x in res):
                raise RuntimeError("hetero batch: engine status")
            hmoves = sum(x["iters"] for x in res)
        hms_max, hmoves_all = replicas.combine(dist, hms, hmoves, device=dev)
        hetero = dict(value=hmoves_all / (hms_max / 1e3), unit="moves/s", cells=len(cells) * world,
                      moves_per_cell=args.cell_moves, ms=hms_max, clusters=plan, plan_estimate_s=est,
                      tune_s=t_tune,
                      outside_domain=dict(count=len(h_rej), cells=sorted({(c["q"], c["n"], c["R"], c["M"])
                                                                           for c in h_rej}),
                                          note="draws with M > 65535: outside the reference engine's domain "
                                               "(covsearch2e.c:1117) and this engine's; redrawn, no CPU baseline "
                                               "/ parity unpinned"),
                      launches=("launches of %d moves, clusters widened between them while SMs are spare"
                                % args.cell_segment) if args.cell_segment else
                      "one graph: one persistent kernel per cluster size")

    # ---------------- serving: Poisson arrivals, continuous batching
    served = None
    if not args.no_serve:
        from coldcase_gb300 import workloads
        from coldcase_gb300.serve import Server
        from coldcase_gb300.batch import tune_batch
        s_rej = []
        reqs = replicas.shard(workloads.serve_requests(args.requests * world, lam=args.lam * world,
                                                       seed=2027, rejected=s_rej), rank, world)
        splan, _, _ = tune_batch(reqs)
        with Server(max_slots=256, chunk=args.serve_chunk, clusters=splan) as srv:
            if dist:
                dist.barrier()
            rep = srv.serve(reqs)
            lat = [r["done"] - r["arrival"] for r in srv.done]
        if dist:
            # the whole job: every rank's requests, the slowest rank's wall time
            lats = [None] * world
            dist.all_gather_object(lats, lat)
            lat = [x for part in lats for x in part]
            wall, moves = replicas.combine(dist, rep["wall_s"], rep["moves"], device=dev)
            rep = dict(rep, requests=len(lat), moves=int(moves), wall_s=wall, moves_per_s=moves / wall,
                       p50_s=float(np.percentile(lat, 50)), p99_s=float(np.percentile(lat, 99)))
        served = dict(rep, lam_per_s=args.lam * world, unit="moves/s", value=rep["moves_per_s"], clusters=splan,
                      elastic=True,
                      outside_domain=dict(count=len(s_rej), cells=sorted({(c["q"], c["n"], c["R"], c["M"])
                                                                           for c in s_rej}),
                                          note="requests with M > 65535: outside the reference engine's domain "
                                               "and this engine's; redrawn, no CPU baseline / parity unpinned"))

    # ---------------- quotient search (symsearch) on the big cell K_8(9,4)@940
    quotient = None
    if not args.no_sym:
        from coldcase_gb300.sym import SymPool
        qq, qn, qR, qM = 8, 9, 4, 940
        one = None
        if rank == 0:
            one = {}
            for form, ge in (("cluster", False), ("grid", True)):
                with SymPool(1, cluster=16, budget_s=120.0, grid_eval=ge) as sp:
                    s = sp.add(qq, qn, qR, qM, seed=1000)
                    sp.run(10)
                    t0 = time.perf_counter()
                    sp.run(args.sym_moves)
                    dt = time.perf_counter() - t0
                    st = sp.status(s)
                    if st["status"] != 0:
                        raise RuntimeError("quotient search: engine status %d" % st["status"])
                    phases, _ = sp.prof(s)
                    one[form] = dict(value=args.sym_moves / dt, unit="moves/s", cluster=16, moves=args.sym_moves,
                                     best_red_uncovered=int(st["best"]))
                    if not ge:
                        one[form]["us_per_move"] = {k: round(v / 2070.0, 1) for k, v in phases.items() if v}
            one["grid"]["note"] = "estimates by a grid-wide launch per move, the rest on the cluster"
        seeds = replicas.shard(list(range(1000, 1000 + args.sym_batch * world)), rank, world)
        with SymPool(len(seeds), cluster=args.sym_cluster, budget_s=120.0) as sp:
            slots = [sp.add(qq, qn, qR, qM, seed=sd) for sd in seeds]
            sp.run(10)
            if dist:
                dist.barrier()
            t0 = time.perf_counter()
            sp.run(args.sym_batch_moves)
            dt = time.perf_counter() - t0
            bmoves = sum(sp.status(x)["it"] - 10 for x in slots)
        dt_max, bmoves_all = replicas.combine(dist, dt, bmoves, device=dev)
        quotient = dict(workload="quotient search K_8(9,4)@940 (117 orbits, 8^8 quotient counters), seeds from 1000",
                        unit="moves/s", single=one,
                        batch=dict(value=bmoves_all / dt_max, instances=len(seeds) * world,
                                   cluster=args.sym_cluster, moves=args.sym_batch_moves))

    portfolio = None
    if rank == 0 and not args.no_portfolio:
        portfolio = portfolio_bench(args)

    lns = None
    if rank == 0 and not args.no_lns:
        lns = lns_bench(args)

    comparators = None
    if rank == 0 and not args.no_comparators:
        comparators = gpu_comparators(args, dev)

    return dict(value=value, ms=ms_max, step_ms=step_ms, moves=moves_all, clocks=clocks, e2e=e2e,
                comparators=comparators, lns=lns, portfolio=portfolio,
                plain=plain, cov=cov, finished=finished, best_unc=best_unc, work=work, hetero=hetero,
                served=served, plain_cfgs=plain_cfgs, quotient=quotient)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--moves", type=int, default=1000, help="moves per restart per step")
    ap.add_argument("--restarts", type=int, default=RESTARTS)
    ap.add_argument("--cluster", type=int, default=2, help="CTAs per restart (batched)")
    ap.add_argument("--plain-cluster", type=int, default=16)
    ap.add_argument("--plain-moves", type=int, default=1000)
    ap.add_argument("--plain-help", type=int, default=64,
                    help="helper clusters that share the plain instance's commits (0: its cluster alone)")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--ref-moves", type=int, default=100,
                    help="moves per reference-engine process per step (CPU baselines and the reference arm)")
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--cell-cpu-moves", type=int, default=200,
                    help="moves per shape of the uneven-cells / served CPU baselines")
    ap.add_argument("--no-graph", dest="graph", action="store_false",
                    help="launch each step directly instead of replaying its captured CUDA graph")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cov", action="store_true")
    ap.add_argument("--no-hetero", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--cells", type=int, default=256, help="heterogeneous cells per GPU")
    ap.add_argument("--cell-moves", type=int, default=20000)
    ap.add_argument("--cell-segment", type=int, default=2000,
                    help="moves per launch of the uneven-cells batch (0: the whole batch as one graph)")
    ap.add_argument("--requests", type=int, default=100, help="served requests per GPU")
    ap.add_argument("--lam", type=float, default=100.0, help="request arrival rate per GPU (1/s)")
    ap.add_argument("--serve-chunk", type=int, default=256)
    ap.add_argument("--no-sym", action="store_true", help="skip the quotient-search leg")
    ap.add_argument("--no-comparators", action="store_true",
                    help="skip timing the reference's own GPU kernels beside this engine")
    ap.add_argument("--comp-chains", type=int, default=256, help="chains per comparator cell")
    ap.add_argument("--no-lns", action="store_true", help="skip the transform-engine search leg")
    ap.add_argument("--no-portfolio", action="store_true", help="skip the N-processes-vs-one-pool leg")
    ap.add_argument("--portfolio-chains", type=int, default=8)
    ap.add_argument("--portfolio-s", type=float, default=10.0, help="seconds per portfolio process")
    ap.add_argument("--lns-rounds", type=int, default=0, help="ruin-and-recreate rounds per LNS cell (0: default)")
    ap.add_argument("--sym-moves", type=int, default=300)
    ap.add_argument("--sym-batch", type=int, default=38, help="quotient-search instances per GPU")
    ap.add_argument("--sym-cluster", type=int, default=4)
    ap.add_argument("--sym-batch-moves", type=int, default=200)
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return 0
        r = ref_measure(args.warmup, args.steps, args.ref_moves)
        if r is None:
            r = cpu_measure(args.warmup, args.steps, args.ref_moves)
            r["sample"] += "; the reference engine's sources are not on this host, so this is the oracle port"
        _, _, at = warm_state()
        line = dict(metric=METRIC, value=r["value"], unit="moves/s", n_gpus=args.gpus, steps=args.steps,
                    warmup=args.warmup, ms_per_step=1e3 * r["seconds"] / args.steps, higher_is_better=True,
                    scaling="weak", vs_baseline=None, dtype="int64", data="synthetic: uniform random codes, seeded",
                    impl="reference",
                    config=dict(workload=workload_name(args.restarts, args.moves), q=Q, n=N_, R=R_, M=M_,
                                tenure=TENURE, window="moves %d.. of each restart (its code after %d moves)"
                                                      % (at + 1, at), cpu_sample=r["sample"]),
                    cpu_baseline=dict(value=r["value"], unit="moves/s", cores=r["cores"], kind=r["kind"],
                                      sample=r["sample"]),
                    e2e=dict(value=r["value"], unit="moves/s", h2d_bytes_per_step=0, d2h_bytes_per_step=0))
        print(json.dumps(line))
        return 0

    cpu = None
    sym_cpu = None
    cells_cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        # before any GPU call: the reference engine and the oracle port on
        # this host's cores, both from the restarts' codes at the start of
        # the timed window
        cpu = ref_measure(1, args.cpu_steps, args.ref_moves)
        port = cpu_measure(1, args.cpu_steps, args.ref_moves)
        if cpu is None:
            cpu = port
        cpu["port"] = dict(value=port["value"], cores=port["cores"], sample=port["sample"])
        if not args.no_sym:
            sym_cpu = sym_cpu_measure(4)
        cells_cpu = cells_cpu_measure(args, world)

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as tdist
        tdist.init_process_group("nccl")
        dist = tdist
    r = gpu_bench(args, rank, world, dist)
    if rank == 0:
        peak, peak_kind = measured_peaks()
        w = r["work"]
        bpm = algo_bytes_per_move(Q, N_, R_, M_, w["ncw"], w["ul_n"])
        dpm = design_bytes_per_move(Q, N_, R_, M_, w["ul_n"])
        launch_ms = statistics.mean(r["step_ms"])
        moves_per_launch = r["moves"] / max(1, args.steps) / max(1, world)
        achieved = bpm * moves_per_launch / (launch_ms / 1e3) / 1e9
        d_achieved = dpm * moves_per_launch / (launch_ms / 1e3) / 1e9
        tpm = profiled_traffic()
        line = dict(
            metric=METRIC, value=r["value"], unit="moves/s", n_gpus=world, steps=args.steps, warmup=args.warmup,
            ms_per_step=r["ms"] / args.steps, higher_is_better=True, scaling="weak", vs_baseline=None,
            dtype="int32", data="synthetic: uniform random codes, seeded (numpy default_rng)",
            config=dict(workload=workload_name(args.restarts, args.moves), q=Q, n=N_, R=R_, M=M_,
                        tenure=TENURE, restarts_per_gpu=args.restarts, moves_per_step=args.moves,
                        cluster=args.cluster, graph=bool(args.graph),
                        l2="inputs larger than L2: 64 x 161 MB counter arrays per GPU"),
            roofline=dict(bound="hbm", achieved=achieved, peak=peak, unit="GB/s", frac=achieved / peak,
                          traffic=(tpm * moves_per_launch) if tpm else None,
                          peak_source=peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
                          algorithmic_bytes_per_move=bpm, mean_candidate_codewords=w["ncw"],
                          mean_list_length=w["ul_n"], moves_per_launch=moves_per_launch,
                          launch_ms=launch_ms, kernel="cov_run_kernel",
                          design=dict(bytes_per_move=dpm, achieved=d_achieved, frac=d_achieved / peak,
                                      note="bytes this engine's own algorithm touches per move")),
            clocks=r["clocks"],
            e2e=r["e2e"],
            gpu_launches=2 * args.steps,
            plain=r["plain"],
            batched_over_plain=(r["value"] / world / r["plain"]["value"]) if r["plain"] else None,
            plain_configs=r["plain_cfgs"],
            hetero=r["hetero"],
            served=r["served"],
            served_over_plain=(r["served"]["value"] / r["plain"]["value"])
            if r["served"] and r["plain"] else None,
            coverage=r["cov"],
            quotient=r["quotient"],
            gpu_comparators=r["comparators"],
            lns=r["lns"],
            portfolio=r["portfolio"],
            finished_restarts=r["finished"],
        )
        if r["quotient"] and sym_cpu:
            line["quotient"]["cpu_baseline"] = sym_cpu
        if cells_cpu:
            if line["hetero"] and "hetero" in cells_cpu:
                line["hetero"]["cpu_baseline"] = cells_cpu["hetero"]
            if line["served"] and "served" in cells_cpu:
                line["served"]["cpu_baseline"] = cells_cpu["served"]
        if cpu:
            line["cpu_baseline"] = dict(value=cpu["value"], unit="moves/s", cores=cpu["cores"], kind=cpu["kind"],
                                        sample=cpu["sample"], port=cpu.get("port"))
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
