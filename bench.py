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
def _cpu_worker(args):
    """One restart on the oracle (single thread): untimed init, then the
    timed steps; each step starts at a shared barrier."""
    idx, steps, moves, barrier = args
    sys.path.insert(0, HERE)
    from oracle.pyoracle import Oracle
    from coldcase_gb300.workloads import instance_seed, uniform_code
    seed = instance_seed(BASE_SEED, idx)
    o = Oracle(Q, N_, R_, M_, seed=seed, tabu=TENURE, threads=1)
    o.init(uniform_code(Q, N_, M_, seed))
    out = []
    for _ in range(steps):
        barrier.wait()
        t0 = time.monotonic()
        made = o.run(moves)
        out.append((made, t0, time.monotonic()))
    o.close()
    return out


def cpu_measure(warmup, steps, moves, cores=None):
    """Aggregate moves/s of `cores` concurrent single-thread restarts."""
    if cores is None:
        cores = len(os.sched_getaffinity(0))
    subprocess.run(["make", "-s", "-C", os.path.join(HERE, "oracle")], check=True)
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    barrier = mgr.Barrier(cores)
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_worker, [(i, warmup + steps, moves, barrier) for i in range(cores)])
    mgr.shutdown()
    rates = []
    total_m, total_t = 0, 0.0
    for k in range(warmup, warmup + steps):
        m = sum(r[k][0] for r in res)
        t = max(r[k][2] for r in res) - min(r[k][1] for r in res)
        total_m += m
        total_t += t
        rates.append(m / t)
    return dict(value=total_m / total_t, cores=cores, moves=total_m, seconds=total_t,
                sample="%d concurrent restarts x %d moves x %d steps (after untimed init)"
                       % (cores, moves, steps))


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

    # ---------------- e2e: host buffers through the public API
    e2e = None
    if not args.no_e2e:
        pinned = [torch.from_numpy(c).pin_memory() for c in codes]
        e_moves, e_t = 0, 0.0
        t_load = t_run = t_read = 0.0
        h2d = sum(int(c.numel()) for c in pinned)
        d2h = args.restarts * M_ * N_
        for k in range(args.e2e_steps):
            torch.cuda.synchronize()
            t0 = time.monotonic()
            for i, sl in enumerate(slots):
                pool.load(sl, code=pinned[i].numpy(), seed=seeds[i] + 1 + k)
            t1 = time.monotonic()
            pool.run(S)
            t2 = time.monotonic()
            stt = pool.status_all(args.restarts)
            for sl in slots:
                pool.best(sl)
            t3 = time.monotonic()
            e_t += t3 - t0
            t_load += t1 - t0
            t_run += t2 - t1
            t_read += t3 - t2
            e_moves += sum(s["it"] for s in stt)
        e_t, e_moves = replicas.combine(dist, e_t, e_moves, device=dev)     # slowest rank, all moves
        e2e = dict(value=e_moves / e_t, unit="moves/s", h2d_bytes_per_step=h2d,
                   d2h_bytes_per_step=d2h + args.restarts * 72,
                   note="per step: %d restarts re-seeded from pinned host codes (state build included), "
                        "%d moves each from the fresh codes, every best code read back" % (args.restarts, S),
                   ms_per_step=dict(load=1e3 * t_load / args.e2e_steps, run=1e3 * t_run / args.e2e_steps,
                                    read=1e3 * t_read / args.e2e_steps))
    pool.close()

    # ---------------- plain: one instance, one wide cluster, same GPU
    plain = None
    if not args.no_plain and rank == 0:
        eng = Search(Q, N_, R_, M_, seed=seeds[0], tabu=TENURE, cluster=args.plain_cluster, budget_s=120.0)
        eng.load(codes[0])
        ps = torch.cuda.Stream(device=dev)
        eng.pool.set_stream(ps.cuda_stream)
        for _ in range(args.warmup):
            eng.pool.run(args.plain_moves)
        i0 = eng.status()["it"]
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(ps)
        for _ in range(args.steps):
            eng.pool.run_async(args.plain_moves)
        b.record(ps)
        ps.synchronize()
        pm = eng.status()["it"] - i0
        plain = dict(value=pm / (a.elapsed_time(b) / 1e3), unit="moves/s", cluster=args.plain_cluster,
                     moves=pm)
        eng.close()

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
        lib = L.load()
        code_d = torch.from_numpy(codes[0]).to(dev)
        Nw = Q ** N_
        dist_d = torch.empty(Nw, dtype=torch.uint8, device=dev)
        cnt_d = torch.empty(Nw + 1, dtype=torch.int16, device=dev)
        cs = torch.cuda.current_stream(dev).cuda_stream
        for _ in range(3):
            L.check(lib.cov_mindist_dev(Q, N_, code_d.data_ptr(), M_, dist_d.data_ptr(), cs))
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = max(5, args.steps)
        a.record()
        for _ in range(reps):
            L.check(lib.cov_mindist_dev(Q, N_, code_d.data_ptr(), M_, dist_d.data_ptr(), cs))
        b.record()
        torch.cuda.synchronize()
        dt_ms = a.elapsed_time(b) / reps
        for _ in range(2):
            L.check(lib.cov_count_dev(Q, N_, R_, code_d.data_ptr(), M_, cnt_d.data_ptr(), cs))
        torch.cuda.synchronize()
        a.record()
        for _ in range(3):
            L.check(lib.cov_count_dev(Q, N_, R_, code_d.data_ptr(), M_, cnt_d.data_ptr(), cs))
        b.record()
        torch.cuda.synchronize()
        ct_ms = a.elapsed_time(b) / 3
        unc_dt = int((dist_d > R_).sum())
        unc_ct = int((cnt_d[:Nw] == 0).sum())
        if unc_dt != unc_ct:
            raise RuntimeError("distance transform and count disagree: %d vs %d" % (unc_dt, unc_ct))
        cov = dict(dt_words_s=Nw / (dt_ms / 1e3), dt_ms=dt_ms, count_words_s=Nw / (ct_ms / 1e3), count_ms=ct_ms,
                   dt_traffic_bytes=int(Nw * 3.25), uncovered=unc_dt)
    # ---------------- heterogeneous cells: one tuned graph launch
    hetero = None
    if not args.no_hetero:
        from coldcase_gb300 import workloads
        from coldcase_gb300.batch import Batch, tune_batch
        cells = replicas.shard(workloads.hetero_cells(count=args.cells * world), rank, world)
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
                      launches=("launches of %d moves, clusters widened between them while SMs are spare"
                                % args.cell_segment) if args.cell_segment else
                      "one graph: one persistent kernel per cluster size")

    # ---------------- serving: Poisson arrivals, continuous batching
    served = None
    if not args.no_serve:
        from coldcase_gb300 import workloads
        from coldcase_gb300.serve import Server
        from coldcase_gb300.batch import tune_batch
        reqs = replicas.shard(workloads.serve_requests(args.requests * world, lam=args.lam * world,
                                                       seed=2027), rank, world)
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
                      elastic=True)

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

    return dict(value=value, ms=ms_max, step_ms=step_ms, moves=moves_all, clocks=clocks, e2e=e2e,
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
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-moves", type=int, default=12)
    ap.add_argument("--cpu-steps", type=int, default=4)
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
        r = cpu_measure(args.warmup, args.steps, args.cpu_moves)
        line = dict(metric=METRIC, value=r["value"], unit="moves/s", n_gpus=args.gpus, steps=args.steps,
                    warmup=args.warmup, ms_per_step=1e3 * r["seconds"] / args.steps, higher_is_better=True,
                    scaling="weak", vs_baseline=None, dtype="int64", data="synthetic: uniform random codes, seeded",
                    impl="reference",
                    config=dict(workload=workload_name(args.restarts, args.moves), q=Q, n=N_, R=R_, M=M_,
                                tenure=TENURE, cpu_sample=r["sample"]),
                    cpu_baseline=dict(value=r["value"], unit="moves/s", cores=r["cores"], kind="port",
                                      sample=r["sample"]),
                    e2e=dict(value=r["value"], unit="moves/s", h2d_bytes_per_step=0, d2h_bytes_per_step=0))
        print(json.dumps(line))
        return 0

    cpu = None
    sym_cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_measure(1, args.cpu_steps, args.cpu_moves)   # before any GPU call
        if not args.no_sym:
            sym_cpu = sym_cpu_measure(4)

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
            finished_restarts=r["finished"],
        )
        if r["quotient"] and sym_cpu:
            line["quotient"]["cpu_baseline"] = sym_cpu
        if cpu:
            line["cpu_baseline"] = dict(value=cpu["value"], unit="moves/s", cores=cpu["cores"], kind="port",
                                        sample=cpu["sample"])
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
