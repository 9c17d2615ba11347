"""Replica sharding on two gloo ranks (CPU): disjoint instance seeds, every
cell owned by exactly one rank, the max-time / sum-of-units summary, and
each rank's instances advanced on the oracle independently of the other."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as tdist
import torch.multiprocessing as tmp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    from coldcase_gb300 import replicas, workloads
    from oracle.pyoracle import Oracle
    seeds = replicas.rank_seeds(1, rank, 3)
    cells = replicas.shard(workloads.hetero_cells(count=12), rank, world)
    moves = 0
    for sd in seeds:
        o = Oracle(4, 6, 1, 420, seed=sd, tabu=10)
        o.init(workloads.uniform_code(4, 6, 420, sd))
        o.run(50)
        moves += o.iters()
    ms = 10.0 + rank
    got = replicas.combine(tdist, ms, moves)
    allseeds = [None] * world
    tdist.all_gather_object(allseeds, seeds)
    allcells = [None] * world
    tdist.all_gather_object(allcells, [c["seed"] for c in cells])
    tot = [None] * world
    tdist.all_gather_object(tot, moves)
    if rank == 0:
        out.put(dict(combined=got, seeds=allseeds, cells=allcells, moves=tot))
    tdist.barrier()
    tdist.destroy_process_group()


def test_two_rank_replicas():
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    s0, s1 = res["seeds"]
    assert not set(s0) & set(s1)
    c0, c1 = res["cells"]
    assert not set(c0) & set(c1) and len(c0) + len(c1) == 12
    ms, units = res["combined"]
    assert ms == 11.0 and units == sum(res["moves"])
