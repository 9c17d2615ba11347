"""Helpers shared by the tests."""
import numpy as np

DIG = "0123456789abcdefghijklmnopqrstuvwxyz"


def code_from_text(text, n):
    rows = [[DIG.index(c) for c in line.strip()] for line in text.splitlines() if line.strip()]
    return np.array(rows, dtype=np.uint8).reshape(-1, n)


def text_from_code(code):
    return "".join("".join(DIG[int(v)] for v in row) + "\n" for row in code)


def oracle_run(run, threads=1):
    """Replay one golden run on the oracle; returns (oracle, trace)."""
    from oracle.pyoracle import Oracle
    o = Oracle(run["q"], run["n"], run["R"], run["M"], seed=run["seed"], tabu=run["tabu"],
               kick=run["kick"], stall=run["stall"], threads=threads, wide=run.get("wide", False),
               fix0=run.get("fix0", False), sa=run.get("sa"), noise=run.get("noise", 0),
               upick=run.get("upick", False), ucache=run.get("ucache", False))
    code = code_from_text(run["code"], run["n"]) if run["code"] else None
    o.init(code, random_init=run["random_init"])
    tr = o.run(run["iters"], trace=True)
    return o, tr


def sym_text(rep, q):
    """symsearch's --out file: orbit by orbit, its q words (j, e + j)."""
    return "".join(DIG[j] + "".join(DIG[(int(x) + j) % q] for x in e) + "\n" for e in rep for j in range(q))


def sym_oracle_run(run, moves=None):
    """Replay one golden quotient-search run on the oracle: (oracle, trace)."""
    from oracle.pyoracle import SymOracle
    o = SymOracle(run["q"], run["n"], run["R"], run["M"], orbits=run["orbits"], seed=run["seed"],
                  kick=run["kick"], stall=run["stall"])
    o.init()
    tr = o.run(run["ref"]["iters"] if moves is None else moves, trace=True)
    return o, tr
