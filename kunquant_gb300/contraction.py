"""Multiply-add contraction plan of the reference CPU build.

KunQuant JIT-compiles its stage code with GCC (``KunQuant/jit/cfake.py:88-114``,
``-std=c++11 -O3 -mfma``).  In C++ mode GCC contracts a multiplication into a
fused multiply-add when every use of the product is an addition or a
subtraction in the same basic block.  To return the reference's exact bits the
GPU code must fuse the same products and no others (everything else is built
with ``-fmad=false``).  This module decides, per stage, which ops are fused.

Basic blocks of the generated stage code (``KunQuant/passes/CodegenCpp.py``):
the body of every back-window loop is one block; at the top level a block ends
at every back-window loop and after every template that branches on the time
index (a windowed read of an input/output buffer, skip-list updates).

GCC also unrolls small back-window loops completely; the first step of a Kahan
sum then sees constant zero state and its product is fused twice.  Whether a
loop is unrolled follows GCC's limits (at most 16 peeled iterations and about
200 statements after a 2/3 discount) with a per-op size estimate calibrated
against the reference build.
"""
from typing import Dict, List, Tuple

ADDITIVE = {"Add", "Sub", "AddConst", "SubConst", "ReduceAdd"}
PRODUCTS = {"Mul", "MulConst"}
_BUFFER_SOURCES = {"Input", "Output"}
UNROLL_MAX_TRIPS = 17
UNROLL_SIZE_BUDGET = 300.0
_RED_SIZE = {"ReduceAdd": 4, "ReduceMul": 1, "ReduceMin": 3, "ReduceMax": 3,
             "ReduceArgMax": 6, "ReduceArgMin": 6, "ReduceRank": 7, "ReduceDecayLinear": 2}


def reduction_loop(ops: List[dict], r: int) -> int:
    src = ops[r]["in"][0]
    return src if ops[src]["k"] == "ForeachBackWindow" else ops[src].get("p", -1)


def _basic_blocks(ops: List[dict]) -> list:
    bb = [None] * len(ops)
    cur = 0
    for i, op in enumerate(ops):
        p = op.get("p", -1)
        if p >= 0:
            bb[i] = ("loop", p)
            continue
        k = op["k"]
        if k == "ForeachBackWindow":
            cur += 1
            bb[i] = cur
            cur += 1
            continue
        bb[i] = cur
        branches = (k == "BackRef" or k.startswith("SkipList") or (
            k in ("FastWindowedSum", "WindowedLinearRegression")
            and ops[op["in"][0]]["k"] in _BUFFER_SOURCES))
        if branches:
            cur += 1
    for i, op in enumerate(ops):
        if op["k"] == "ReduceAdd":
            bb[i] = ("loop", reduction_loop(ops, i))
    return bb


def plan(ops: List[dict]) -> Dict[int, Tuple[int, int]]:
    """{use op index: (input position, product op index)} for fused products."""
    n = len(ops)
    bb = _basic_blocks(ops)
    users = [[] for _ in range(n)]
    for i, op in enumerate(ops):
        for j, v in enumerate(op["in"]):
            users[v].append((i, j))
    converted = set()
    out = {}
    for i, op in enumerate(ops):
        if op["k"] not in PRODUCTS or not users[i]:
            continue
        ok = True
        for u, j in users[i]:
            k = ops[u]["k"]
            if k not in ADDITIVE or u in converted or bb[u] != bb[i]:
                ok = False
            elif k == "ReduceAdd" and j != 0:
                ok = False
            elif k in ("Add", "Sub") and ops[u]["in"][0] == ops[u]["in"][1]:
                ok = False
            if not ok:
                break
        if ok:
            for u, j in users[i]:
                out[u] = (j, i)
                converted.add(u)
    return out


def _prev_loop(ops, loop):
    for j in range(loop - 1, -1, -1):
        if ops[j]["k"] == "ForeachBackWindow":
            return j
    return None


def loop_body_size(ops: List[dict], loop: int) -> float:
    size = 2.0
    if ops[loop].get("copy_prev_body"):
        prev = _prev_loop(ops, loop)
        if prev is not None:
            size += loop_body_size(ops, prev) - 2.0
    for j, q in enumerate(ops):
        if q.get("p", -1) == loop:
            if q["k"] == "IterValue":
                size += 4.5 if ops[q["in"][1]]["k"] in _BUFFER_SOURCES else 6.0
            else:
                size += 1.0
        elif q["k"] in _RED_SIZE and reduction_loop(ops, j) == loop:
            size += _RED_SIZE[q["k"]]
    return size


def loop_unrolled(ops: List[dict], loop: int) -> bool:
    trips = ops[loop]["window"] - ops[loop].get("segment_end", 0)
    if trips > UNROLL_MAX_TRIPS:
        return False
    return trips * loop_body_size(ops, loop) <= UNROLL_SIZE_BUDGET


def regression_shares_square(ops: List[dict], i: int) -> bool:
    """cur*cur of a regression is CSE'd with another regression on the same
    input of the stage; the shared product spans blocks and is not fused."""
    src = ops[i]["in"][0]
    return sum(1 for q in ops if q["k"] == "WindowedLinearRegression" and q["in"][0] == src) > 1
