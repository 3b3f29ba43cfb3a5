"""The sliding-moment form of an fp32 module spec (form "slide").

The reference's fp32 build computes a windowed variance, covariance or
correlation in two passes (``KunQuant/ops/CompOp.py:225-234, 270-281,
307-324``): the window mean from a running sum, then a back-window loop
``ReduceAdd((x - mean_x) * (y - mean_y))`` -- O(window) work per output, in an
order that only a sequential loop reproduces.  This form is not bound to that
order; it is scored against the fp64 build instead.

A ``ReduceAdd`` whose loop body is a polynomial of degree <= 2 in the window
values (``IterValue``), with coefficients that are loop invariants (the
means), is expanded:

    sum_i (x_i - a)(y_i - b) = S[xy] - b S[x] - a S[y] + a b S[1]

and replaced by one ``SlideReduce`` op.  Its window sums ``S[m]`` of the
monomials m are sliding sums (add the new row, subtract the row leaving the
window) kept in two-float compensated fp32 with exact products, and the
polynomial is evaluated in the same arithmetic, so the cancellation between
its terms costs no fp32 precision.  NaN semantics are the loop's: the output
is NaN while any row of the window has a NaN operand (rows before the run
start count as NaN, as ``getWindow`` reads them, ``cpp/Kun/Ops.hpp:87-92``).

Only whole loop chains (loops merged by ``merge_loops``) whose reductions are
all such ``ReduceAdd``s are rewritten; any other loop is kept as it is.

``SlideReduce`` op: ``{"k": "SlideReduce", "in": [source series...,
invariants...], "p": -1, "window": w, "nsrc": number of sources, "terms":
[[coefficient, [exponent per source], [exponent per invariant]], ...]}``.
"""
from fractions import Fraction
from typing import Dict, List, Optional, Tuple

from . import contraction

# polynomial: {(source exponents, invariant exponents): Fraction}
Poly = Dict[Tuple[Tuple[int, ...], Tuple[int, ...]], Fraction]


class _Expand:
    def __init__(self, ops: List[dict]):
        self.ops = ops
        self.srcs: List[int] = []
        self.invs: List[int] = []

    def _var(self, lst: List[int], x: int) -> int:
        if x not in lst:
            lst.append(x)
        return lst.index(x)

    def poly(self, i: int) -> Optional[Poly]:
        """Polynomial of body op i, in variables keyed by position in
        self.srcs / self.invs (tuples are padded later)."""
        op = self.ops[i]
        k = op["k"]
        if op.get("p", -1) < 0:
            # a value from outside the loop: an invariant
            return {((), ((self._var(self.invs, i), 1),)): Fraction(1)}
        if k == "IterValue":
            return {(((self._var(self.srcs, op["in"][1]), 1),), ()): Fraction(1)}
        if k in ("Add", "Sub", "Mul"):
            a = self.poly(op["in"][0])
            b = self.poly(op["in"][1])
            if a is None or b is None:
                return None
            if k == "Add":
                return _padd(a, b, 1)
            if k == "Sub":
                return _padd(a, b, -1)
            return _pmul(a, b)
        return None


def _canon(m):
    d: Dict[int, int] = {}
    for v, e in m:
        d[v] = d.get(v, 0) + e
    return tuple(sorted((v, e) for v, e in d.items() if e))


def _padd(a: Poly, b: Poly, sign: int) -> Poly:
    out = dict(a)
    for k, c in b.items():
        out[k] = out.get(k, Fraction(0)) + sign * c
    return {k: c for k, c in out.items() if c != 0}


def _pmul(a: Poly, b: Poly) -> Poly:
    out: Poly = {}
    for (sa, ia), ca in a.items():
        for (sb, ib), cb in b.items():
            k = (_canon(sa + sb), _canon(ia + ib))
            out[k] = out.get(k, Fraction(0)) + ca * cb
    return {k: c for k, c in out.items() if c != 0}


def _chains(ops: List[dict]) -> List[List[int]]:
    chains, cur = [], []
    for i, op in enumerate(ops):
        if op["k"] != "ForeachBackWindow":
            continue
        if op.get("copy_prev_body") and cur:
            cur.append(i)
        else:
            cur = [i]
            chains.append(cur)
    return chains


def _rewrite_stage(ops: List[dict]) -> Tuple[List[dict], int, Dict[int, int]]:
    """(rewritten ops, number of ReduceAdds rewritten, old index -> new
    index of every op kept)."""
    n = len(ops)
    red_loop = {j: contraction.reduction_loop(ops, j) for j in range(n)
                if ops[j]["k"].startswith("Reduce")}
    new_ops = [dict(op) for op in ops]
    dead = set()
    rewritten = 0
    for chain in _chains(ops):
        reds = [j for j, lp in red_loop.items() if lp in chain]
        if not reds or any(ops[j]["k"] != "ReduceAdd" for j in reds):
            continue
        repl = {}
        for r in reds:
            ex = _Expand(ops)
            p = ex.poly(ops[r]["in"][0])
            if p is None or not p:
                break
            if any(sum(e for _, e in s) > 2 for s, _ in p):
                break
            ns, ni = len(ex.srcs), len(ex.invs)
            terms = []
            for (s, iv), c in sorted(p.items()):
                if c.denominator != 1 or abs(c.numerator) > 1 << 20:
                    break
                se = [0] * ns
                for v, e in s:
                    se[v] = e
                ie = [0] * ni
                for v, e in iv:
                    ie[v] = e
                terms.append([int(c), se, ie])
            else:
                repl[r] = {"k": "SlideReduce", "in": ex.srcs + ex.invs, "p": -1,
                           "window": int(ops[red_loop[r]]["window"]), "nsrc": ns, "terms": terms}
                continue
            break
        if len(repl) != len(reds):
            continue
        for r, op in repl.items():
            new_ops[r] = op
        rewritten += len(repl)
        body = {j for j, op in enumerate(ops) if op.get("p", -1) in chain}
        dead |= set(chain) | body
    if not dead:
        return new_ops, 0, {i: i for i in range(n)}
    # drop the dead loops and bodies; renumber the references
    keep = [i for i in range(n) if i not in dead]
    remap = {old: new for new, old in enumerate(keep)}
    out = []
    for old in keep:
        op = new_ops[old]
        op["in"] = [remap[x] for x in op["in"]]
        if op.get("p", -1) >= 0:
            op["p"] = remap[op["p"]]
        out.append(op)
    return out, rewritten, remap


def rewrite(spec: dict) -> dict:
    """The sliding-moment form of an fp32 batch module spec: two-pass window
    moments become ``SlideReduce`` ops (in place, a new dict); the running
    sums take two-float compensated fp32 (``accum: df32`` on the rolling
    states) and the scans run in time chunks with a warm-up of one window."""
    if spec["dtype"] != "float":
        raise RuntimeError("the slide form is an fp32 form")
    if spec["output_layout"] == "STREAM":
        raise RuntimeError("the slide form is a batch form")
    out = dict(spec)
    out["stages"] = []
    total = 0
    for st in spec["stages"]:
        st = dict(st)
        if st["kind"] == "ts":
            st["ops"], k, _ = _rewrite_stage(st["ops"])
            total += k
        out["stages"].append(st)
    out.update({"form": "slide", "accum": "df32", "accum_scope": "rolling", "slide_rewritten": total})
    return out
