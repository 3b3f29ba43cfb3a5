"""The sliding-moment rewrite (kunquant_gb300/slide.py) on CPU: every
expanded ReduceAdd equals its loop, evaluated in float64 on random windows,
and the rewritten specs still plan into levels."""
import numpy as np
import pytest

from kunquant_gb300 import contraction, slide
from kunquant_gb300.graph import predefined_spec


def _eval_body(ops, i, win, inv):
    """Value of loop-body op i over a window: IterValue -> the source's
    window values, an op from outside the loop -> its invariant value."""
    op = ops[i]
    if op.get("p", -1) < 0:
        return inv[i]
    k = op["k"]
    if k == "IterValue":
        return win[op["in"][1]]
    a = _eval_body(ops, op["in"][0], win, inv)
    b = _eval_body(ops, op["in"][1], win, inv)
    return {"Add": a + b, "Sub": a - b, "Mul": a * b}[k]


def _eval_slide(op, win, inv):
    ns = op["nsrc"]
    srcs, invs = op["in"][:ns], op["in"][ns:]
    total = 0.0
    for c, se, ie in op["terms"]:
        m = np.ones_like(next(iter(win.values())))
        for x, e in zip(srcs, se):
            m = m * win[x] ** e
        t = c * m.sum()
        for x, e in zip(invs, ie):
            t *= inv[x] ** e
        total += t
    return total


@pytest.mark.parametrize("key", ["alpha158_f32", "alpha101_f32"])
def test_expansion_equals_the_loop(key):
    spec = predefined_spec(key)
    rng = np.random.default_rng(3)
    checked = 0
    for st in spec["stages"]:
        if st["kind"] != "ts":
            continue
        ops = st["ops"]
        new_ops, n, remap = slide._rewrite_stage(ops)
        if not n:
            continue
        back = {v: k for k, v in remap.items()}
        for r in [j for j, o in enumerate(ops) if o["k"] == "ReduceAdd"]:
            sop = new_ops[remap[r]]
            if sop["k"] != "SlideReduce":
                continue  # a loop chain the rewrite left alone
            w = ops[contraction.reduction_loop(ops, r)]["window"]
            assert sop["window"] == w
            win = {x: rng.normal(50, 10, w) for x in range(len(ops))}
            inv = {x: rng.normal(50, 10) for x in range(len(ops))}
            want = _eval_body(ops, ops[r]["in"][0], win, inv).sum()
            got = _eval_slide(sop, {x: win[back[x]] for x in sop["in"][:sop["nsrc"]]},
                              {x: inv[back[x]] for x in sop["in"][sop["nsrc"]:]})
            assert got == pytest.approx(want, rel=1e-9, abs=1e-6), (r, sop)
            checked += 1
    assert checked >= (40 if key.startswith("alpha158") else 150)


@pytest.mark.parametrize("key", ["alpha158_slide_f32", "alpha101_slide_f32"])
def test_slide_specs_plan_and_generate(key, tmp_path):
    from kunquant_gb300 import codegen
    spec = predefined_spec(key)
    assert spec["form"] == "slide" and spec["slide_rewritten"] > 0
    assert not any(o["k"] == "ReduceAdd" for st in spec["stages"] for o in st["ops"])
    paths = codegen.generate_module(spec, str(tmp_path), tag=spec["name"])
    src = "".join(open(p).read() for p in paths)
    # the window moments are two-float sliding sums in time-chunked scans
    assert "kun::df_acc_prod(" in src and "const long long tw = t0 >" in src
