"""The interior instance of a vector-form kernel body reads rows with no
bounds test.  A launch takes it only for tiles with t0 >= WMAX and
t1 + FWD <= length (the constants in the kernel's entry point); such a tile
is a whole tile, t1 = t0 + tile, and tiles are multiples of 4 (the generated
defaults, checked here, and the tuner's candidates), so with U rows per
thread (U dividing 4) t runs over t0, t0 + U, ..., t1 - U.  This checks, on
the generated sources of the shipped modules, that every row such a body
reads lies inside [0, length) under that condition: for a read at row
t + off, -off <= WMAX and t1 - U + off <= t1 + FWD - 1."""
import re

import pytest

from kunquant_gb300 import codegen
from kunquant_gb300.graph import predefined_spec

READ = re.compile(r"kun::ldw<KE>\(b\d+, st\d+, \(long long\)\(([^)]*)\), length\)")
LOOP = re.compile(r"for \(int iter = (\d+); iter >= (\d+); --iter\)")
# the shared run of a window extreme (kun::RExt): d counts down, row t - d
DLOOP = re.compile(r"for \(int d = (\d+); d >= (\d+); --d\)")


def _offsets(expr, U, loop, dloop=None):
    """(min, max) of expr - t.  The edge rows of a window extreme are read
    for k < U - 1."""
    m = re.fullmatch(r"t \+ u", expr)
    if m:
        return 0, U - 1
    m = re.fullmatch(r"t \+ u - (\d+)", expr)
    if m:
        k = int(m.group(1))
        return -k, U - 1 - k
    m = re.fullmatch(r"t \+ (\d+) - iter", expr)
    if m:
        assert loop is not None, expr
        n = int(m.group(1))
        a, b = loop
        return n - a, n - b
    if expr == "t - d":
        assert dloop is not None, expr
        return -dloop[0], -dloop[1]
    m = re.fullmatch(r"t \+ 1 - (\d+) \+ k", expr)
    if m:
        w = int(m.group(1))
        return 1 - w, U - 1 - w
    if expr == "t + 1 + k":
        return 1, U - 1
    raise AssertionError(f"unrecognised row expression: {expr}")


@pytest.mark.parametrize("key", ["alpha158_f32", "alpha101_f32"])
def test_interior_reads_stay_in_bounds(key, tmp_path):
    spec = predefined_spec(key)
    tag = spec["name"]
    paths = codegen.generate_module(spec, str(tmp_path), tag=tag)
    src = "".join(open(p).read() for p in paths)
    bodies = list(re.finditer(r"template <bool KE> __device__ __forceinline__ void (\w+)_body\(", src))
    assert bodies, "no vector-form kernels generated"
    checked = 0
    for i, m in enumerate(bodies):
        name = m.group(1)
        end = bodies[i + 1].start() if i + 1 < len(bodies) else len(src)
        text = src[m.end():end]
        cond = re.search(r"if \(t0_ >= (\d+) && t1_ \+ (\d+) <= P\.length\) " + re.escape(name) + r"_body<false>",
                         text)
        assert cond, f"{name}: no interior condition"
        wmax, fwd = int(cond.group(1)), int(cond.group(2))
        step = re.search(r"for \(long long t = t0; t < t1; t \+= (\d+)\)", text)
        assert step, name
        U = int(step.group(1))
        assert 4 % U == 0, f"{name}: {U} rows per thread do not divide a tile"
        for r in READ.finditer(text):
            loops = [l for l in LOOP.finditer(text, 0, r.start())]
            loop = (int(loops[-1].group(1)), int(loops[-1].group(2))) if loops else None
            dloops = [l for l in DLOOP.finditer(text, 0, r.start())]
            dloop = (int(dloops[-1].group(1)), int(dloops[-1].group(2))) if dloops else None
            lo, hi = _offsets(r.group(1), U, loop, dloop)
            assert -lo <= wmax, f"{name}: reads t{lo:+d}, interior needs t0 >= {-lo}, has {wmax}"
            assert hi - U <= fwd - 1, f"{name}: reads t+{hi} with t <= t1 - {U}, interior has t1 + {fwd} <= length"
            checked += 1
    assert checked > 100
    # the generated default tiles are multiples of 4
    tiles = re.findall(r"P\.tile\[\d+\] = \(a->tune_tile && a->tune_tile\[\d+\] > 0\) \? a->tune_tile\[\d+\] : (\d+);",
                       src)
    assert tiles
    assert all(int(d) % 4 == 0 for d in tiles), tiles


RING = re.compile(r"kun::ring_row\(nm(\d+), \(int\)\((\w+)\), (\d+)\)")


@pytest.mark.parametrize("key", ["alpha101_stream_f32", "alpha158_stream_f32"])
def test_stream_ring_rows_wrap_once(key, tmp_path):
    """Stream kernels find a ring row as nm - off wrapped once (nm = n % W):
    right only for 0 <= off < W.  Every such read in the generated sources
    has a constant offset or a window-loop index below its ring depth, and
    names the ring position of its own depth."""
    spec = predefined_spec(key)
    paths = codegen.generate_module(spec, str(tmp_path), tag=spec["name"])
    src = "".join(open(p).read() for p in paths)
    n = 0
    for m in RING.finditer(src):
        nm_w, off, W = int(m.group(1)), m.group(2), int(m.group(3))
        assert nm_w == W, m.group(0)
        if off == "iter":
            loops = list(LOOP.finditer(src, 0, m.start()))
            assert loops, m.group(0)
            hi = int(loops[-1].group(1))
            assert 0 <= int(loops[-1].group(2)) and hi < W, f"{m.group(0)} inside a loop from {hi}"
        else:
            assert 0 <= int(off) < W, m.group(0)
        n += 1
    assert n > 100
    # every ring position a kernel uses is declared in it
    for k in re.finditer(r"__global__ void __launch_bounds__\(KUN_TS_THREADS\) (\w+)\(", src):
        end = src.find("\n}\n", k.end())
        body = src[k.end():end]
        for w in set(re.findall(r"\bnm(\d+)\b", body)):
            assert f"const int nm{w} = (int)(n % {w});" in body, f"{k.group(1)}: nm{w}"
