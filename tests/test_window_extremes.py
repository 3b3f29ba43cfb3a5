"""Window Min/Max/ArgMin/ArgMax in runs of positions (kun::RExt in
csrc/kun_device.cuh, emitted by LeveledStage._emit_ext_chain in leveled.py).

A vector kernel computes U = 4 output rows per thread.  For a window of w rows
the positions t+U-w .. t are common to all U rows and are stepped once; each
row u then steps its older edge (t+u-w+1 .. t+U-1-w), continues with the
common run (RExt::then) and steps its newer edge (t+1 .. t+u).  This restates
that decomposition and the RExt rules in Python and checks them against the
reference's loop (cpp/Kun/Ops.hpp ReduceMin/ReduceMax/ReduceArgMin/
ReduceArgMax over a back window, oldest first, as kun::RMin/RMax/RArg step):
NaN anywhere gives NaN, Min/Max keep the later of equal values (the sign of
zero shows it), ArgMin/ArgMax keep the earlier position and give 0 when no
value beat the starting infinity.  The GPU tests hold the kernels bit for bit
to the oracle; this pins the decomposition itself on edge values."""
import math
import random

import pytest

from kunquant_gb300 import codegen
from kunquant_gb300.graph import predefined_spec

INF = float("inf")
U = 4


def _isnan(x):
    return x != x


def _loop(vals, is_max, is_arg):
    """The reference loop over one window, oldest value first; `iter` is the
    distance back from the output row."""
    w = len(vals)
    v = -INF if is_max else INF
    idx = 0.0
    for k, x in enumerate(vals):
        it = w - 1 - k
        nan = _isnan(v) or _isnan(x)
        if is_arg:
            cmp = (v < x) if is_max else (v > x)
            v = x if cmp else v
            idx = float(it) if cmp else idx
            v = math.nan if nan else v
            idx = math.nan if nan else idx
        else:
            v = math.nan if nan else ((v if v > x else x) if is_max else (v if v < x else x))
    return idx if is_arg else v


class _Ext:
    """kun::RExt"""

    def __init__(self, is_max, is_arg):
        self.is_max, self.is_arg = is_max, is_arg
        self.v = -INF if is_max else INF
        self.pos = 0.0

    def _join(self, x, p):
        nan = _isnan(self.v) or _isnan(x)
        if self.is_arg:
            cmp = (self.v < x) if self.is_max else (self.v > x)
            self.v, self.pos = (x, p) if cmp else (self.v, self.pos)
        else:
            self.v = (self.v if self.v > x else x) if self.is_max else (self.v if self.v < x else x)
        if nan:
            self.v = math.nan

    def step(self, x, p):
        self._join(x, p)

    def then(self, b):
        self._join(b.v, b.pos)

    def arg(self, row):
        if _isnan(self.v):
            return math.nan
        return 0.0 if self.v == (-INF if self.is_max else INF) else row - self.pos


def _split(xs, t, w, is_max, is_arg):
    """The U rows t..t+U-1 as the generated code computes them."""
    c = _Ext(is_max, is_arg)
    for d in range(w - U, -1, -1):
        c.step(xs[t - d], float(-d))
    older = [xs[t + 1 - w + k] for k in range(U - 1)]
    newer = [xs[t + 1 + k] for k in range(U - 1)]
    out = []
    for u in range(U):
        a = _Ext(is_max, is_arg)
        for k in range(u, U - 1):
            a.step(older[k], float(k + 1 - w))
        a.then(c)
        for k in range(u):
            a.step(newer[k], float(k + 1))
        out.append(a.arg(float(u)) if is_arg else a.v)
    return out


def _same(a, b):
    if _isnan(a) or _isnan(b):
        return _isnan(a) and _isnan(b)
    return a == b and math.copysign(1.0, a) == math.copysign(1.0, b)


@pytest.mark.parametrize("w", [4, 5, 7, 10, 20, 30, 60])
def test_split_equals_loop(w):
    rng = random.Random(w)
    pools = [[0.0, -0.0, 1.0, 2.0, -1.0, INF, -INF, math.nan, 3.0],
             [0.0, -0.0, 1.0, -INF, INF],
             [-INF], [INF], [0.0, -0.0],
             [float(i) for i in range(4)]]
    for trial in range(600):
        pool = pools[trial % len(pools)]
        xs = [rng.choice(pool) for _ in range(w + U + 2)]
        t = w
        for is_max in (True, False):
            for is_arg in (True, False):
                got = _split(xs, t, w, is_max, is_arg)
                for u in range(U):
                    want = _loop(xs[t + u - w + 1:t + u + 1], is_max, is_arg)
                    assert _same(got[u], want), (w, u, is_max, is_arg, xs, got[u], want)


@pytest.mark.parametrize("key", ["alpha158_f32", "alpha101_f32"])
def test_generated_runs_cover_each_window(key, tmp_path):
    """Each emitted run loop `for (int d = hi; d >= lo; --d)` steps exactly
    the windows that include row t - d, longest first, and the shared runs
    of one chain together cover d = w_max - U .. 0 once."""
    import re
    spec = predefined_spec(key)
    paths = codegen.generate_module(spec, str(tmp_path), tag=spec["name"])
    src = "".join(open(p).read() for p in paths)
    chains = re.findall(r"kun::RVal<float> r\d+\[4\];.*?\n(\s*)\{\n(.*?)\n\1\}", src, re.S)
    assert chains, "no window-extreme chains emitted"
    for _, body in chains:
        loops = [(int(a), int(b)) for a, b in re.findall(r"for \(int d = (\d+); d >= (\d+); --d\)", body)]
        assert loops
        # contiguous, descending, ending at 0
        for (hi, lo), (hi2, _) in zip(loops, loops[1:]):
            assert hi >= lo and hi2 == lo - 1, loops
        assert loops[-1][1] == 0
        windows = sorted({int(w) for w in re.findall(r"o\d+_(\d+)\[", body)}, reverse=True)
        assert loops[0][0] == windows[0] - U
