"""Stream mode on the GPU against the reference StreamContext's own outputs
(golden fixtures) and the serialisation round trip of the reference's
tests/test_stream.py: dump after 50 ticks, restore from bytes and from a file,
continue, and the two truncation errors."""
import os

import numpy as np
import pytest

from kunquant_gb300 import build
from kunquant_gb300 import runner as kr
from tests import golden_util as G
from tests.parity import compare_close, compare_exact

STREAM = [n for n in G.names() if G.is_stream(n)]
# float outputs: 1e-5 relative in fp32, 1e-12 in fp64; NaN positions identical
TOL = {np.float32: (1e-5, 1e-6), np.float64: (1e-12, 1e-13)}
# index and rank outputs are bit-exact: those of the unit graphs, and the
# Alpha158 factors that rank, arg-max/min or take the extreme of a raw input
EXACT = {"argmin", "tsrank", "rank", "rank_sum", "max"}
EXACT_PREFIX = ("RANK", "IMAX", "IMIN", "IMXD")


def _exact(name):
    return name in EXACT or name.startswith(EXACT_PREFIX)

_lib = {}


def _module(spec):
    name = spec["name"]
    if name in ("alpha101_stream", "alpha158_stream"):
        key = name + "_f32"
        if key not in _lib:
            _lib[key] = kr.Library.predefined(key)
        return _lib[key].getModule(name)
    if "unit" not in _lib:
        specs = [G.load(n)[0] for n in STREAM]
        specs = [s for s in specs if not s["name"].startswith(("alpha101", "alpha158"))]
        _lib["unit"] = kr.Library.load(build.build_module_library(specs, "kun_golden_stream_units"))
    return _lib["unit"].getModule(name)


def _drive(ctx, mod, inputs, t0, t1, out):
    hin = {k: ctx.queryBufferHandle(k) for k in inputs}
    hout = {k: ctx.queryBufferHandle(k) for k in mod.getOutputNames()}
    for t in range(t0, t1):
        for k, h in hin.items():
            ctx.pushData(h, np.ascontiguousarray(inputs[k][t]))
        ctx.run()
        for k, h in hout.items():
            out[k][t] = ctx.getCurrentBuffer(h)


def _empty(mod, inputs):
    T, S = next(iter(inputs.values())).shape
    return {k: np.empty((T, S), mod.dtype) for k in mod.getOutputNames()}


@pytest.mark.gpu
@pytest.mark.parametrize("name", STREAM)
def test_stream_matches_reference(name):
    spec, inp, ref, meta = G.load(name)
    mod = _module(spec)
    T, S = next(iter(inp.values())).shape
    ex = kr.createSingleThreadExecutor()
    ctx = kr.StreamContext(ex, mod, S)
    got = _empty(mod, inp)
    _drive(ctx, mod, inp, 0, T, got)
    assert ctx.tick() == T
    ticks = meta.get("ticks")
    if ticks is not None:
        # long fixtures keep the reference's outputs at these ticks only
        got = {k: v[ticks] for k, v in got.items()}
    rtol, atol = TOL[mod.dtype]
    bad = compare_close(got, ref, rtol, atol)
    assert not bad, f"outside tolerance: {bad}"
    exact = [k for k in got if _exact(k)]
    if exact:
        bad = compare_exact(got, ref, exact)
        assert not bad, f"not bit-exact: {bad}"


@pytest.mark.gpu
def test_stream_serialize_roundtrip(tmp_path):
    spec, inp, ref, _ = G.load("stream_unit_f64")
    mod = _module(spec)
    T, S = inp["a"].shape
    ex = kr.createSingleThreadExecutor()
    ctx = kr.StreamContext(ex, mod, S)
    straight = _empty(mod, inp)
    _drive(ctx, mod, inp, 0, T, straight)

    ctx = kr.StreamContext(ex, mod, S)
    first = _empty(mod, inp)
    _drive(ctx, mod, inp, 0, 50, first)
    path = str(tmp_path / "state.bin")
    ctx.serializeStates(path)
    states = ctx.serializeStates()
    with open(path, "rb") as f:
        assert f.read() == states
    del ctx

    for init in (states, path):
        ctx = kr.StreamContext(ex, mod, S, init)
        assert ctx.tick() == 50
        out = {k: v.copy() for k, v in first.items()}
        _drive(ctx, mod, inp, 50, T, out)
        # restoring is exact: the continued run equals the uninterrupted one
        assert not compare_exact(out, straight)
        del ctx

    with pytest.raises(kr.KunError, match="^Failed to deserialize state buffer$"):
        kr.StreamContext(ex, mod, S, states[:-10])
    with open(path, "wb") as f:
        f.write(states[:20])
    with pytest.raises(kr.KunError, match="^Failed to read initial stream buffer$"):
        kr.StreamContext(ex, mod, S, path)
    os.remove(path)


@pytest.mark.gpu
def test_stream_errors():
    spec, inp, _, _ = G.load("stream_unit_f64")
    mod = _module(spec)
    ex = kr.createSingleThreadExecutor()
    ctx = kr.StreamContext(ex, mod, 24)
    with pytest.raises(kr.KunError, match="Cannot find the buffer name"):
        ctx.queryBufferHandle("nope")
    h = ctx.queryBufferHandle("a")
    with pytest.raises(kr.KunError, match="Bad input type to push"):
        ctx.pushData(h, np.zeros(24, np.float32))
    with pytest.raises(kr.KunError, match="Bad dimension for input data to push"):
        ctx.pushData(h, np.zeros(23, np.float64))
    batch = kr.Library.predefined("alpha101_f32").getModule("alpha101")
    with pytest.raises(kr.KunError, match="Cannot run batch mode module via StreamContext"):
        kr.StreamContext(ex, batch, 24)


@pytest.mark.gpu
def test_stream_device_rows_match_host_rows():
    """torch CUDA rows pushed device to device give the same outputs."""
    torch = pytest.importorskip("torch")
    spec, inp, ref, _ = G.load("stream_misc_f32")
    mod = _module(spec)
    T, S = inp["a"].shape
    ex = kr.createSingleThreadExecutor()
    ctx = kr.StreamContext(ex, mod, S)
    host = _empty(mod, inp)
    _drive(ctx, mod, inp, 0, T, host)
    ctx = kr.StreamContext(ex, mod, S)
    dev_in = {k: torch.from_numpy(v).cuda() for k, v in inp.items()}
    hin = {k: ctx.queryBufferHandle(k) for k in inp}
    hout = {k: ctx.queryBufferHandle(k) for k in mod.getOutputNames()}
    got = {k: [] for k in hout}
    for t in range(T):
        for k, h in hin.items():
            ctx.pushData(h, dev_in[k][t])
        ctx.run(synchronize=False)
        for k, h in hout.items():
            got[k].append(ctx.getCurrentBufferDevice(h))
    got = {k: torch.stack(v).cpu().numpy() for k, v in got.items()}
    assert not compare_exact(got, host)
