"""GPU vs oracle parity on the predefined factor libraries.

The oracle restates the reference CPU executor (including the multiply-add
contractions of its GCC build); the GPU path must reproduce it bit for bit.
"""
import numpy as np
import pytest

from kunquant_gb300 import runner as kr
from kunquant_gb300 import synth
from kunquant_gb300.graph import predefined_spec
from oracle.oracle import OracleProgram
from tests.parity import compare_exact

CASES = [
    # (library key, module name, stocks, days, nan fraction, cur_time)
    ("alpha158_f32", "alpha158", 64, 260, 0.0, 0),
    ("alpha158_f32", "alpha158", 61, 300, 0.005, 0),
    ("alpha158_f32", "alpha158", 64, 260, 0.0, 50),
    ("alpha101_f32", "alpha101", 64, 260, 0.0, 0),
    ("alpha101_f32", "alpha101", 62, 260, 0.005, 0),
    ("alpha101_f32", "alpha101", 64, 260, 0.0, 50),
    ("alpha158_f64", "alpha158_f64", 32, 260, 0.005, 0),
    ("alpha101_f64", "alpha101_f64", 32, 260, 0.005, 0),
    ("alpha158_fast_f32", "alpha158_fast", 64, 300, 0.005, 0),
    ("alpha158_fast_f32", "alpha158_fast", 61, 260, 0.0, 40),
    ("alpha101_fast_f32", "alpha101_fast", 64, 260, 0.005, 0),
    ("alpha158_plain_f32", "alpha158_plain", 64, 300, 0.005, 0),
]

_programs = {}
_libs = {}


def _oracle(key):
    if key not in _programs:
        _programs[key] = OracleProgram(predefined_spec(key))
    return _programs[key]


def _module(key, name):
    if key not in _libs:
        _libs[key] = kr.Library.predefined(key)
    return _libs[key].getModule(name)


@pytest.mark.gpu
@pytest.mark.parametrize("key,name,S,T,nanf,start", CASES)
def test_numpy_path_bit_exact(key, name, S, T, nanf, start):
    spec = predefined_spec(key)
    dt = np.float32 if spec["dtype"] == "float" else np.float64
    data = synth.ohlcv(S, T, seed=S * 7 + T, nan_frac=nanf, dtype=dt)
    want = _oracle(key).run(data, cur_time=start, length=T - start)
    ex = kr.createSingleThreadExecutor()
    got = kr.runGraph(ex, _module(key, name), data, start, T - start)
    bad = compare_exact(got, want)
    assert not bad, f"{len(bad)} outputs differ: {dict(list(bad.items())[:5])}"


@pytest.mark.gpu
def test_torch_device_path_bit_exact():
    import torch
    key, name, S, T = "alpha158_f32", "alpha158", 128, 300
    data = synth.ohlcv(S, T, seed=3, nan_frac=0.005)
    want = _oracle(key).run(data)
    ex = kr.createSingleThreadExecutor()
    dev = {k: torch.from_numpy(v).cuda() for k, v in data.items()}
    got = kr.runGraph(ex, _module(key, name), dev, 0, T)
    torch.cuda.synchronize()
    got = {k: v.cpu().numpy() for k, v in got.items()}
    bad = compare_exact(got, want)
    assert not bad, f"{len(bad)} outputs differ: {dict(list(bad.items())[:5])}"


@pytest.mark.gpu
def test_multistream_graph_replay_bit_exact():
    """Concurrent stages on 4 streams; the third run replays a captured graph."""
    import torch
    key, name, S, T = "alpha101_f32", "alpha101", 96, 260
    data = synth.ohlcv(S, T, seed=5, nan_frac=0.005)
    want = _oracle(key).run(data)
    ex = kr.createMultiThreadExecutor(4)
    mod = _module(key, name)
    dev = {k: torch.from_numpy(v).cuda() for k, v in data.items()}
    outs = {n: torch.empty((T, S), dtype=torch.float32, device="cuda") for n in mod.getOutputNames()}
    for it in range(3):
        for o in outs.values():
            o.fill_(-7.0)
        kr.runGraph(ex, mod, dev, 0, T, outputs=outs)
        torch.cuda.synchronize()
        got = {k: v.cpu().numpy() for k, v in outs.items()}
        bad = compare_exact(got, want)
        assert not bad, f"run {it}: {len(bad)} outputs differ: {dict(list(bad.items())[:5])}"


@pytest.mark.gpu
@pytest.mark.parametrize("fixture,S", [("rank_ties_nan", 2047), ("rank_ties_nan", 2048), ("rank_ties_nan", 5000),
                                       ("rank_ties_nan", 8192), ("rank_ties_nan", 9000),
                                       ("rank2_exact", 3000), ("rank029_f64", 3000)])
def test_rank_long_rows_bit_exact(fixture, S):
    """Rows long enough for the bucketed rank or, when a bucket overflows,
    the radix-sort rank (and the wider 16-key form above 8192 stocks), with
    ties, +-0 and NaN rows, against the oracle."""
    from kunquant_gb300 import build
    from tests import golden_util as G
    spec = G.load(fixture)[0]
    dt = np.float32 if spec["dtype"] == "float" else np.float64
    rng = np.random.default_rng(S)
    T = 40 if fixture != "rank029_f64" else 30
    a = (rng.integers(0, 50, size=(T, S)) / 7).astype(dt)     # many ties
    a[3, :] = np.nan
    a[5, ::3] = np.nan
    a[7, :] = 0.0
    a[7, ::2] = -0.0
    a[9] = rng.random(S).astype(dt)                              # no ties
    # rows for the bucketed rank: spread values with a few ties, +-0 and NaN
    a[11] = rng.normal(0, 1, S).astype(dt)
    a[11, 1::5] = a[11, ::5][:len(a[11, 1::5])]
    a[11, ::97] = np.nan
    a[11, 10], a[11, 20], a[11, 30] = 0.0, -0.0, 0.0
    a[13] = rng.random(S).astype(dt)
    a[13, 17] = 1e30                                             # stretched range
    a[15] = np.exp(rng.uniform(-20, 20, S)).astype(dt)           # many binades
    a[15, ::7] = a[15, 3]
    key = "units_" + fixture
    if key not in _libs:
        _libs[key] = kr.Library.load(build.build_module_library([spec], "kun_rank_" + fixture))
    mod = _libs[key].getModule(spec["name"])
    ex = kr.createSingleThreadExecutor()
    got = kr.runGraph(ex, mod, {"a": a}, 0, T)
    want = OracleProgram(spec).run({"a": a})
    bad = compare_exact(got, want)
    assert not bad, f"{len(bad)} outputs differ: {dict(list(bad.items())[:5])}"
