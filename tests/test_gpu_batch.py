"""Many universes in one run (kunRunGraphBatch) and the launch-shape
autotuner.  Universes of uneven stock counts and lengths must give exactly
the outputs of one runGraph per universe, before and after tuning."""
import numpy as np
import pytest

from kunquant_gb300 import runner as kr
from kunquant_gb300 import synth
from kunquant_gb300.graph import predefined_spec
from oracle.oracle import OracleProgram
from tests.parity import compare_exact

SHAPES = [(37, 300), (100, 260), (250, 410), (61, 280), (8, 120), (513, 300)]


def _universes(shapes, seed=0, nan=0.005):
    import torch
    out = []
    for i, (S, T) in enumerate(shapes):
        d = synth.ohlcv(S, T, seed=seed + i, nan_frac=nan)
        out.append((d, {k: torch.from_numpy(v).cuda() for k, v in d.items()}))
    return out


def _singles(ex, mod, unis):
    res = []
    for _, dev in unis:
        T = next(iter(dev.values())).shape[0]
        o = kr.runGraph(ex, mod, dev, 0, T)
        res.append({k: v.cpu().numpy() for k, v in o.items()})
    return res


def _cpu(outs):
    return [{k: v.cpu().numpy() for k, v in o.items()} for o in outs]


@pytest.mark.gpu
@pytest.mark.parametrize("key,name", [("alpha158_f32", "alpha158"), ("alpha101_f32", "alpha101")])
def test_batch_equals_one_run_per_universe(key, name):
    mod = kr.Library.predefined(key).getModule(name)
    unis = _universes(SHAPES)
    ex = kr.createSingleThreadExecutor()
    want = _singles(ex, mod, unis)
    got = _cpu(kr.runGraphBatch(ex, mod, [dev for _, dev in unis]))
    for i in range(len(unis)):
        assert not compare_exact(got[i], want[i]), f"universe {i} {SHAPES[i]}"
    # and the oracle on one of them
    assert not compare_exact(got[2], OracleProgram(predefined_spec(key)).run(unis[2][0]))


@pytest.mark.gpu
def test_tuning_keeps_results():
    mod = kr.Library.predefined("alpha158_f32").getModule("alpha158")
    unis = _universes(SHAPES, seed=40)
    ex = kr.createSingleThreadExecutor()
    want = _singles(ex, mod, unis)
    n = kr.tune(ex, mod, [dev for _, dev in unis], reps=1)
    assert n > 0
    shapes = [kr.tunedShape(ex, mod, si) for si in range(len(predefined_spec("alpha158_f32")["stages"]))]
    assert any(s is not None for s in shapes)
    for s in shapes:
        if s:
            tiles, blocks = s
            # a block entry may carry the 64-register-instance flag
            assert all(t % 4 == 0 for t in tiles) and all(0 < (b & 0xffff) <= 128 for b in blocks)
            assert all(b & ~0x1ffff == 0 for b in blocks)
    got = _cpu(kr.runGraphBatch(ex, mod, [dev for _, dev in unis]))
    again = _singles(ex, mod, unis)  # single runs with the tuned shapes
    for i in range(len(unis)):
        assert not compare_exact(got[i], want[i]), f"batched universe {i}"
        assert not compare_exact(again[i], want[i]), f"single universe {i}"


@pytest.mark.gpu
def test_more_universes_than_one_group():
    """300 small universes: the grouped launches split into groups of 256."""
    mod = kr.Library.predefined("alpha158_f32").getModule("alpha158")
    shapes = [(3 + (i % 13), 70 + (i % 5) * 3) for i in range(300)]
    unis = _universes(shapes, seed=7, nan=0.0)
    ex = kr.createSingleThreadExecutor()
    got = _cpu(kr.runGraphBatch(ex, mod, [dev for _, dev in unis]))
    for i in (0, 1, 255, 256, 299):
        want = _singles(ex, mod, [unis[i]])[0]
        assert not compare_exact(got[i], want), f"universe {i}"


@pytest.mark.gpu
def test_batch_rank_long_and_short_rows():
    """Alpha101 in a batch with a universe long enough for the radix Rank
    (2100 stocks) beside short ones (bitonic network): every universe
    bit-identical to its own run."""
    mod = kr.Library.predefined("alpha101_f32").getModule("alpha101")
    unis = _universes([(2100, 300), (37, 260), (700, 280)], seed=12)
    ex = kr.createSingleThreadExecutor()
    want = _singles(ex, mod, unis)
    got = _cpu(kr.runGraphBatch(ex, mod, [dev for _, dev in unis]))
    for i in range(len(unis)):
        assert not compare_exact(got[i], want[i]), f"universe {i}"
