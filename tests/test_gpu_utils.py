"""corrWith / RankCorrWith and aggregrate on the GPU, against the reference's
own outputs (golden fixtures) and the CPU restatement at larger sizes."""
import numpy as np
import pytest

from kunquant_gb300 import runner as kr
from oracle import utils as U
from tests import golden_util as G
from tests.parity import compare_exact


@pytest.mark.gpu
@pytest.mark.parametrize("tag", ["f32", "f64"])
def test_aggregrate_matches_reference(tag):
    _, inp, ref, _ = G.load("util_aggregrate_" + tag)
    ex = kr.createSingleThreadExecutor()
    ng = ref["a_sum"].shape[0]
    outs = [{k: np.empty((ng, 16), inp["a"].dtype) for k in U.KINDS} for _ in range(2)]
    kr.aggregrate(ex, [inp["a"], inp["b"]], [inp["labels"], inp["labels"]], outs)
    for name, o in zip(("a", "b"), outs):
        assert not compare_exact(o, {k: ref[f"{name}_{k}"] for k in U.KINDS}), name


@pytest.mark.gpu
def test_aggregrate_large_and_partial_outputs():
    import torch
    rng = np.random.default_rng(3)
    T, S = 2500, 3000
    x = rng.random((T, S)).astype(np.float32)
    x[rng.random((T, S)) < 0.001] = np.nan
    labels = np.repeat(np.arange(T // 25), 25).astype(np.float32)
    want = U.aggregrate(x, labels)
    ex = kr.createSingleThreadExecutor()
    out = {"mean": torch.empty((T // 25, S), device="cuda"), "max": np.empty((T // 25, S), np.float32)}
    kr.aggregrate(ex, [torch.from_numpy(x).cuda()], [torch.from_numpy(labels).cuda()], [out])
    got = {"mean": out["mean"].cpu().numpy(), "max": out["max"]}
    assert not compare_exact(got, {k: want[k] for k in got})


@pytest.mark.gpu
def test_corrwith_matches_reference():
    _, inp, ref, _ = G.load("util_corrwith")
    ex = kr.createSingleThreadExecutor()
    o = [np.empty(24, np.float32), np.empty(24, np.float32)]
    kr.corrWith(ex, [inp["a"], inp["b"]], inp["ret"], o, "TS")
    r = [np.empty(24, np.float32), np.empty(24, np.float32)]
    kr.corrWith(ex, [inp["a"], inp["b"]], inp["ret"], r, "TS", rank_inputs=True)
    for name, g, rg in (("a", o[0], r[0]), ("b", o[1], r[1])):
        np.testing.assert_allclose(g, ref[name], rtol=1e-4, atol=1e-6)
        np.testing.assert_allclose(rg, ref["rank_" + name], rtol=1e-4, atol=1e-6)


@pytest.mark.gpu
def test_corrwith_large_ts_and_sts():
    import torch
    rng = np.random.default_rng(11)
    T, S = 300, 5000
    xs = [rng.standard_normal((T, S)).astype(np.float32) for _ in range(3)]
    y = (0.3 * xs[0] + rng.standard_normal((T, S))).astype(np.float32)
    xs[2][5, 7] = np.nan  # a NaN row stays NaN, as the reference's sums do
    ex = kr.createSingleThreadExecutor()
    outs = [np.empty(T, np.float32) for _ in xs]
    kr.corrWith(ex, [torch.from_numpy(x).cuda() for x in xs], torch.from_numpy(y).cuda(), outs, "TS")
    for x, o in zip(xs, outs):
        np.testing.assert_allclose(o, U.corr_with(x, y), rtol=2e-6, atol=1e-7)
    # STs layout [S/8][T][8]
    sts = lambda a: np.ascontiguousarray(a.T.reshape(S // 8, 8, T).transpose(0, 2, 1))  # noqa: E731
    o2 = [np.empty(T, np.float32)]
    kr.corrWith(ex, [sts(xs[0])], sts(y), o2, "STs")
    np.testing.assert_allclose(o2[0], U.corr_with(xs[0], y), rtol=2e-6, atol=1e-7)
    # ranked inputs
    o3 = [np.empty(T, np.float32)]
    kr.corrWith(ex, [xs[1]], y, o3, "TS", rank_inputs=True)
    np.testing.assert_allclose(o3[0], U.corr_with(xs[1], y, rank_inputs=True), rtol=2e-6, atol=1e-7)
