"""The sliding-moment form (kunquant_gb300/slide.py) against the fp64 truth.

The slide form is not bound to the reference's fp32 summation order, so it is
scored against the reference's fp64 TS build restated (the fp64 oracle, and at
the benchmarked size the fp64 GPU build, which the fp64 parity tests hold bit
for bit to that oracle).  Relative error per cell as in the precision test:
|got - want| / max(|want|, 1e-3 * median |want| of the factor), over cells
where both are numbers; NaN cells must be the fp64 build's exactly.

Bounds: every factor's median error <= 1e-5; every factor's maximum error
<= 1e-5 except the ones whose loss is in fp32 factor arithmetic outside the
window sums (listed in ILL), which are held to the fp64-accumulator form's own
maximum (alpha158_acc64) times 2."""
import numpy as np
import pytest

from kunquant_gb300 import runner as kr
from kunquant_gb300 import synth
from kunquant_gb300.graph import predefined_spec
from oracle.oracle import OracleProgram
from tests.test_gpu_precision import _errors

# fp32 arithmetic after the sums: the deviations of CORR/CORD's log-volume
# inputs, the difference of two fp32 sums in VSUMD, the ratio in WVMA at
# short windows
ILL = ("CORR", "CORD", "VSUMD", "WVMA5", "WVMA10")


def _ill(name):
    return name.startswith(ILL[:3]) or name in ILL[3:]


@pytest.mark.gpu
def test_alpha158_slide_vs_fp64():
    S, T = 256, 600
    d32 = synth.ohlcv(S, T, seed=21, nan_frac=0.005)
    want = OracleProgram(predefined_spec("alpha158_f64")).run({k: v.astype(np.float64) for k, v in d32.items()})
    ex = kr.createSingleThreadExecutor()
    got = kr.runGraph(ex, kr.Library.predefined("alpha158_slide_f32").getModule("alpha158_slide"), d32, 0, T)
    acc = kr.runGraph(ex, kr.Library.predefined("alpha158_acc64_f32").getModule("alpha158_acc64"), d32, 0, T)
    st, sa = _errors(got, want), _errors(acc, want)
    report = {f: v for f, v in st.items() if v[0] > 1e-5 or v[1] > 1e-5 or v[2]}
    print("slide factors over 1e-5 or with NaN differences:", report)
    assert sum(v[2] for v in st.values()) == 0, "NaN cells differ from fp64"
    assert all(v[1] <= 1e-5 for v in st.values()), {f: v for f, v in st.items() if v[1] > 1e-5}
    over = [f for f, v in st.items() if v[0] > 1e-5]
    assert all(_ill(f) for f in over), [f for f in over if not _ill(f)]
    for f in over:
        assert st[f][0] <= 2 * sa[f][0] + 1e-5, (f, st[f], sa[f])


@pytest.mark.gpu
def test_alpha101_slide_vs_fp64():
    S, T = 128, 400
    d32 = synth.ohlcv(S, T, seed=23, nan_frac=0.0)
    want = OracleProgram(predefined_spec("alpha101_f64")).run({k: v.astype(np.float64) for k, v in d32.items()})
    ex = kr.createSingleThreadExecutor()
    got = kr.runGraph(ex, kr.Library.predefined("alpha101_slide_f32").getModule("alpha101_slide"), d32, 0, T)
    base = kr.runGraph(ex, kr.Library.predefined("alpha101_f32").getModule("alpha101"), d32, 0, T)
    st, sb = _errors(got, want), _errors(base, want)
    # at least as many factors within 1e-5 (median and max) as the exact
    # fp32 build, and no more NaN differences
    assert sum(v[1] <= 1e-5 for v in st.values()) >= sum(v[1] <= 1e-5 for v in sb.values())
    assert sum(v[0] <= 1e-5 for v in st.values()) >= sum(v[0] <= 1e-5 for v in sb.values())
    assert sum(v[2] for v in st.values()) <= sum(v[2] for v in sb.values())


@pytest.mark.gpu
def test_alpha158_slide_benchmarked_size():
    """5000 stocks x 2500 days, 0.5% NaN cells, the bench's inputs and the
    autotuned launch shapes, against the fp64 GPU build."""
    import torch
    S, T = 5000, 2500
    data = synth.ohlcv(S, T, seed=1234, nan_frac=0.005)
    dev = {k: torch.from_numpy(v).cuda() for k, v in data.items()}
    ex = kr.createMultiThreadExecutor(8)
    mod = kr.Library.predefined("alpha158_slide_f32").getModule("alpha158_slide")
    assert kr.tune(ex, mod, [dev], reps=2) > 0
    got = kr.runGraph(ex, mod, dev, 0, T)
    got = kr.runGraph(ex, mod, dev, 0, T, outputs=got)  # graph replay
    m64 = kr.Library.predefined("alpha158_f64").getModule("alpha158_f64")
    want = kr.runGraph(ex, m64, {k: v.double() for k, v in dev.items()}, 0, T)
    torch.cuda.synchronize()
    bad_nan, bad_med = [], []
    for k, w in want.items():
        g = got[k].double()
        gn, wn = torch.isnan(g), torch.isnan(w)
        if bool((gn != wn).any()):
            bad_nan.append(k)
        both = ~gn & ~wn
        if bool(both.any()):
            wb = w[both]
            m = wb.abs().median()
            rel = (g[both] - wb).abs() / torch.clamp(wb.abs(), min=float(1e-3 * m + 1e-30))
            if float(rel.median()) > 1e-5:
                bad_med.append((k, float(rel.median())))
    assert not bad_nan, bad_nan
    assert not bad_med, bad_med


@pytest.mark.gpu
def test_alpha158_slide_regression_near_equal_prices():
    """Prices log-uniform in [1, 1e5], and every 16th stock's second close
    set 1e-5 (relative) from its first: the two-row regression windows at the
    start then have a variance ~1e10 times below the square of their sum.
    Every BETA/RSQR/RESI cell stays within 1e-5 of fp64 (R^2 of two rows is
    exactly 1)."""
    S, T = 256, 300
    d32 = synth.ohlcv(S, T, seed=77, nan_frac=0.0, price_range=(1.0, 1e5))
    close = d32["close"]
    for s in range(0, S, 16):
        close[1, s] = np.float32(close[0, s] * (1.0 + 1e-5))
    want = OracleProgram(predefined_spec("alpha158_f64")).run({k: v.astype(np.float64) for k, v in d32.items()})
    ex = kr.createSingleThreadExecutor()
    got = kr.runGraph(ex, kr.Library.predefined("alpha158_slide_f32").getModule("alpha158_slide"), d32, 0, T)
    st = _errors(got, want)
    reg = [f for f in st if f.startswith(("BETA", "RSQR", "RESI"))]
    assert len(reg) == 15
    assert all(st[f][0] <= 1e-5 and st[f][2] == 0 for f in reg), {f: st[f] for f in reg if st[f][0] > 1e-5}
    assert np.all(np.abs(np.asarray(got["RSQR5"])[1, ::16] - 1.0) <= 1e-5)
