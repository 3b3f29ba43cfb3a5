"""Parity at the benchmarked configuration: Alpha158 fp32, [T][S], 5000 stocks
x 2500 days with 0.5% NaN cells, the same seeded inputs as bench.py, on an
executor with 8 streams and the launch shapes the autotuner picks (time tiles,
block sizes, 64-register instances).  Every one of the 158 outputs must be
bit-identical to the oracle (the reference executor's algorithm restated on
the CPU), which runs on all host cores."""
import numpy as np
import pytest

from kunquant_gb300 import synth
from kunquant_gb300.graph import predefined_spec
from oracle.oracle import OracleProgram
from tests.parity import bits_equal

S, T = 5000, 2500


@pytest.mark.gpu
def test_alpha158_headline_tuned_bit_exact():
    import os
    import torch
    from kunquant_gb300 import runner as kr
    data = synth.ohlcv(S, T, seed=1234, nan_frac=0.005)
    want = OracleProgram(predefined_spec("alpha158_f32")).run(data, nthreads=os.cpu_count() or 1)

    mod = kr.Library.predefined("alpha158_f32").getModule("alpha158")
    dev_in = {k: torch.from_numpy(v).cuda() for k, v in data.items()}
    ex = kr.createMultiThreadExecutor(8)
    tuned = kr.tune(ex, mod, [dev_in], reps=2)
    assert tuned > 0
    out = {n: torch.empty((T, S), dtype=torch.float32, device="cuda") for n in mod.getOutputNames()}
    # the second run replays the captured graph, as the timed bench steps do
    for _ in range(2):
        kr.runGraph(ex, mod, dev_in, 0, T, outputs=out)
    torch.cuda.synchronize()
    bad = {}
    for k, w in want.items():
        g = out[k].cpu().numpy()
        eq = bits_equal(g, w)
        if not eq.all():
            idx = tuple(np.argwhere(~eq)[0])
            bad[k] = (int((~eq).sum()), idx, float(g[idx]), float(w[idx]))
    assert len(want) == 158
    assert not bad, f"{len(bad)} outputs differ from the oracle: {dict(list(bad.items())[:6])}"
