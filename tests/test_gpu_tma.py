"""The staged (bulk-copy, mbarrier) instances of the elementwise kernels,
switched on with KUN_TMA=1 (read once per process, so the check runs in a
child process): outputs bit-identical to the oracle where the staged
instance runs (stock counts that are multiples of 4) and where the launcher
falls back to the plain one."""
import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import sys
sys.path.insert(0, REPO)
import numpy as np
from kunquant_gb300 import runner as kr, synth
from kunquant_gb300.graph import predefined_spec
from oracle.oracle import OracleProgram
from tests.parity import compare_exact
mod = kr.Library.predefined("alpha158_f32").getModule("alpha158")
prog = OracleProgram(predefined_spec("alpha158_f32"))
ex = kr.createSingleThreadExecutor()
for S, T, start in ((256, 300, 0), (132, 260, 40), (61, 200, 0)):
    d = synth.ohlcv(S, T, seed=S + T, nan_frac=0.005)
    got = kr.runGraph(ex, mod, d, start, T - start)
    bad = compare_exact(got, prog.run(d, cur_time=start, length=T - start))
    assert not bad, (S, T, start, list(bad)[:5])
print("staged ok")
"""


@pytest.mark.gpu
def test_staged_elementwise_kernels_bit_exact():
    env = dict(os.environ, KUN_TMA="1")
    code = CHILD.replace("REPO", repr(REPO))
    r = subprocess.run([sys.executable, "-c", code], cwd=REPO, env=env, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0 and "staged ok" in r.stdout, r.stdout[-2000:] + r.stderr[-3000:]
