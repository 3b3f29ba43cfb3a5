"""GPU results against the reference's own outputs (golden fixtures) and
against the oracle.  The GPU path must be bit-identical to the oracle on every
output; against the reference the oracle's few known-inexact outputs are held
to 1e-5."""
import pytest

from kunquant_gb300 import build
from kunquant_gb300 import runner as kr
from oracle.oracle import OracleProgram
from tests import golden_util as G
from tests.parity import compare_exact
from tests.test_oracle_golden import BATCH, check_against_reference

_lib = {}


def _module(spec):
    if "unit" not in _lib:
        specs = []
        for n in BATCH:
            s = G.load(n)[0]
            if not s["name"].startswith(("alpha101", "alpha158")):
                specs.append(s)
        _lib["unit"] = kr.Library.load(build.build_module_library(specs, "kun_golden_units"))
    name = spec["name"]
    if name.startswith(("alpha101", "alpha158")):
        key = {"alpha101": "alpha101_f32", "alpha101_sts": "alpha101_sts_f32",
               "alpha158": "alpha158_f32", "alpha101_f64": "alpha101_f64",
               "alpha158_f64": "alpha158_f64", "alpha101_fast": "alpha101_fast_f32",
               "alpha158_fast": "alpha158_fast_f32"}[name]
        if key not in _lib:
            _lib[key] = kr.Library.predefined(key)
        return _lib[key].getModule(name)
    return _lib["unit"].getModule(name)


@pytest.mark.gpu
@pytest.mark.parametrize("name", BATCH)
def test_gpu_matches_reference_and_oracle(name):
    spec, inp, ref, meta = G.load(name)
    start = meta.get("cur_time", 0)
    T = G.num_time(inp)
    ex = kr.createSingleThreadExecutor()
    got = kr.runGraph(ex, _module(spec), inp, start, T - start)
    want = OracleProgram(spec).run(inp, cur_time=start, length=T - start)
    bad = compare_exact(got, want)
    assert not bad, f"GPU differs from the oracle: {bad}"
    check_against_reference(name, got, ref, meta)
