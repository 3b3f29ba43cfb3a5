"""The compile front door keeps the reference's signature
(``KunQuant/jit/cfake.py:174``): a reference test script runs with only its
imports changed.  Needs KunQuant's front end (the graph builder and passes);
skipped where it is not importable."""
import os

import numpy as np
import pytest


def _front_end():
    try:
        from kunquant_gb300.graphs import export_predefined
        export_predefined._front_end()
        import KunQuant.Op  # noqa: F401
    except Exception:
        pytest.skip("KunQuant front end not importable")


def _diff_with_weighted_sum_graph():
    # the graph of the reference's test_generic_cross_sectional
    # (tests/test_runtime.py:78-100)
    from KunQuant.Op import Builder, Input, Output
    from KunQuant.ops import DiffWithWeightedSum
    from KunQuant.Stage import Function
    builder = Builder()
    with builder:
        inp1 = Input("a")
        inp2 = Input("b")
        inp3 = Input("c")
        Output(DiffWithWeightedSum(inp1 - inp2, inp3), "out")
    return Function(builder.ops)


def _rolling_graph():
    from KunQuant.Op import Builder, Input, Output
    from KunQuant.ops import WindowedAvg, WindowedStddev
    from KunQuant.Stage import Function
    builder = Builder()
    with builder:
        x = Input("x")
        Output(WindowedAvg(x, 5), "ma5")
        Output(WindowedStddev(x, 10), "std10")
    return Function(builder.ops)


def test_compileit_loads_a_library(tmp_path):
    _front_end()
    from kunquant_gb300 import cfake
    lib = cfake.compileit([("test1", _diff_with_weighted_sum_graph(),
                            cfake.KunCompilerConfig(input_layout="TS", output_layout="TS"))],
                          "cfaketest", cfake.CppCompilerConfig(machine=cfake.NativeCPUFlags()))
    mod = lib.getModule("test1")
    assert mod.getOutputNames() == ["out"]
    assert sorted(mod.getInputNames()) == ["a", "b", "c"]


def test_compileit_keep_files_and_no_load(tmp_path):
    _front_end()
    from kunquant_gb300 import cfake
    with pytest.raises(RuntimeError, match="tempdir should not be empty"):
        cfake.compileit([("m", _rolling_graph(), cfake.KunCompilerConfig())], "x", keep_files=True)
    path = cfake.compileit([("roll", _rolling_graph(), cfake.KunCompilerConfig(input_layout="TS",
                                                                                output_layout="TS"))],
                           "rolltest", cfake.CppCompilerConfig(), tempdir=str(tmp_path), keep_files=True,
                           load=False)
    assert os.path.exists(path) and path.startswith(str(tmp_path))
    assert any(f.endswith(".cu") for f in os.listdir(os.path.dirname(path)))
    path2 = cfake.compileit([("roll", _rolling_graph(), cfake.KunCompilerConfig(input_layout="TS",
                                                                                 output_layout="TS"))],
                            "rolltest2", cfake.GpuCompilerConfig(), load=False)
    assert os.path.exists(path2)
    from kunquant_gb300 import runner as kr
    mod = kr.Library.load(path2).getModule("roll")
    assert sorted(mod.getOutputNames()) == ["ma5", "std10"]


@pytest.mark.gpu
def test_compileit_runs_the_reference_test():
    """The body of the reference's test_generic_cross_sectional with the
    imports changed."""
    _front_end()
    from kunquant_gb300 import cfake
    from kunquant_gb300 import runner as kr
    lib = cfake.compileit([("test1", _diff_with_weighted_sum_graph(),
                            cfake.KunCompilerConfig(input_layout="TS", output_layout="TS"))],
                          "cfaketest", cfake.CppCompilerConfig())
    a = np.random.rand(24, 16).astype("float32")
    b = np.random.rand(24, 16).astype("float32")
    c = np.random.rand(24, 16).astype("float32")
    ret = np.random.rand(24, 16).astype("float32")
    executor = kr.createSingleThreadExecutor()
    kr.runGraph(executor, lib.getModule("test1"), {"a": a, "b": b, "c": c}, 0, 24, {"out": ret})
    v1 = a - b
    v2 = np.sum(v1 * c, axis=1)
    expected = v1 - v2.reshape((-1, 1))
    np.testing.assert_allclose(expected, ret, atol=1e-6, rtol=1e-4, equal_nan=True)
