"""GenericCrossSectionalOp subclasses with their own C++ bodies
(KunQuant/ops/MiscOp.py:201-224).  The reference pastes generate_head() and
generate_body() into its stage function and runs the body once per time
index over the stocks (KunQuant/passes/CodegenCpp.py:107-138); the GPU backend
compiles the same text as device code, one thread per time row.  The
fixtures (tests/golden/make_golden.py, `_generic_graphs`) hold the reference's
own outputs for two such ops in TS and STs layouts, with a time-series stage
before and after them; the bodies add in stock order and divide once, so the
GPU must match bit for bit."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from kunquant_gb300 import codegen
from tests import golden_util as G

CASES = ["generic_cs_f32", "generic_cs_sts_f32"]


def test_fixtures_carry_the_bodies():
    for name in CASES:
        assert G.is_generic(name)
        spec = G.load(name)[0]
        gen = [o for st in spec["stages"] for o in st["ops"] if o["k"] == "GenericCrossSectional"]
        assert len(gen) == 3 and all("num_stocks" in o["body"] for o in gen)
        assert sum(st["kind"] == "generic" for st in spec["stages"]) == 3


def test_oracle_refuses_generic_bodies():
    from oracle.oracle import OracleProgram
    with pytest.raises(NotImplementedError, match="GenericCrossSectionalOp"):
        OracleProgram(G.load("generic_cs_f32")[0])


@pytest.mark.skipif(shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"),
                    reason="nvcc not available")
@pytest.mark.parametrize("name", CASES)
def test_generated_source_compiles(name, tmp_path):
    """The body is pasted into a kernel with `T`, `num_stocks`, `input_N`
    and `output_N` in scope; nvcc compiles it for sm_103a (no GPU needed)."""
    from kunquant_gb300 import build
    spec = G.load(name)[0]
    paths = codegen.generate_module(spec, str(tmp_path), tag=spec["name"])
    src = "".join(open(p).read() for p in paths)
    assert "kun::CsRow<const float> input_1" in src and "const T kZero = 0;" in src
    for p in paths:
        if "kcs_" not in open(p).read():
            continue
        r = subprocess.run([build.NVCC] + build.MODULE_FLAGS + ["-c", p, "-o", str(tmp_path / "x.o")],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-2000:]


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_matches_reference(name):
    from kunquant_gb300 import build
    from kunquant_gb300 import runner as kr
    from tests.parity import compare_exact
    spec, inputs, ref, meta = G.load(name)
    lib = kr.Library.load(build.build_module_library([spec], "kun_" + name))
    mod = lib.getModule(spec["name"])
    T = G.num_time(inputs)
    got = kr.runGraph(kr.createSingleThreadExecutor(), mod, inputs, 0, T)
    got = {k: np.asarray(v) for k, v in got.items()}
    assert sorted(got) == sorted(ref)
    assert not compare_exact(got, ref)


@pytest.mark.parametrize("name", CASES + ["misc_f32", "rank029_f64", "stats_sts_f32", "alpha158_f32", "alpha101_f32"])
def test_launch_struct_holds_every_slot(name, tmp_path):
    """Every stage launcher fills P.p[k] only for k below the size of its
    struct's slot array."""
    import re
    spec = G.load(name)[0]
    paths = codegen.generate_module(spec, str(tmp_path), tag=spec["name"])
    src = "".join(open(p).read() for p in paths)
    sizes = {m.group(1): int(m.group(2)) for m in re.finditer(r"struct (P_\w+) \{\n  void\* p\[(\d+)\];", src)}
    launchers = list(re.finditer(r"extern \"C\" int (\w+)_launch\(const KunGpuStageArgs\* a, void\* stream\) \{\n"
                                 r"  (P_\w+) P;(.*?)\n\}\n", src, re.S))
    assert len(launchers) == len(spec["stages"])
    for m in launchers:
        n = sizes[m.group(2)]
        used = [int(k) for k in re.findall(r"P\.p\[(\d+)\] = ", m.group(3))]
        assert all(k < n for k in used), (m.group(1), n, used)


def test_stream_mode_refuses_generic_bodies(tmp_path):
    """Stream modules refuse a GenericCrossSectionalOp body at code
    generation, with a message (needs KunQuant's front end)."""
    try:
        from kunquant_gb300.graphs import export_predefined
        export_predefined._front_end()
        from KunQuant.Op import Builder, Input, Output
        from KunQuant.ops.MiscOp import GenericCrossSectionalOp
        from KunQuant.Stage import Function
    except Exception:
        pytest.skip("KunQuant front end not importable")
    from kunquant_gb300.graph import export_function

    class Copy(GenericCrossSectionalOp):
        def __init__(self, v):
            super().__init__([v], None)

        def generate_head(self):
            return ""

        def generate_body(self):
            return "for (size_t i = 0; i < num_stocks; i++) output_0[i] = input_0[i];"

    b = Builder()
    with b:
        Output(Copy(Input("a")), "out")
    spec = export_function(Function(b.ops), "gen_stream", input_layout="STREAM", output_layout="STREAM")
    with pytest.raises(RuntimeError, match="stream mode"):
        codegen.generate_module(spec, str(tmp_path), tag="gen_stream")
