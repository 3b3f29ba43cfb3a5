"""Module specs: the backend IR between KunQuant's front end and the GPU code
generator.

The front end (``KunQuant.Op`` graphs, ``KunCompilerConfig``, the passes in
``KunQuant/passes``) is used unchanged.  ``export_function`` runs the same
pipeline as the reference driver (``KunQuant/Driver.py:91-245``): config
validation, ``optimize`` -> ``do_partition`` -> ``post_optimize``, then the
buffer table.  Instead of emitting C++ (``KunQuant/passes/CodegenCpp.py``) it
serialises the post-partition stage functions into a plain dict ("spec"):

``{"name", "dtype", "blocking_len", "input_layout", "output_layout",
"aligned", "options", "buffers": [...], "stages": [...]}``

Each stage is ``{"name", "kind": "ts"|"rank"|"scale"|"xsec", "in", "out",
"deps", "pending", "ops": [...]}`` and each op is
``{"k": class name, "in": [op idx], "p": parent loop idx or -1, ...attrs}``.
Constants keep the exact decimal text the reference codegen prints
(``CodegenCpp.py:60-72``) so both the GPU code and the oracle round the same
literal.

Specs are JSON-serialisable, so the predefined Alpha101/Alpha158 graphs can be
exported once (``graphs/export_predefined.py``) and shipped without the
front end.
"""
import gzip
import json
import os
from typing import Dict, List, Tuple

GRAPH_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "graphs")

# op class name -> category used by the code generators
ELEMENTWISE_BINARY = {"Add", "Sub", "Mul", "Div", "Max", "Min", "Or", "And",
                      "GreaterThan", "GreaterEqual", "LessThan", "LessEqual", "Equals"}
BINARY_CONST = {"AddConst", "SubConst", "MulConst", "DivConst", "GreaterThanConst",
                "LessThanConst"}
ELEMENTWISE_UNARY = {"Sqrt", "Log", "Abs", "Sign", "Not", "Exp", "SetInfOrNanToValue"}
BOOL_OPS = {"Or", "And", "GreaterThan", "GreaterEqual", "LessThan", "LessEqual", "Equals",
            "GreaterThanConst", "LessThanConst", "Not"}
REDUCTIONS = {"ReduceAdd", "ReduceMul", "ReduceMin", "ReduceMax", "ReduceArgMax",
              "ReduceArgMin", "ReduceRank", "ReduceDecayLinear"}
STATEFUL = {"FastWindowedSum", "ExpMovingAvg", "WindowedLinearRegression", "SkipListState",
            "Accumulator"}
SUPPORTED = (ELEMENTWISE_BINARY | BINARY_CONST | ELEMENTWISE_UNARY | REDUCTIONS | STATEFUL | {
    "Input", "Output", "WindowedTempOutput", "ConstantOp", "Select", "ForeachBackWindow",
    "IterValue", "WindowLoopIndex", "BackRef", "SkipListQuantile", "SkipListArgMin",
    "SkipListRank", "SkipListMin", "SkipListMax", "WindowedLinearRegressionRSqaureImpl",
    "WindowedLinearRegressionSlopeImpl", "WindowedLinearRegressionResiImpl",
    "SetAccumulator", "ReturnFirstValue", "Rank", "Scale", "DiffWithWeightedSum"})


def _value_text(v) -> str:
    """The decimal text of a constant, as ``str(v)`` like the reference codegen."""
    return str(v)


def _generic_cross_sectional(op) -> bool:
    """A GenericCrossSectionalOp with its own C++ body
    (``KunQuant/ops/MiscOp.py:201-224``); DiffWithWeightedSum has a row kernel
    of its own."""
    from KunQuant.ops.MiscOp import GenericCrossSectionalOp
    return isinstance(op, GenericCrossSectionalOp) and op.__class__.__name__ != "DiffWithWeightedSum"


def _encode_op(op, f, bufid_of_name: Dict[str, int], stream_temp_bufs: Dict[int, int]):
    name = op.__class__.__name__
    if _generic_cross_sectional(op):
        # the body runs as device code, one thread per time row, over the
        # stocks in order, as the reference's stage loop runs it per row
        # (KunQuant/passes/CodegenCpp.py:107-138)
        return {"k": "GenericCrossSectional", "op_class": name, "in": [f.get_op_idx(i) for i in op.inputs],
                "p": -1, "head": op.generate_head(), "body": op.generate_body()}
    if name not in SUPPORTED:
        raise RuntimeError(f"op {name} is not supported by the GPU backend: {op}")
    d = {"k": name, "in": [f.get_op_idx(i) for i in op.inputs]}
    parent = op.get_parent()
    d["p"] = f.get_op_idx(parent) if parent is not None else -1
    a = op.attrs
    if name in ("Input", "Output"):
        d["buf"] = bufid_of_name[a["name"]]
        if a.get("single_value", False):
            d["single_value"] = True
    if "window" in a:
        d["window"] = int(a["window"])
    if "value" in a:
        d["value"] = _value_text(a["value"])
    if a.get("swap", False):
        d["swap"] = True
    if "q" in a:
        d["q"] = _value_text(a["q"])
    if "segment_end" in a:
        d["segment_end"] = int(a["segment_end"])
    if a.get("copy_prev_body", False):
        d["copy_prev_body"] = True
    if name == "Accumulator":
        d["acc"] = a["name"]
    if name == "WindowedTempOutput" and f.get_op_idx(op) in stream_temp_bufs:
        d["buf"] = stream_temp_bufs[f.get_op_idx(op)]
    return d


def _stage_kind(f) -> str:
    from KunQuant.Op import Input, Output
    for op in f.ops:
        if isinstance(op, (Input, Output)):
            continue
        n = op.__class__.__name__
        if n == "Rank":
            return "rank"
        if n == "Scale":
            return "scale"
        if n == "DiffWithWeightedSum":
            return "xsec"
        if _generic_cross_sectional(op):
            return "generic"
    return "ts"


def validate_config(dtype, blocking_len, input_layout, output_layout, allow_unaligned,
                    options: dict, module_name: str):
    """Config checks of the reference driver (``KunQuant/Driver.py:92-144``) for
    a device without SIMD lanes: ``blocking_len`` keeps its meaning for the STs
    layout and for the skip-list decision, so the x86 defaults are used."""
    suggested = {"float": 8, "double": 4}
    if input_layout == "ST8s":
        input_layout = "STs"
    if output_layout == "ST8s":
        output_layout = "STs"
    if dtype not in ("float", "double"):
        raise RuntimeError("Bad dtype " + dtype)
    if blocking_len is None:
        blocking_len = suggested[dtype]
    if {"float": 32, "double": 64}[dtype] * blocking_len not in (256, 512):
        raise RuntimeError(f"Blocking length {blocking_len} is not supported for {dtype}")
    options["blocking_len"] = blocking_len
    if output_layout not in ("STs", "TS", "STREAM"):
        raise RuntimeError("Bad output_layout name " + output_layout)
    if input_layout not in ("STs", "TS", "STREAM"):
        raise RuntimeError("Bad input_layout name " + input_layout)
    stream_mode = output_layout == "STREAM"
    if stream_mode and input_layout != "STREAM":
        input_layout = "STREAM"
    if stream_mode and options.get("opt_reduce", False):
        raise RuntimeError("Currently opt_reduce in stream mode is not supported.")
    if options.get("no_fast_stat", False) == "no_warn":
        options["no_fast_stat"] = False
    if stream_mode:
        if "no_fast_stat" not in options:
            options["no_fast_stat"] = True
        elif not options["no_fast_stat"]:
            raise RuntimeError("no_fast_stat=False is not supported in stream mode.")
    elif "no_fast_stat" not in options:
        options["no_fast_stat"] = dtype == "float"
    if stream_mode and allow_unaligned is None:
        allow_unaligned = False
    elif allow_unaligned is None:
        allow_unaligned = True
    if allow_unaligned and stream_mode:
        raise RuntimeError("Currently allow_unaligned in stream mode is not supported.")
    return blocking_len, input_layout, output_layout, allow_unaligned, stream_mode


def export_function(f, module_name: str, partition_factor=3, dtype="float", blocking_len=None,
                    input_layout="STs", output_layout="STs", allow_unaligned=None,
                    split_source=0, options=None) -> dict:
    """Compile a front-end ``Function`` with KunQuant's own passes and return the
    module spec.  Same keyword arguments as ``KunCompilerConfig``."""
    from KunQuant.Driver import optimize, post_optimize
    from KunQuant.passes import do_partition
    from KunQuant.Op import Input, Output, WindowedTempOutput
    options = dict(options or {})
    blocking_len, input_layout, output_layout, allow_unaligned, stream_mode = validate_config(
        dtype, blocking_len, input_layout, output_layout, allow_unaligned, options, module_name)

    buffers: List[dict] = []
    idx_of: Dict[str, int] = {}

    def insert(name: str, kind: str) -> dict:
        if name not in idx_of:
            idx_of[name] = len(buffers)
            buffers.append({"id": len(buffers), "name": name, "kind": kind, "num_users": 0})
        return buffers[idx_of[name]]

    for op in f.ops:
        if isinstance(op, Input):
            insert(op.attrs["name"], "INPUT")
        elif isinstance(op, Output):
            insert(op.attrs["name"], "OUTPUT")
    single_value_inputs = sorted({op.attrs["name"] for op in f.ops
                                  if isinstance(op, Input) and op.attrs.get("single_value", False)})

    required_windows = optimize(f, options)
    mainf, impl = do_partition(f, partition_factor, options)
    input_windows = post_optimize(impl, options)

    stages = []
    stage_idx = {}
    for func in impl:
        ins, outs = [], []
        for op in func.ops:
            if isinstance(op, Input):
                b = insert(op.attrs["name"], "TEMP")
                if b["id"] not in ins:
                    ins.append(b["id"])
            elif isinstance(op, Output):
                b = insert(op.attrs["name"], "TEMP")
                outs.append(b["id"])
        for bid in ins:
            buffers[bid]["num_users"] += 1
        stream_temp = {}
        if stream_mode:
            for op in func.ops:
                if op.get_parent() is None and isinstance(op, WindowedTempOutput):
                    idx = func.get_op_idx(op)
                    tname = f"{func.name}_{idx}"
                    input_windows[tname] = op.attrs["window"]
                    stream_temp[idx] = insert(tname, "TEMP")["id"]
        ops = [_encode_op(op, func, idx_of, stream_temp) for op in func.ops]
        stage_idx[func.name] = len(stages)
        stages.append({"name": func.name, "kind": _stage_kind(func), "in": ins, "out": outs,
                       "ops": ops})
    for p in mainf.ops:
        st = stages[stage_idx[p.attrs["name"]]]
        st["pending"] = len(p.inputs)
        st["deps"] = [stage_idx[u.attrs["name"]] for u in mainf.op_to_id[p].uses]
    for b in buffers:
        b["unreliable_count"] = int(required_windows.get(b["name"], 0))
        b["window"] = int(input_windows.get(b["name"], 1))
    return {
        "version": 1,
        "name": module_name,
        "dtype": dtype,
        "blocking_len": blocking_len,
        "input_layout": input_layout,
        "output_layout": output_layout,
        "aligned": not allow_unaligned,
        "options": {k: v for k, v in options.items() if isinstance(v, (bool, int, float, str))},
        "single_value_inputs": single_value_inputs,
        "buffers": buffers,
        "stages": stages,
    }


def save_spec(spec: dict, path: str):
    data = json.dumps(spec, separators=(",", ":")).encode()
    if path.endswith(".gz"):
        with gzip.GzipFile(path, "wb", mtime=0) as f:
            f.write(data)
    else:
        with open(path, "wb") as f:
            f.write(data)


def load_spec(path: str) -> dict:
    if path.endswith(".gz"):
        with gzip.open(path, "rb") as f:
            return json.loads(f.read())
    with open(path) as f:
        return json.load(f)


def predefined_spec(name: str) -> dict:
    """Load a spec shipped in ``kunquant_gb300/graphs`` (``alpha158_f32`` ...).

    ``<base>_acc64_f32`` is the fp32 module ``<base>_f32`` with its running
    sums (Kahan window sums, two-pass window reductions, regression sums)
    accumulated in fp64, and ``<base>_comp_f32`` the same with two-float
    compensated fp32 sums; every other op stays fp32.  ``<base>_mixed_f32``
    keeps the window-loop reductions in Kahan fp32 and makes only the rolling
    states (Kahan window sums, regression sums) two-float compensated.
    ``<base>_plain_f32`` is the one-launch-per-op baseline form of
    ``<base>_f32``.  ``<base>_slide_f32`` is the sliding-moment form
    (``slide.py``): two-pass window moments expanded into two-float sliding
    window sums, scans in time chunks."""
    if name.endswith("_slide_f32"):
        from . import slide
        spec = slide.rewrite(predefined_spec(name[:-len("_slide_f32")] + "_f32"))
        spec["name"] = spec["name"] + "_slide"
        return spec
    for suffix, sets in (("_acc64_f32", {"accum": "f64"}), ("_comp_f32", {"accum": "df32"}),
                         ("_mixed_f32", {"accum": "df32", "accum_scope": "rolling"}),
                         ("_plain_f32", {"form": "plain"})):
        if name.endswith(suffix):
            spec = predefined_spec(name[:-len(suffix)] + "_f32")
            spec["name"] = spec["name"] + suffix[:-4]
            spec.update(sets)
            return spec
    for ext in (".json.gz", ".json"):
        p = os.path.join(GRAPH_DIR, name + ext)
        if os.path.exists(p):
            return load_spec(p)
    raise FileNotFoundError(f"no predefined module spec named {name}")


def predefined_names() -> List[str]:
    out = []
    for fn in sorted(os.listdir(GRAPH_DIR)):
        if fn.endswith(".json.gz"):
            out.append(fn[:-8])
        elif fn.endswith(".json"):
            out.append(fn[:-5])
    return out


def output_names(spec: dict) -> List[str]:
    return [b["name"] for b in spec["buffers"] if b["kind"] == "OUTPUT"]


def input_names(spec: dict) -> List[str]:
    return [b["name"] for b in spec["buffers"] if b["kind"] == "INPUT"]
