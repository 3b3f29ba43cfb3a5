"""Export the predefined factor libraries as module specs.

Runs KunQuant's own front end (``KunQuant/predefined/Alpha101.py``,
``KunQuant/predefined/Alpha158.py`` and the passes) and writes the post-partition
stage graphs next to this file, so the GPU backend can build and run them on a
machine without the front end installed.  The front end is looked up on
``sys.path`` first, then under ``$KUN_REFERENCE_ROOT``.

    python kunquant_gb300/graphs/export_predefined.py

The configurations follow the reference's own tests (``tests/test_alpha101.py``,
``tests/test_alpha158.py``) with [T][S] ("TS") input and output layouts.
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def _front_end():
    try:
        import KunQuant.Op  # noqa: F401
    except ImportError:
        # the reference checkout, by default the "reference" folder beside
        # this repository
        repo = os.path.dirname(os.path.dirname(HERE))
        root = os.environ.get("KUN_REFERENCE_ROOT",
                              os.path.join(os.path.dirname(repo), "reference"))
        sys.path.append(root)
        import KunQuant.Op  # noqa: F401


def build_alpha101():
    from KunQuant.Op import Builder, Input, Output
    from KunQuant.Stage import Function
    from KunQuant.predefined.Alpha101 import AllData, all_alpha
    b = Builder()
    with b:
        d = AllData(low=Input("low"), high=Input("high"), close=Input("close"), open=Input("open"),
                    amount=Input("amount"), volume=Input("volume"))
        for fn in all_alpha:
            Output(fn(d), fn.__name__)
    return Function(b.ops)


def build_alpha158():
    from KunQuant.Op import Builder, Input, Output
    from KunQuant.Stage import Function
    from KunQuant.predefined.Alpha158 import AllData
    b = Builder()
    with b:
        p = AllData(low=Input("low"), high=Input("high"), close=Input("close"), open=Input("open"),
                    amount=Input("amount"), volume=Input("volume"))
        fields, names = p.build({
            "kbar": {},
            "price": {"windows": [0], "feature": [("OPEN", p.open), ("HIGH", p.high),
                                                  ("LOW", p.low), ("VWAP", p.vwap)]},
            "rolling": {"windows": [5, 10, 20, 30, 60]},
        })
        for v, k in zip(fields, names):
            Output(v, k)
    return Function(b.ops)


CONFIGS = {
    # name: (builder, module name, KunCompilerConfig kwargs)
    "alpha101_f32": (build_alpha101, "alpha101", dict(
        dtype="float", input_layout="TS", output_layout="TS",
        options={"opt_reduce": True, "fast_log": True})),
    # the reference's default layout in and out: [S/8][T][8]
    "alpha101_sts_f32": (build_alpha101, "alpha101_sts", dict(
        dtype="float", input_layout="STs", output_layout="STs",
        options={"opt_reduce": True, "fast_log": True})),
    "alpha101_f64": (build_alpha101, "alpha101_f64", dict(
        dtype="double", input_layout="TS", output_layout="TS",
        options={"opt_reduce": True, "fast_log": True, "no_fast_stat": True})),
    "alpha101_stream_f32": (build_alpha101, "alpha101_stream", dict(
        dtype="float", partition_factor=8, input_layout="STREAM", output_layout="STREAM",
        options={"opt_reduce": False, "fast_log": True})),
    "alpha158_f32": (build_alpha158, "alpha158", dict(
        dtype="float", partition_factor=4, input_layout="TS", output_layout="TS",
        options={"opt_reduce": True, "fast_log": True})),
    "alpha158_f64": (build_alpha158, "alpha158_f64", dict(
        dtype="double", partition_factor=4, input_layout="TS", output_layout="TS",
        options={"opt_reduce": True, "fast_log": True, "no_fast_stat": True})),
    # fp32 with the reference's fast-stat accumulators (O(1) Kahan-compensated
    # rolling moments instead of two-pass window loops)
    "alpha158_fast_f32": (build_alpha158, "alpha158_fast", dict(
        dtype="float", partition_factor=4, input_layout="TS", output_layout="TS",
        options={"opt_reduce": True, "fast_log": True, "no_fast_stat": "no_warn"})),
    "alpha101_fast_f32": (build_alpha101, "alpha101_fast", dict(
        dtype="float", input_layout="TS", output_layout="TS",
        options={"opt_reduce": True, "fast_log": True, "no_fast_stat": "no_warn"})),
    "alpha158_stream_f32": (build_alpha158, "alpha158_stream", dict(
        dtype="float", partition_factor=4, input_layout="STREAM", output_layout="STREAM",
        options={"opt_reduce": False, "fast_log": True})),
}


def main(names=None):
    _front_end()
    from kunquant_gb300.graph import export_function, save_spec
    for key, (builder, modname, kw) in CONFIGS.items():
        if names and key not in names:
            continue
        spec = export_function(builder(), modname, **kw)
        path = os.path.join(HERE, key + ".json.gz")
        save_spec(spec, path)
        print(key, len(spec["stages"]), "stages", len(spec["buffers"]), "buffers ->", path)


if __name__ == "__main__":
    main(sys.argv[1:])
