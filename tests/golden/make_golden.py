"""Generates the golden fixtures of tests/golden from the reference itself.

Needs the reference sources (``$KUN_REFERENCE_ROOT``, default the
``reference`` folder beside this repository):
the reference CPU runtime is built by ``oracle/build_ref.py`` and its own JIT
compiles every graph below.  For each case the fixture holds the inputs, the
reference's outputs and the module spec the GPU backend compiles, so the tests
need neither the reference nor its front end.

    python tests/golden/make_golden.py            # all cases
    python tests/golden/make_golden.py rank2 ...  # some cases

The unit graphs follow the reference's own runtime tests
(tests/test_runtime.py: rolling stats, argmin issue #19, rank with ties and
NaN rows, bit-exact rank(x+x)+x and the alpha029 rank chain, log special
values) plus graphs that reach the skip-list path (windows > 400 with 8 lanes)
and the loop-index op (max drawdown).
"""
import gzip
import io
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)


def _graphs():
    from KunQuant.Op import Builder, Input, Output, Rank, Scale, ConstantOp
    from KunQuant.Stage import Function
    from KunQuant.ops import (TsArgMin, TsArgMax, WindowedMin, WindowedMax, TsRank, WindowedStddev,
                              WindowedCorrelation, WindowedCovariance, WindowedSum, WindowedAvg,
                              WindowedQuantile, Log, Exp, DecayLinear, WindowedLinearRegressionSlope,
                              ExpMovingAvg, WindowedMaxDrawdown, WindowedSkew, WindowedKurt, Pow,
                              WindowedProduct, SetInfOrNanToValue, Sign, Abs, Select, DiffWithWeightedSum)

    def mk(body):
        def build():
            b = Builder()
            with b:
                body()
            return Function(b.ops)
        return build

    def argmin():
        a = Input("a")
        Output(TsArgMin(a, 5), "ou2")
        Output(WindowedMin(a, 5), "tsmin")
        Output(TsRank(a, 5), "tsrank")

    def rank():
        Output(Rank(Input("a")), "ou2")

    def rank2():
        a = Input("a")
        Output(Rank(a + a) + a, "out")

    def rank029():
        a = Input("a")
        inner = WindowedSum(Rank(Rank(-1 * Rank(a))), 5)
        Output(inner, "ou1")
        Output(Rank(inner), "ou2")

    def logexp():
        a = Input("a")
        Output(Log(a), "outlog")
        Output(Exp(a), "outexp")

    def stats():
        a, b = Input("a"), Input("b")
        Output(WindowedAvg(a, 10), "avg")
        Output(WindowedStddev(a, 10), "std")
        Output(WindowedCorrelation(a, 10, b), "corr")
        Output(WindowedCovariance(a, 20, b), "cov")
        Output(WindowedQuantile(a, 10, 0.49), "q49")
        Output(DecayLinear(a, 7), "decay")
        Output(WindowedLinearRegressionSlope(a, 12), "slope")
        Output(WindowedProduct(Abs(a) + 1, 6), "prod")
        Output(TsArgMax(a, 200), "argmax200")
        Output(WindowedMax(a, 200), "max200")
        Output(TsRank(a, 200), "tsrank200")
        Output(Sign(a - 0.5), "sign")
        Output(Pow(Abs(a), ConstantOp(2.5)), "pow")
        Output(Select(a > b, a, b * 2), "sel")
        Output(SetInfOrNanToValue(a / (b - 0.5)), "infnan")

    def skiplists():
        a = Input("a")
        Output(TsRank(a, 500), "tsrank500")
        Output(TsArgMin(a, 450), "argmin450")
        Output(TsArgMax(a, 450), "argmax450")
        Output(WindowedMin(a, 430), "min430")
        Output(WindowedMax(a, 430), "max430")
        Output(WindowedQuantile(a, 420, 0.3), "q30")

    def misc():
        a, b = Input("a"), Input("b")
        Output(ExpMovingAvg(a, 10), "ema")
        Output(WindowedMaxDrawdown(a, 12), "mdd")
        Output(WindowedSkew(a, 12), "skew")
        Output(WindowedKurt(a, 12), "kurt")
        Output(Scale(a - 0.5), "scale")
        Output(DiffWithWeightedSum(a, b), "diffw")

    def stream_unit():
        # the graph of the reference's tests/test_stream.py
        a = Input("a")
        Output(WindowedQuantile(a, 10, 0.49), "quantile")
        Output(ExpMovingAvg(a, 10), "ema")
        Output(WindowedLinearRegressionSlope(a, 10), "slope")

    def stream_misc():
        a, b = Input("a"), Input("b")
        Output(WindowedAvg(a, 10), "avg")
        Output(WindowedStddev(a, 10), "std")
        Output(WindowedCorrelation(a, 10, b), "corr")
        Output(TsArgMin(a, 7), "argmin")
        Output(TsRank(a, 9), "tsrank")
        Output(WindowedMax(a, 6), "max")
        Output(DecayLinear(a, 7), "decay")
        Output(WindowedSkew(a, 12), "skew")
        Output(WindowedKurt(a, 12), "kurt")
        Output(Rank(a), "rank")
        Output(Rank(WindowedSum(a, 5) - b), "rank_sum")
        Output(Scale(a - 0.5), "scale")

    return {
        # name: (builder, config kwargs, input maker)
        "stream_unit_f64": (mk(stream_unit), dict(dtype="double", input_layout="STREAM",
                                                  output_layout="STREAM"), "stream24"),
        "stream_misc_f32": (mk(stream_misc), dict(input_layout="STREAM", output_layout="STREAM"),
                            "stream_ab"),
        "argmin_issue19": (mk(argmin), dict(input_layout="TS", output_layout="TS"), "issue19"),
        "rank_ties_nan": (mk(rank), dict(input_layout="TS", output_layout="TS"), "rank"),
        "rank2_exact": (mk(rank2), dict(input_layout="TS", output_layout="TS"), "u24"),
        "rank2_unaligned": (mk(rank2), dict(input_layout="TS", output_layout="TS"), "u20"),
        "rank029_f64": (mk(rank029), dict(input_layout="TS", output_layout="TS", dtype="double",
                                          options={"opt_reduce": True, "fast_log": True,
                                                   "no_fast_stat": True}), "u20_300"),
        "logexp_f32": (mk(logexp), dict(input_layout="TS", output_layout="TS",
                                        options={"fast_log": True}), "special"),
        "logexp_f64": (mk(logexp), dict(input_layout="TS", output_layout="TS", dtype="double",
                                        options={"fast_log": True, "no_fast_stat": True}), "special"),
        "stats_f32": (mk(stats), dict(input_layout="TS", output_layout="TS",
                                      options={"opt_reduce": True}), "ab"),
        "stats_f32_noopt": (mk(stats), dict(input_layout="TS", output_layout="TS",
                                            options={"opt_reduce": False}), "ab"),
        "skiplists_f32": (mk(skiplists), dict(input_layout="TS", output_layout="TS"), "long"),
        "misc_f32": (mk(misc), dict(input_layout="TS", output_layout="TS",
                                    options={"opt_reduce": True}), "ab"),
        # the reference's default [S/8][T][8] layout in and out
        "stats_sts_f32": (mk(stats), dict(input_layout="STs", output_layout="STs",
                                          options={"opt_reduce": True}), "ab_sts"),
        "rank_sts_f32": (mk(rank029), dict(input_layout="STs", output_layout="STs"), "u24_sts"),
        "stats_ts_sts_f32": (mk(stats), dict(input_layout="TS", output_layout="STs",
                                             options={"opt_reduce": True}), "ab"),
    }


def _generic_graphs():
    """GenericCrossSectionalOp subclasses with their own C++ bodies
    (KunQuant/ops/MiscOp.py:201-224): the reference compiles the body into its
    stage function; the GPU backend compiles the same text as device code.
    Sums in stock order and one IEEE division, so the bits must agree."""
    from KunQuant.Op import Builder, Input, Output
    from KunQuant.ops.MiscOp import GenericCrossSectionalOp
    from KunQuant.Stage import Function

    class NanDemean(GenericCrossSectionalOp):
        """x minus the mean of the row's numbers (NaN cells skipped)"""

        def __init__(self, v):
            super().__init__([v], None)

        def generate_head(self):
            return "    const T kZero = 0;"

        def generate_body(self):
            return """
        T sum = kZero;
        size_t n = 0;
        for (size_t i = 0; i < num_stocks; i++) {
            T v = input_0[i];
            if (v == v) {
                sum += v;
                n++;
            }
        }
        T mean = sum / (T)n;
        for (size_t i = 0; i < num_stocks; i++) {
            output_0[i] = input_0[i] - mean;
        }
        """

    class RatioToRowMax(GenericCrossSectionalOp):
        """a over the row's largest b (NaN cells skipped)"""

        def __init__(self, a, b):
            super().__init__([a, b], None)

        def generate_head(self):
            return ""

        def generate_body(self):
            return """
        T mx = (T)(-1e30);
        for (size_t i = 0; i < num_stocks; i++) {
            T v = input_1[i];
            if (v > mx) mx = v;
        }
        for (size_t i = 0; i < num_stocks; i++) {
            output_0[i] = input_0[i] / mx;
        }
        """

    def build():
        bld = Builder()
        with bld:
            a, c = Input("a"), Input("b")
            Output(NanDemean(a), "demean")
            Output(RatioToRowMax(a * 2, c), "ratio")
            Output(NanDemean(a - c) + a, "mixed")
        return Function(bld.ops)

    return {
        "generic_cs_f32": (build, dict(input_layout="TS", output_layout="TS"), "ab"),
        "generic_cs_sts_f32": (build, dict(input_layout="STs", output_layout="STs"), "ab_sts"),
    }


def _inputs(kind, dtype):
    rng = np.random.default_rng(2024)
    if kind == "issue19":
        data = [0.6898481863442985, 0.6992020600574415, 0.6992020600574417, 0.6968635916291558,
                0.6968635916291558, 0.6968635916291558]
        a = np.empty((6, 8), dtype)
        for i in range(6):
            a[i, :] = data[i]
        return {"a": a}
    if kind == "rank":
        a = rng.random((20, 24)).astype(dtype)
        a[3:9] = (np.arange(6)[:, None] // 2).astype(dtype)
        a[10, :] = np.nan
        a[12, ::3] = np.nan
        a[14, :] = 0.0
        a[14, ::2] = -0.0
        return {"a": a}
    if kind == "u24":
        return {"a": rng.random((20, 24)).astype(dtype)}
    if kind == "u20":
        return {"a": rng.random((20, 20)).astype(dtype)}
    if kind == "u20_300":
        return {"a": rng.random((300, 20)).astype(dtype)}
    if kind == "special":
        vals = [0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan, 88.7, 88.8, -87.3, -87.4, 1e-40,
                1e-30, 3.4e38, 2.0, 0.5, 100.0, 1e5, 1e-5, 709.0, 710.0, -745.0]
        extra = rng.uniform(-100, 100, 64 * 8 - len(vals))
        return {"a": np.array(vals + list(extra), dtype=dtype).reshape(64, 8)}
    if kind == "ab":
        a = rng.random((260, 16)).astype(dtype)
        b = rng.random((260, 16)).astype(dtype)
        a[50:53, 3] = np.nan
        a[100, :] = 0.5
        b[120:124, 5] = np.nan
        a[200:203, 7] = a[199, 7]
        return {"a": a, "b": b}
    if kind == "long":
        a = rng.integers(0, 40, size=(600, 8)).astype(dtype) / 4
        a[300:305, 2] = np.nan
        return {"a": a}
    if kind in ("ab_sts", "u24_sts"):
        base = _inputs("ab" if kind == "ab_sts" else "u24", dtype)
        return {k: _to_sts(v) for k, v in base.items()}
    if kind == "stream24":
        return {"a": rng.random((100, 24)).astype(dtype)}
    if kind == "stream_ab":
        a = rng.random((80, 24)).astype(dtype)
        b = rng.random((80, 24)).astype(dtype)
        a[30:33, 3] = np.nan
        a[40, :] = 0.5
        return {"a": a, "b": b}
    raise KeyError(kind)


def _to_sts(a, L=8):
    """[T][S] -> [S/L][T][L]."""
    T, S = a.shape
    return np.ascontiguousarray(a.T.reshape(S // L, L, T).transpose(0, 2, 1))


def _save(name, spec, inputs, outputs, extra=None):
    path = os.path.join(HERE, name + ".npz")
    arrays = {"in__" + k: v for k, v in inputs.items()}
    arrays.update({"out__" + k: v for k, v in outputs.items()})
    buf = io.BytesIO()
    np.savez_compressed(buf, **arrays)
    with open(path, "wb") as f:
        f.write(buf.getvalue())
    meta = {"spec": spec}
    meta.update(extra or {})
    with gzip.GzipFile(os.path.join(HERE, name + ".json.gz"), "wb", mtime=0) as f:
        f.write(json.dumps(meta, separators=(",", ":")).encode())
    print(name, "->", os.path.relpath(path, REPO), os.path.getsize(path), "bytes")


def _digest(a) -> str:
    """SHA-256 of an output's bytes with every NaN written as the one quiet
    NaN (NaN payloads are not part of the parity contract)."""
    import hashlib
    a = np.array(a, copy=True)
    a[np.isnan(a)] = np.nan
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _save_digests(name, key, inputs, ref, cur_time=0):
    """A large batch fixture: every reference output as a SHA-256 of its
    bytes; outputs where the oracle is not bit-identical to the reference are
    stored in full (the tests hold those to 1e-5)."""
    from oracle.oracle import OracleProgram
    from kunquant_gb300.graph import predefined_spec
    a0 = next(iter(inputs.values()))
    T = a0.shape[1] if a0.ndim == 3 else a0.shape[0]
    mine = OracleProgram(predefined_spec(key)).run(inputs, cur_time=cur_time, length=T - cur_time)
    full = {k: v for k, v in ref.items() if _digest(mine[k]) != _digest(v)}
    _save(name, {"predefined": key}, inputs, full,
          {"cur_time": cur_time, "digests": {k: _digest(v) for k, v in ref.items()}})


def _stream_ticks(T, dense_from, every):
    """Ticks whose outputs a stream fixture stores: every `every`-th tick,
    and every tick from `dense_from` on (past the longest window)."""
    return [t for t in range(T) if t % every == 0 or t >= dense_from]


STREAM_CASES = {
    # fixture: (library key, stocks, ticks, nan fraction, dense from, every)
    "alpha101_stream_f32": ("alpha101_stream_f32", 64, 300, 0.0, 240, 8),
    "alpha158_stream_f32": ("alpha158_stream_f32", 64, 300, 0.002, 240, 8),
}


def predefined_cases():
    from kunquant_gb300 import synth
    from kunquant_gb300.graph import predefined_spec
    return {
        # fixture name: (library key, stocks, days, nan fraction, cur_time)
        "alpha158_f32": ("alpha158_f32", 8, 160, 0.005, 0),
        "alpha101_f32": ("alpha101_f32", 16, 200, 0.005, 0),
        "alpha101_f32_start50": ("alpha101_f32", 16, 200, 0.0, 50),
        "alpha158_f64": ("alpha158_f64", 4, 160, 0.005, 0),
        "alpha158_fast_f32": ("alpha158_fast_f32", 8, 160, 0.005, 0),
        "alpha101_fast_f32": ("alpha101_fast_f32", 16, 200, 0.005, 0),
        "alpha101_f64": ("alpha101_f64", 8, 200, 0.005, 0),
    }


def _utilities():
    """The reference's aggregrate and corrWith (tests/test_runtime.py shapes:
    240 rows x 16 stocks, labels = day of a sorted random minute stamp)."""
    from KunQuant.runner import KunRunner as kr
    rng = np.random.default_rng(77)
    ex = kr.createMultiThreadExecutor(3)
    for dt, tag in ((np.float32, "f32"), (np.float64, "f64")):
        a = rng.random((240, 16)).astype(dt)
        b = rng.random((240, 16)).astype(dt)
        a[17, 3] = np.nan
        b[100:103, 5] = np.nan
        days = np.sort(rng.integers(1, 8, 240)).astype(dt)
        ng = len(np.unique(days))
        outs = [{k: np.empty((ng, 16), dt) for k in ("sum", "min", "max", "first", "last", "count", "mean")}
                for _ in range(2)]
        kr.aggregrate(ex, [a, b], [days, days], outs)
        out = {f"a_{k}": v for k, v in outs[0].items()}
        out.update({f"b_{k}": v for k, v in outs[1].items()})
        _save("util_aggregrate_" + tag, {"utility": "aggregrate"}, {"a": a, "b": b, "labels": days}, out)
    a = rng.random((24, 40)).astype(np.float32)
    b = rng.random((24, 40)).astype(np.float32)
    ret = rng.random((24, 40)).astype(np.float32)
    o1, o2 = np.empty(24, np.float32), np.empty(24, np.float32)
    kr.corrWith(ex, [a, b], ret, [o1, o2], "TS")
    r1, r2 = np.empty(24, np.float32), np.empty(24, np.float32)
    kr.corrWith(ex, [a, b], ret, [r1, r2], "TS", rank_inputs=True)
    _save("util_corrwith", {"utility": "corrWith"}, {"a": a, "b": b, "ret": ret},
          {"a": o1, "b": o2, "rank_a": r1, "rank_b": r2})


def main(names):
    from oracle import refkun
    from oracle.build_ref import import_reference
    import_reference()
    from kunquant_gb300 import synth
    from kunquant_gb300.graph import predefined_spec
    for name, (key, S, T, nanf, start) in predefined_cases().items():
        if names and name not in names:
            continue
        spec = predefined_spec(key)
        dt = np.float32 if spec["dtype"] == "float" else np.float64
        data = synth.ohlcv(S, T, seed=S * 1000 + T, nan_frac=nanf, dtype=dt)
        out = refkun.run_batch(key, data, cur_time=start, length=T - start)
        _save(name, {"predefined": key}, data, out, {"cur_time": start})
    if not names or "alpha101_sts_f32" in names:
        # the reference's own Alpha101 configuration: fp32, STs in and out,
        # 64 stocks x 260 days
        S, T = 64, 260
        data = synth.ohlcv(S, T, seed=S * 1000 + T, nan_frac=0.0)
        sts = {k: _to_sts(v) for k, v in data.items()}
        out = refkun.run_batch("alpha101_sts_f32", sts)
        _save_digests("alpha101_sts_f32", "alpha101_sts_f32", sts, out)
    for name, (key, S, T, nanf, dense, every) in STREAM_CASES.items():
        if names and name not in names:
            continue
        data = synth.ohlcv(S, T, seed=99 + S + T, nan_frac=nanf)
        out = refkun.run_stream(key, data)
        ticks = _stream_ticks(T, dense, every)
        _save(name, {"predefined": key}, data, {k: v[ticks] for k, v in out.items()},
              {"stream": True, "ticks": ticks})
    if not names or any(n.startswith("util_") for n in names):
        _utilities()
    for name, (build, cfg, kind) in _generic_graphs().items():
        if names and name not in names:
            continue
        spec, mod = refkun.compile_function("g_" + name, build, name, **cfg)
        dt = np.float32 if spec["dtype"] == "float" else np.float64
        inputs = _inputs(kind, dt)
        _save(name, spec, inputs, refkun.run_module(mod, inputs), {"generic_cs": True})
    for name, (build, cfg, kind) in _graphs().items():
        if names and name not in names:
            continue
        spec, mod = refkun.compile_function("g_" + name, build, name, **cfg)
        dt = np.float32 if spec["dtype"] == "float" else np.float64
        inputs = _inputs(kind, dt)
        if cfg.get("output_layout") == "STREAM":
            out = refkun.run_stream_module(mod, inputs)
            _save(name, spec, inputs, out, {"stream": True})
        else:
            out = refkun.run_module(mod, inputs)
            _save(name, spec, inputs, out)


if __name__ == "__main__":
    main(sys.argv[1:])
