"""CUDA code generator: module spec -> sm_103a sources.

Replaces the reference's C++ generator (``KunQuant/passes/CodegenCpp.py:95-307``).
Every time-series stage becomes one ``__global__`` function instantiating the
device templates of ``csrc/kun_device.cuh``; cross-sectional stages
(Rank/Scale/DiffWithWeightedSum) instantiate the block-sort / row kernels of
``csrc/kun_xsec.cuh``.  A module becomes a set of ``.cu`` files plus a
descriptor table (``csrc/kun_module_abi.h``) that the runtime loads.

Time-series stage kernel ("scan" form): one thread per stock walks the time
axis like the reference's per-stock-block loop nest (``CodegenCpp.py:189``);
all reads are [T][S] rows, so a warp's loads of one row are coalesced.  In-stage
windowed temporaries go to a private [length][S] scratch buffer instead of a
register ring.
"""
import math
import os
from fractions import Fraction
from typing import Dict, List, Tuple

import numpy as np

from . import contraction

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")

ELEMENTWISE_BIN = {"Add": "kadd", "Sub": "ksub", "Mul": "kmul", "Div": "kdiv", "Max": "kmax",
                   "Min": "kmin", "Or": "kor", "And": "kand"}
CMP = {"GreaterThan": ">", "GreaterEqual": ">=", "LessThan": "<", "LessEqual": "<=",
       "Equals": "=="}
CONST_BIN = {"AddConst": "kadd", "SubConst": "ksub", "MulConst": "kmul", "DivConst": "kdiv"}
CONST_CMP = {"GreaterThanConst": ">", "LessThanConst": "<"}
UNARY = {"Sqrt": "ksqrt", "Abs": "kabs", "Sign": "ksign", "Not": "knot", "Exp": "kexpk"}
REDUCTIONS = {"ReduceAdd", "ReduceMul", "ReduceMin", "ReduceMax", "ReduceArgMax",
              "ReduceArgMin", "ReduceRank", "ReduceDecayLinear"}


def _f32_exact(text: str) -> float:
    """Correctly rounded float32 value of a decimal literal (no double rounding)."""
    q = Fraction(text)
    f = np.float32(float(q))
    best = None
    for c in (np.nextafter(f, np.float32(-np.inf)), f, np.nextafter(f, np.float32(np.inf))):
        if not np.isfinite(c):
            continue
        err = abs(Fraction(float(c)) - q)
        even = (int(np.array(c).view(np.uint32)) & 1) == 0
        key = (err, not even)
        if best is None or key < best[0]:
            best = (key, c)
    return float(best[1])


def literal(text: str, dtype: str) -> str:
    """C++ expression of the constant ``text`` in the module dtype, bit-exact
    with the reference's literal ``str(v)`` + 'f' (``CodegenCpp.py:60-72``)."""
    T = "float" if dtype == "float" else "double"
    low = text.strip().lower()
    if "nan" in low:
        return f"kun::knan<{T}>()"
    if low in ("inf", "+inf", "infinity"):
        return f"kun::kinf<{T}>()"
    if low in ("-inf", "-infinity"):
        return f"(-kun::kinf<{T}>())"
    if dtype == "float":
        v = _f32_exact(text)
        return f"{float(v).hex()}f" if v >= 0 else f"(-{float(-v).hex()}f)"
    v = float(Fraction(text))
    return f"{v.hex()}" if v >= 0 else f"(-{(-v).hex()})"


def log_tables(dtype: str) -> Tuple[List[str], List[str]]:
    """Literal tables of the table-driven log (r_i = reciprocal of the centre of
    mantissa bin i rounded to a 1/32 or 1/16 grid; logr_i = -log(r_i) - bias*ln2),
    see cpp/KunSIMD/cpu/Math.hpp:20-93."""
    from .logtables import table
    return table(dtype)


class StageGen:
    """Emits the kernel and launcher of one stage."""

    def __init__(self, spec: dict, si: int, tag: str):
        self.spec = spec
        self.si = si
        self.st = spec["stages"][si]
        self.ops = self.st["ops"]
        self.tag = tag
        self.dtype = spec["dtype"]
        self.T = "float" if self.dtype == "float" else "double"
        # type of the running sums in the precision forms of an fp32 module:
        # fp64 or two-float compensated fp32.  RT is the type of the rolling
        # states (Kahan window sums, regression sums), AT that of the
        # window-loop reductions; scope "rolling" upgrades only the former
        at = {"f64": "double", "df32": "kun::DFloat"}.get(spec.get("accum"), self.T)
        self.RT = at
        self.AT = at if spec.get("accum_scope", "all") == "all" else self.T
        self.kname = f"kst_{tag}_{si}"
        self.bufs = spec["buffers"]
        self.slots: Dict[int, int] = {}      # module buffer id -> param slot
        self.scratch: Dict[int, int] = {}    # WTO op index -> scratch slot
        self.lines: List[str] = []
        self.blocking = spec["blocking_len"]
        # set by generators whose stages support grouped launches and tuning
        self.kernel_info = None
        self.num_kernels_override = None

    # ------------------------------------------------------------ helpers
    def slot(self, bid: int) -> int:
        if bid not in self.slots:
            self.slots[bid] = len(self.slots)
        return self.slots[bid]

    def is_user_input(self, op) -> bool:
        b = self.bufs[op["buf"]]
        return b["kind"] == "INPUT" and not op.get("single_value", False)

    def layout_of(self, op) -> str:
        b = self.bufs[op["buf"]]
        if op.get("single_value"):
            return "TS"
        if b["kind"] == "INPUT":
            return self.spec["input_layout"]
        if b["kind"] == "OUTPUT":
            return self.spec["output_layout"]
        return "TS"

    def ptr_name(self, i: int) -> str:
        return f"b{i}"

    def read_at(self, src: int, texpr: str) -> str:
        """Value of windowed source op `src` at relative time `texpr`."""
        return f"{self.ptr_name(src)}[({texpr}) * st{src}]"

    def window_read(self, src: int, off: str) -> str:
        return f"((t >= (long long)({off})) ? {self.read_at(src, f't - (long long)({off})')} : kun::knan<{self.T}>())"

    def val(self, i: int) -> str:
        if self.ops[i]["k"] in REDUCTIONS:
            return self.reduction_value(i, f"r{i}")
        return f"v{i}"

    def reduction_value(self, i: int, obj: str) -> str:
        if self.ops[i]["k"] == "ReduceAdd" and self.AT != self.T:
            return f"(({self.T}){obj}.value())"
        return f"{obj}.value()"

    def lit(self, text: str) -> str:
        return literal(text, self.dtype)

    # ------------------------------------------------------------ ops
    def simple_expr(self, i: int, fplan):
        """Right-hand side of a pointwise op, or None for other ops."""
        op = self.ops[i]
        k = op["k"]
        T = self.T
        a = op["in"]
        if i in fplan:
            pos, prod = fplan[i]
            po = self.ops[prod]
            A = self.val(po["in"][0])
            B = self.val(po["in"][1]) if po["k"] == "Mul" else self.lit(po["value"])
            if k == "Add":
                return f"kun::kfma({A}, {B}, {self.val(a[1 - pos])})"
            if k == "Sub":
                o = self.val(a[1 - pos])
                return f"kun::kfma({A}, {B}, -({o}))" if pos == 0 else f"kun::kfma(-({A}), {B}, {o})"
            if k == "AddConst":
                return f"kun::kfma({A}, {B}, {self.lit(op['value'])})"
            if k == "SubConst":
                c = self.lit(op["value"])
                return f"kun::kfma(-({A}), {B}, {c})" if op.get("swap") else f"kun::kfma({A}, {B}, -({c}))"
            raise RuntimeError("bad fused op " + k)
        if k == "ConstantOp":
            return self.lit(op["value"])
        if k in ELEMENTWISE_BIN:
            return f"kun::{ELEMENTWISE_BIN[k]}({self.val(a[0])}, {self.val(a[1])})"
        if k in CMP:
            return f"kun::kmask<{T}>({self.val(a[0])} {CMP[k]} {self.val(a[1])})"
        if k in CONST_BIN:
            c = self.lit(op["value"])
            x, y = (c, self.val(a[0])) if op.get("swap") else (self.val(a[0]), c)
            return f"kun::{CONST_BIN[k]}({x}, {y})"
        if k in CONST_CMP:
            c = self.lit(op["value"])
            x, y = (c, self.val(a[0])) if op.get("swap") else (self.val(a[0]), c)
            return f"kun::kmask<{T}>({x} {CONST_CMP[k]} {y})"
        if k in UNARY:
            return f"kun::{UNARY[k]}({self.val(a[0])})"
        if k == "Log":
            fn = "klogfast" if self.spec.get("options", {}).get("fast_log", True) else "klogstd"
            return f"kun::{fn}({self.val(a[0])})"
        if k == "SetInfOrNanToValue":
            return f"kun::ksetinfnan({self.val(a[0])}, {self.lit(op['value'])})"
        if k == "Select":
            return f"kun::kselect({self.val(a[0])}, {self.val(a[1])}, {self.val(a[2])})"
        if k == "ReturnFirstValue":
            return self.val(a[0])
        return None

    def emit_simple(self, i: int, ind: str, fplan) -> bool:
        e = self.simple_expr(i, fplan)
        if e is None:
            return False
        self.lines.append(f"{ind}const {self.T} v{i} = {e};")
        return True

    def reduction_decl(self, r: int) -> str:
        op = self.ops[r]
        k = op["k"]
        T = self.T
        if k == "ReduceAdd":
            return f"kun::RAdd<{self.AT}> r{r};"
        if k == "ReduceMul":
            return f"kun::RMul<{T}> r{r};"
        if k == "ReduceMin":
            return f"kun::RMin<{T}> r{r};"
        if k == "ReduceMax":
            return f"kun::RMax<{T}> r{r};"
        if k == "ReduceArgMax":
            return f"kun::RArg<{T}, true> r{r};"
        if k == "ReduceArgMin":
            return f"kun::RArg<{T}, false> r{r};"
        if k == "ReduceRank":
            return f"kun::RRank<{T}> r{r}({self.val(op['in'][1])});"
        if k == "ReduceDecayLinear":
            return f"kun::RDecay<{T}, {op['window']}> r{r};"
        raise RuntimeError(k)

    def reduction_step(self, r: int, fplan, ind: str):
        op = self.ops[r]
        k = op["k"]
        x = self.val(op["in"][0])
        if k == "ReduceAdd" and r in fplan:
            _, prod = fplan[r]
            po = self.ops[prod]
            A = self.val(po["in"][0])
            B = self.val(po["in"][1]) if po["k"] == "Mul" else self.lit(po["value"])
            loop = contraction.reduction_loop(self.ops, r)
            if contraction.loop_unrolled(self.ops, loop):
                first = self.ops[loop]["window"] - 1
                self.lines.append(f"{ind}if (iter == {first}) r{r}.step_fma_first({A}, {B}); "
                                  f"else r{r}.step_fma({A}, {B});")
            else:
                self.lines.append(f"{ind}r{r}.step_fma({A}, {B});")
        elif k in ("ReduceArgMax", "ReduceArgMin"):
            self.lines.append(f"{ind}r{r}.step({x}, iter);")
        else:
            self.lines.append(f"{ind}r{r}.step({x});")

    # ------------------------------------------------------------ stage
    def gen_ts(self) -> Tuple[str, str]:
        ops = self.ops
        T = self.T
        fplan = contraction.plan(ops)
        n = len(ops)
        # loop structure (CodegenCpp.py:242-270 with merge_loops' copy_prev_body)
        loop_body: Dict[int, List[int]] = {}
        loop_reds: Dict[int, List[int]] = {}
        own_reds: Dict[int, List[int]] = {}
        prev = None
        for i, op in enumerate(ops):
            if op["k"] != "ForeachBackWindow":
                continue
            if op.get("p", -1) >= 0:
                raise RuntimeError("nested loops are not supported")
            body, reds = [], []
            if op.get("copy_prev_body") and prev is not None:
                body += loop_body[prev]
                reds += loop_reds[prev]
            own = [j for j in range(n) if ops[j]["k"] in REDUCTIONS
                   and contraction.reduction_loop(ops, j) == i]
            body += [j for j in range(n) if ops[j].get("p", -1) == i]
            reds += own
            loop_body[i], loop_reds[i], own_reds[i] = body, reds, own
            prev = i
        # pointers
        decl: List[str] = []
        state: List[str] = []
        for i, op in enumerate(ops):
            k = op["k"]
            if k in ("Input", "Output"):
                sl = self.slot(op["buf"])
                const = "const " if k == "Input" else ""
                lay = self.layout_of(op)
                rowoff = "start" if self.is_user_input(op) else "0"
                rows = "total_time" if self.is_user_input(op) else "length"
                if op.get("single_value"):
                    decl.append(f"  {const}{T}* __restrict__ b{i} = ({const}{T}*)P.p[{sl}] + s;")
                    decl.append(f"  const long long st{i} = 0;")
                elif lay == "TS":
                    decl.append(f"  {const}{T}* __restrict__ b{i} = ({const}{T}*)P.p[{sl}] + {rowoff} * S + s;")
                    decl.append(f"  const long long st{i} = S;")
                else:
                    L = self.blocking
                    decl.append(f"  {const}{T}* __restrict__ b{i} = ({const}{T}*)P.p[{sl}] + "
                                f"(s / {L}) * {rows} * {L} + {rowoff} * {L} + s % {L};")
                    decl.append(f"  const long long st{i} = {L};")
            elif k == "WindowedTempOutput" and op.get("p", -1) < 0:
                sc = len(self.scratch)
                self.scratch[i] = sc
                decl.append(f"  {T}* __restrict__ b{i} = ({T}*)P.w[{sc}] + s;")
                decl.append(f"  const long long st{i} = S;")
            elif k == "FastWindowedSum":
                state.append(f"  kun::FWSum<{self.RT}> fw{i}({op['window']});")
            elif k == "WindowedLinearRegression":
                state.append(f"  kun::LinReg<{self.RT}, {op['window']}> lr{i};")
            elif k == "ExpMovingAvg":
                init = f"kun::knan<{T}>()"
                if len(op["in"]) == 2:
                    init = f"b{op['in'][1]}[0]"
                state.append(f"  kun::EMA<{T}, {op['window']}> ema{i}({init});")
            elif k == "Accumulator":
                state.append(f"  {T} acc{i} = 0;")
            elif k == "SkipListState":
                state.append(f"  kun::SortedWindow<{op['window']}> sl{i};")
        # the EMA init reads a single-value input declared above
        self.lines = []
        last_loop_window = 0
        for i, op in enumerate(ops):
            if op.get("p", -1) >= 0:
                continue
            k = op["k"]
            a = op["in"]
            ind = "    "
            if k == "Input":
                if op.get("single_value"):
                    self.lines.append(f"{ind}const {T} v{i} = b{i}[0];")
                else:
                    self.lines.append(f"{ind}const {T} v{i} = b{i}[t * st{i}];")
            elif k == "Output":
                self.lines.append(f"{ind}b{i}[t * st{i}] = {self.val(a[0])};")
                self.lines.append(f"{ind}const {T} v{i} = {self.val(a[0])};")
            elif k == "WindowedTempOutput":
                self.lines.append(f"{ind}b{i}[t * st{i}] = {self.val(a[0])};")
                self.lines.append(f"{ind}const {T} v{i} = {self.val(a[0])};")
            elif k == "ForeachBackWindow":
                w, seg = op["window"], op.get("segment_end", 0)
                last_loop_window = w
                for r in own_reds[i]:
                    self.lines.append(f"{ind}{self.reduction_decl(r)}")
                self.lines.append(f"{ind}for (int iter = {w - 1}; iter >= {seg}; --iter) {{")
                bind = ind + "    "
                for j in loop_body[i]:
                    bo = ops[j]
                    if bo["k"] == "IterValue":
                        src = bo["in"][1]
                        self.lines.append(f"{bind}const {T} v{j} = {self.window_read(src, 'iter')};")
                    elif bo["k"] == "WindowLoopIndex":
                        self.lines.append(f"{bind}const {T} v{j} = ({T})({bo.get('loop_window', w)} - 1 - iter);")
                    elif not self.emit_simple(j, bind, fplan):
                        raise RuntimeError(f"unsupported op in loop body: {bo['k']}")
                for r in loop_reds[i]:
                    self.reduction_step(r, fplan, bind)
                self.lines.append(f"{ind}}}")
            elif k in REDUCTIONS:
                pass
            elif k == "BackRef":
                self.lines.append(f"{ind}const {T} v{i} = {self.window_read(a[0], op['window'])};")
            elif k == "FastWindowedSum":
                self.lines.append(f"{ind}const {T} v{i} = ({T})fw{i}.step({self.window_read(a[0], op['window'])}, {self.val(a[0])});")
            elif k == "WindowedLinearRegression":
                shared = "true" if contraction.regression_shares_square(ops, i) else "false"
                self.lines.append(f"{ind}lr{i}.template step<{shared}>({self.window_read(a[0], op['window'])}, {self.val(a[0])});")
            elif k == "WindowedLinearRegressionRSqaureImpl":
                self.lines.append(f"{ind}const {T} v{i} = ({T})lr{a[0]}.rsq();")
            elif k == "WindowedLinearRegressionSlopeImpl":
                self.lines.append(f"{ind}const {T} v{i} = ({T})lr{a[0]}.slope();")
            elif k == "WindowedLinearRegressionResiImpl":
                self.lines.append(f"{ind}const {T} v{i} = ({T})lr{a[0]}.resi({self.val(a[1])});")
            elif k == "ExpMovingAvg":
                self.lines.append(f"{ind}const {T} v{i} = ema{i}.step({self.val(a[0])});")
            elif k == "SkipListState":
                self.lines.append(f"{ind}sl{i}.step({self.val(a[0])}, {self.val(a[1])}, (int)t);")
            elif k == "SkipListQuantile":
                self.lines.append(f"{ind}const {T} v{i} = sl{a[0]}.quantile<{T}>({self.lit(op['q'])});")
            elif k == "SkipListMin":
                self.lines.append(f"{ind}const {T} v{i} = sl{a[0]}.vmin<{T}>();")
            elif k == "SkipListMax":
                self.lines.append(f"{ind}const {T} v{i} = sl{a[0]}.vmax<{T}>();")
            elif k == "SkipListArgMin":
                self.lines.append(f"{ind}const {T} v{i} = sl{a[0]}.argmin<{T}>(t);")
            elif k == "SkipListRank":
                self.lines.append(f"{ind}const {T} v{i} = sl{a[0]}.rank<{T}>({self.val(a[1])});")
            elif k == "Accumulator":
                self.lines.append(f"{ind}const {T} v{i} = acc{i};")
            elif k == "SetAccumulator":
                acc = a[0]
                self.lines.append(f"{ind}acc{acc} = kun::ksel({self.val(a[1])}) ? {self.val(a[2])} : {self.val(acc)};")
                self.lines.append(f"{ind}const {T} v{i} = acc{acc};")
            elif not self.emit_simple(i, ind, fplan):
                raise RuntimeError(f"unsupported op {k}")
        nslots = max(1, len(self.slots))
        nscr = max(1, len(self.scratch))
        pstruct = f"P_{self.kname}"
        body = "\n".join(self.lines)
        src = f"""
struct {pstruct} {{
  void* p[{nslots}];
  void* w[{nscr}];
  long long S, total_time, start, length;
}};

__global__ void __launch_bounds__(KUN_TS_THREADS) {self.kname}(const {pstruct} P) {{
  const long long S = P.S;
  const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= S) return;
  const long long total_time = P.total_time, start = P.start, length = P.length;
  (void)total_time; (void)start;
{chr(10).join(decl)}
{chr(10).join(state)}
  for (long long t = 0; t < length; ++t) {{
{body}
  }}
}}
"""
        launch = self.launcher(pstruct, f"{self.kname}<<<(unsigned)((a->num_stocks + KUN_TS_THREADS - 1) / KUN_TS_THREADS), KUN_TS_THREADS, 0, (cudaStream_t)stream>>>(P);")
        return src, launch

    def launcher(self, pstruct: str, call: str) -> str:
        fill = "\n".join(f"  P.p[{sl}] = a->buffers[{bid}];" for bid, sl in self.slots.items())
        fillw = "\n".join(f"  P.w[{sc}] = a->scratch[{sc}];" for sc in range(len(self.scratch)))
        return f"""
extern "C" int {self.kname}_launch(const KunGpuStageArgs* a, void* stream) {{
  {pstruct} P;
{fill}
{fillw}
  P.S = a->num_stocks; P.total_time = a->total_time; P.start = a->start; P.length = a->length;
  if (a->num_stocks <= 0 || a->length <= 0) return 0;
  {call}
  return (int)cudaGetLastError();
}}
"""

    def gen_generic(self) -> Tuple[str, str]:
        """A GenericCrossSectionalOp: its head and body (C++ text over `T`,
        `num_stocks`, `input_N[i]`, `output_N[i]`, KunQuant/ops/MiscOp.py:
        201-224) compiled as device code, one thread per time row, each row
        walking its stocks in order as the reference's stage loop does for
        each time index (KunQuant/passes/CodegenCpp.py:107-138).  STs operands
        go through [length][S] scratch like the other row kernels."""
        ops, T = self.ops, self.T
        xop = next(i for i, o in enumerate(ops) if o["k"] == "GenericCrossSectional")
        ins = [ops[j] for j in ops[xop]["in"]]
        outs = [o for o in ops if o["k"] == "Output"]
        for o in ins:
            if o["k"] != "Input":
                raise RuntimeError("cross-sectional stage input must be a buffer")
        for o in ins + outs:  # register every slot before sizing the slot array
            self.slot(o["buf"])
        nslots = len(self.slots)
        pstruct = f"P_{self.kname}"
        kern = f"kcs_{self.kname}"
        L = self.blocking
        pre, post, argin, argout = [], [], [], []
        for k, o in enumerate(ins):
            sl, user = self.slot(o["buf"]), self.is_user_input(o)
            if self.layout_of(o) == "STs":
                sc = len(self.scratch)
                self.scratch[("in", k)] = sc
                rows, row0 = ("P.total_time", "P.start") if user else ("P.length", "0")
                pre.append(f"  if (int e = kun::launch_sts_to_ts<{T}>((const {T}*)P.p[{sl}], ({T}*)a->scratch[{sc}], "
                           f"P.S, {rows}, {row0}, P.length, {L}, (cudaStream_t)stream)) return e;")
                argin.append(f"(const {T}*)a->scratch[{sc}]")
            else:
                argin.append(f"(const {T}*)P.p[{sl}] + ({1 if user else 0} ? P.start : 0) * P.S")
        for k, o in enumerate(outs):
            sl = self.slot(o["buf"])
            if self.layout_of(o) == "STs":
                sc = len(self.scratch)
                self.scratch[("out", k)] = sc
                argout.append(f"({T}*)a->scratch[{sc}]")
                post.append(f"  if (int e = kun::launch_ts_to_sts<{T}>(({T}*)a->scratch[{sc}], ({T}*)P.p[{sl}], "
                            f"P.S, P.length, {L}, (cudaStream_t)stream)) return e;")
            else:
                argout.append(f"({T}*)P.p[{sl}]")
        params = [f"const {T}* __restrict__ kun_in_{k}" for k in range(len(ins))] + \
                 [f"{T}* __restrict__ kun_out_{k}" for k in range(len(outs))]
        rows = [f"    const kun::CsRow<const {T}> input_{k}{{kun_in_{k} + kun_t * kun_S}};" for k in range(len(ins))] + \
               [f"    const kun::CsRow<{T}> output_{k}{{kun_out_{k} + kun_t * kun_S}};" for k in range(len(outs))]
        src = f"""
struct {pstruct} {{
  void* p[{nslots}];
  long long S, total_time, start, length;
}};
__global__ void __launch_bounds__(128) {kern}({", ".join(params)}, long long kun_S, long long kun_length) {{
  const long long kun_t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (kun_t >= kun_length) return;
  using T = {T};
  const size_t num_stocks = (size_t)kun_S;
  (void)num_stocks;
  // {ops[xop].get("op_class", "GenericCrossSectionalOp")}: generate_head()
{ops[xop].get("head", "")}
  {{
{chr(10).join(rows)}
    // generate_body()
{ops[xop]["body"]}
  }}
}}
"""
        call = (f"  {kern}<<<(unsigned)((P.length + 127) / 128), 128, 0, (cudaStream_t)stream>>>("
                f"{', '.join(argin + argout)}, P.S, P.length);\n"
                f"  if (int e = (int)cudaGetLastError()) return e;")
        fill = "\n".join(f"  P.p[{sl}] = a->buffers[{bid}];" for bid, sl in self.slots.items())
        body = "\n".join(pre + [call] + post + ["  return 0;"])
        launch = f"""
extern "C" int {self.kname}_launch(const KunGpuStageArgs* a, void* stream) {{
  {pstruct} P;
{fill}
  P.S = a->num_stocks; P.total_time = a->total_time; P.start = a->start; P.length = a->length;
  if (a->num_stocks <= 0 || a->length <= 0) return 0;
{body}
}}
"""
        return src, launch

    def gen_xsec(self) -> Tuple[str, str]:
        ops = self.ops
        T = self.T
        kind = self.st["kind"]
        if kind == "generic":
            return self.gen_generic()
        xop = next(i for i, o in enumerate(ops) if o["k"] in ("Rank", "Scale", "DiffWithWeightedSum"))
        ins = [ops[j] for j in ops[xop]["in"]]
        outop = next(o for o in ops if o["k"] == "Output")
        for o in ins:
            if o["k"] != "Input":
                raise RuntimeError("cross-sectional stage input must be a buffer")
        in_slots = [self.slot(o["buf"]) for o in ins]
        out_slot = self.slot(outop["buf"])
        in_user = ["1" if self.is_user_input(o) else "0" for o in ins]
        lay_in = [self.layout_of(o) for o in ins]
        lay_out = self.layout_of(outop)
        nslots = len(self.slots)
        pstruct = f"P_{self.kname}"
        src = f"""
struct {pstruct} {{
  void* p[{nslots}];
  long long S, total_time, start, length;
}};
"""
        # STs operands go through [length][S] scratch copies (the row
        # kernels read and write [T][S] rows)
        pre, post = [], []
        L = self.blocking
        argin = []
        for k, (o, sl, lay) in enumerate(zip(ins, in_slots, lay_in)):
            if lay == "STs":
                sc = len(self.scratch)
                self.scratch[("in", k)] = sc
                rows = "P.total_time" if in_user[k] == "1" else "P.length"
                row0 = "P.start" if in_user[k] == "1" else "0"
                pre.append(f"  if (int e = kun::launch_sts_to_ts<{T}>((const {T}*)P.p[{sl}], ({T}*)a->scratch[{sc}], "
                           f"P.S, {rows}, {row0}, P.length, {L}, (cudaStream_t)stream)) return e;")
                argin.append(f"(const {T}*)a->scratch[{sc}]")
            else:
                argin.append(f"(const {T}*)P.p[{sl}] + ({in_user[k]} ? P.start : 0) * P.S")
        if lay_out == "STs":
            sc = len(self.scratch)
            self.scratch[("out", 0)] = sc
            argout = f"({T}*)a->scratch[{sc}]"
            post.append(f"  if (int e = kun::launch_ts_to_sts<{T}>(({T}*)a->scratch[{sc}], ({T}*)P.p[{out_slot}], "
                        f"P.S, P.length, {L}, (cudaStream_t)stream)) return e;")
        else:
            argout = f"({T}*)P.p[{out_slot}]"
        if kind == "rank":
            call = f"kun::launch_rank<{T}>({argin[0]}, {argout}, P.S, P.length, (cudaStream_t)stream)"
        elif kind == "scale":
            call = f"kun::launch_scale<{T}>({argin[0]}, {argout}, P.S, P.length, (cudaStream_t)stream)"
        else:
            call = f"kun::launch_diffwsum<{T}>({argin[0]}, {argin[1]}, {argout}, P.S, P.length, (cudaStream_t)stream)"
        fill = "\n".join(f"  P.p[{sl}] = a->buffers[{bid}];" for bid, sl in self.slots.items())
        body = "\n".join(pre + [f"  if (int e = {call}) return e;"] + post + ["  return 0;"])
        launch = f"""
extern "C" int {self.kname}_launch(const KunGpuStageArgs* a, void* stream) {{
  {pstruct} P;
{fill}
  P.S = a->num_stocks; P.total_time = a->total_time; P.start = a->start; P.length = a->length;
  if (a->num_stocks <= 0 || a->length <= 0) return 0;
{body}
}}
"""
        return src, launch

    def generate(self) -> Tuple[str, int, int]:
        if self.st["kind"] == "ts":
            src, launch = self.gen_ts()
        else:
            src, launch = self.gen_xsec()
        nk = self.num_kernels_override or max(1, launch.count("<<<"))
        return src + launch, len(self.scratch), nk


def stage_generator(spec: dict, si: int, tag: str, mode: str = "leveled") -> StageGen:
    """Leveled kernels where the stage allows them, else the single-scan form."""
    if spec["output_layout"] == "STREAM":
        from .streamgen import StreamGen
        return StreamGen(spec, si, tag)
    if mode == "leveled" and spec["stages"][si]["kind"] == "ts":
        from .leveled import LeveledGen, Unsupported
        try:
            g = LeveledGen(spec, si, tag)
            g.generate()  # dry run: fall back on anything the levels cannot express
            return LeveledGen(spec, si, tag)
        except Unsupported:
            pass
    return StageGen(spec, si, tag)


def _c_str(s: str) -> str:
    return '"' + s.replace("\\", "\\\\").replace('"', '\\"') + '"'


def generate_module(spec: dict, out_dir: str, tag: str = None, stages_per_file: int = 8, file_bytes: int = 48000,
                    mode: str = "leveled") -> List[str]:
    """Write the CUDA sources of one module; returns the list of .cu paths."""
    os.makedirs(out_dir, exist_ok=True)
    name = spec["name"]
    tag = tag or name
    dtype = spec["dtype"]
    T = "float" if dtype == "float" else "double"
    r, lr = log_tables(dtype)
    header = f"""// generated by kunquant_gb300.codegen for module {name}; do not edit
#include "kun_device.cuh"
#include "kun_xsec.cuh"
#include "kun_module_abi.h"
#ifndef KUN_TS_THREADS
#define KUN_TS_THREADS 128
#endif
#ifndef KUN_TS_MINB
#define KUN_TS_MINB 1
#endif
namespace kun {{
// LogFast's tables in global memory (one 128- or 256-byte line each, read
// through the cache): a table local to the function would be rebuilt in
// local memory on every call
__device__ const {T} kLogR[32] = {{{", ".join(r)}}};
__device__ const {T} kLogLR[32] = {{{", ".join(lr)}}};
template <> struct LogTables<{T}> {{
  static __device__ __forceinline__ {T} r(unsigned long long i) {{ return kLogR[i]; }}
  static __device__ __forceinline__ {T} lr(unsigned long long i) {{ return kLogLR[i]; }}
}};
}}  // namespace kun
"""
    paths = []
    n_stages = len(spec["stages"])
    scratch_counts = [0] * n_stages
    kernel_counts = [1] * n_stages
    state_t = [0] * n_stages
    state_i = [0] * n_stages
    init_fn = ["nullptr"] * n_stages
    extern_init = []
    kinfo: Dict[int, List[int]] = {}
    imax: Dict[int, List[int]] = {}
    files: List[List[str]] = []
    cur: List[str] = []
    for si in range(n_stages):
        g = stage_generator(spec, si, tag, mode)
        src, nscr, nk = g.generate()
        scratch_counts[si] = nscr
        kernel_counts[si] = nk
        state_t[si], state_i[si] = getattr(g, "state_t_vars", 0), getattr(g, "state_i_vars", 0)
        if state_i[si]:
            imax[si] = list(g.state_i_max)
            assert len(imax[si]) == state_i[si]
        if getattr(g, "has_init", False):
            init_fn[si] = f"kst_{tag}_{si}_init"
            extern_init.append(si)
        if g.kernel_info:
            kinfo[si] = g.kernel_info
        cur.append(src)
        # translation units of similar size compile in parallel in about
        # the time of the largest one
        if len(cur) >= stages_per_file or sum(len(c) for c in cur) >= file_bytes:
            files.append(cur)
            cur = []
    if cur:
        files.append(cur)
    for fi, chunks in enumerate(files):
        p = os.path.join(out_dir, f"{tag}_{fi}.cu")
        with open(p, "w") as f:
            f.write(header + "\n".join(chunks))
        paths.append(p)
    # descriptor
    lines = [f"// generated module descriptor for {name}", '#include "kun_module_abi.h"', ""]
    for si in range(n_stages):
        lines.append(f'extern "C" int kst_{tag}_{si}_launch(const KunGpuStageArgs*, void*);')
    for si in extern_init:
        lines.append(f'extern "C" int kst_{tag}_{si}_init(const KunGpuStageArgs*, void*);')
    for si, ki in kinfo.items():
        lines.append(f'extern "C" size_t kst_{tag}_{si}_prepare(const KunGpuStageArgs*, int, void*);')
        lines.append(f'extern "C" int kst_{tag}_{si}_launch_group(const KunGpuStageArgs*, int, const void*, void*);')
        lines.append(f"static const int32_t st{si}_kinfo[] = {{{', '.join(str(v) for v in ki)}}};")
    for si, mx in imax.items():
        lines.append(f"static const int32_t st{si}_imax[] = {{{', '.join(str(v) for v in mx)}}};")
    for si, st in enumerate(spec["stages"]):
        for key in ("in", "out", "deps"):
            vals = st.get(key, []) or []
            arr = ", ".join(str(v) for v in vals) if vals else "-1"
            lines.append(f"static const int32_t st{si}_{key}[] = {{{arr}}};")
    kinds = {"ts": "KUN_STAGE_TS", "rank": "KUN_STAGE_RANK", "scale": "KUN_STAGE_SCALE",
             "xsec": "KUN_STAGE_XSEC", "generic": "KUN_STAGE_XSEC"}
    lines.append(f"static const KunGpuStageDesc stages_{tag}[] = {{")
    for si, st in enumerate(spec["stages"]):
        lines.append(f"  {{{_c_str(st['name'][:200])}, {kinds[st['kind']]}, {len(st['in'])}, st{si}_in, "
                     f"{len(st['out'])}, st{si}_out, {len(st.get('deps', []))}, st{si}_deps, "
                     f"{st.get('pending', 0)}, {scratch_counts[si]}, 0, kst_{tag}_{si}_launch, {kernel_counts[si]}, "
                     f"{state_t[si]}, {state_i[si]}, {init_fn[si]}, "
                     + (f"st{si}_imax, " if si in imax else "nullptr, ")
                     + (f"st{si}_kinfo, kst_{tag}_{si}_prepare, kst_{tag}_{si}_launch_group}},"
                        if si in kinfo else "nullptr, nullptr, nullptr},"))
    lines.append("};")
    bk = {"INPUT": "KUN_BUF_INPUT", "OUTPUT": "KUN_BUF_OUTPUT", "TEMP": "KUN_BUF_TEMP"}
    lines.append(f"static const KunGpuBufferDesc buffers_{tag}[] = {{")
    for b in spec["buffers"]:
        lines.append(f"  {{{b['id']}, {_c_str(b['name'])}, {bk[b['kind']]}, {b['num_users']}, "
                     f"{b['unreliable_count']}, {b['window']}}},")
    lines.append("};")
    lay = {"STs": "KUN_LAYOUT_STS", "TS": "KUN_LAYOUT_TS", "STREAM": "KUN_LAYOUT_STREAM"}
    lines.append(f"""extern "C" __attribute__((visibility("default"))) const KunGpuModuleDesc kun_module_{name} = {{
  KUN_GPU_MODULE_ABI, {_c_str(name)}, {n_stages}, stages_{tag}, {len(spec['buffers'])}, buffers_{tag},
  {lay[spec['input_layout']]}, {lay[spec['output_layout']]}, {spec['blocking_len']}, {0 if dtype == 'float' else 1},
  {1 if spec['aligned'] else 0}
}};
""")
    p = os.path.join(out_dir, f"{tag}_desc.cu")
    with open(p, "w") as f:
        f.write("\n".join(lines))
    paths.append(p)
    return paths
