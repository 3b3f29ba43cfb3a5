"""Stream-mode code generator: one tick of every stage for many sessions.

Replaces the reference's stream executor (``cpp/Kun/Runtime.cpp:385-546``,
``StreamWindow`` in ``cpp/Kun/Ops.hpp:212-269``).  Every buffer of a stream
module is a device ring of ``window`` rows x ``capacity`` stocks, NaN
initialised; a value written at tick n sits in row ``n % window`` and the
value ``k`` ticks back is row ``(n - k) % window`` (NaN before the first
write, as the reference's NaN-filled ring).  Op states that carry over ticks
(Kahan running sums, regression sums, EMA, order-statistic windows) live in
struct-of-arrays device memory, one column per stock, loaded at the start of
a tick kernel and stored at its end.

A launch covers a list of segments (sessions), each a contiguous range of
stocks at its own tick, so the serving layer can advance hundreds of sessions
of different sizes in one launch per stage.
"""
from typing import Dict, List, Tuple

from . import contraction
from .codegen import REDUCTIONS, StageGen

_SEG_HELPER = """
#ifndef KUN_SEG_HELPER
#define KUN_SEG_HELPER
// segment of active stock i: the k with seg_off[k] <= i < seg_off[k + 1]
__device__ __forceinline__ int kun_segment(const int32_t* __restrict__ off, int nseg, long long i) {
  int lo = 0, hi = nseg - 1;
  while (lo < hi) {
    const int m = (lo + hi + 1) >> 1;
    if ((long long)off[m] <= i) lo = m; else hi = m - 1;
  }
  return lo;
}
#endif
"""


class StreamGen(StageGen):
    """Tick kernel, state initialiser and launchers of one stream stage."""

    def __init__(self, spec: dict, si: int, tag: str):
        super().__init__(spec, si, tag)
        self.fplan = contraction.plan(self.ops) if self.st["kind"] == "ts" else {}
        self.state_t_vars = 0
        self.state_i_vars = 0
        self.state_i_max: List[int] = []
        self.has_init = False
        self.windows = {b["id"]: b["window"] for b in spec["buffers"]}

    # --------------------------------------------------------------- rings
    def ring_window(self, i: int) -> int:
        return max(1, int(self.windows[self.ops[i]["buf"]]))

    def read_at(self, src: int, texpr: str) -> str:
        raise RuntimeError("stream kernels read rings by offset")

    def window_read(self, src: int, off, max_off=None) -> str:
        """Row `off` ticks back in the ring of `src` (NaN before tick 0).  When
        `off` is known to stay below the ring depth W (a constant, or a loop
        index bounded by `max_off`), the row is nm - off wrapped once, from
        the tick's ring position nm = n % W computed once per kernel."""
        W = self.ring_window(src)
        bound = max_off if max_off is not None else (off if isinstance(off, int) else None)
        if bound is not None and 0 <= bound < W:
            self.ring_ws.add(W)
            return (f"((nc >= (int)({off})) ? r{src}[(long long)kun::ring_row(nm{W}, (int)({off}), {W}) * S] "
                    f": kun::knan<{self.T}>())")
        return (f"((n - (long long)({off}) >= 0) ? r{src}[((n - (long long)({off})) % {W}) * S] "
                f": kun::knan<{self.T}>())")

    def cur_read(self, src: int) -> str:
        W = self.ring_window(src)
        self.ring_ws.add(W)
        return f"r{src}[(long long)nm{W} * S]"

    # --------------------------------------------------------------- state
    def _state_fields(self) -> Dict[int, Tuple[List[str], List[str]]]:
        """op -> (float/double fields, int fields) of its persistent state."""
        out = {}
        for i, op in enumerate(self.ops):
            k = op["k"]
            if k == "FastWindowedSum":
                out[i] = (["v", "cadd", "csub"], ["nn"])
            elif k == "WindowedLinearRegression":
                out[i] = (["isum", "xsum", "x2sum", "ysum", "y2sum", "xysum"], ["nn"])
            elif k == "ExpMovingAvg":
                if len(op["in"]) == 2:
                    raise RuntimeError("EMA with init_val is not supported in stream mode")
                out[i] = (["v"], [])
            elif k == "SkipListState":
                W = op["window"]
                idx = self._sl_idx(i)
                tf = [f"v[{j}]" for j in range(W)]
                if W <= 64:
                    inf = ["size", "last_rank"] + ([f"ix[{j}]" for j in range(W)] if idx else [])
                else:
                    inf = ["size", "last_rank"] + [f"idx[{j}]" for j in range(W)]
                out[i] = (tf, inf)
            elif k == "Accumulator":
                out[i] = (["v"], [])
        return out

    def _sl_idx(self, i: int) -> bool:
        return any(q["k"] == "SkipListArgMin" and q["in"][0] == i for q in self.ops)

    def _state_decl(self, i: int) -> str:
        op, T = self.ops[i], self.T
        k = op["k"]
        if k == "FastWindowedSum":
            return f"kun::FWSum<{T}> fw{i}({op['window']});"
        if k == "WindowedLinearRegression":
            return f"kun::LinReg<{T}, {op['window']}> lr{i};"
        if k == "ExpMovingAvg":
            return f"kun::EMA<{T}, {op['window']}> ema{i}(kun::knan<{T}>());"
        if k == "SkipListState":
            W = op["window"]
            if W <= 64:
                return f"kun::RegWindow<{T}, {W}, {'true' if self._sl_idx(i) else 'false'}> sl{i};"
            return f"kun::SortedWindow<{W}> sl{i};"
        if k == "Accumulator":
            return f"{T} acc{i} = 0;"
        raise RuntimeError(k)

    def _obj(self, i: int) -> str:
        k = self.ops[i]["k"]
        return {"FastWindowedSum": "fw", "WindowedLinearRegression": "lr", "ExpMovingAvg": "ema",
                "SkipListState": "sl", "Accumulator": "acc"}[k] + str(i)

    def _field(self, i: int, f: str) -> str:
        if self.ops[i]["k"] == "Accumulator":
            return self._obj(i)
        if self.ops[i]["k"] == "SkipListState" and self.ops[i]["window"] > 64 and f.startswith("v["):
            return f"{self._obj(i)}.{f}"
        return f"{self._obj(i)}.{f}"

    # --------------------------------------------------------------- ts
    def gen_ts(self):
        ops, T = self.ops, self.T
        fields = self._state_fields()
        toff, ioff = {}, {}
        nt = ni = 0
        for i, (tf, inf) in fields.items():
            toff[i], ioff[i] = nt, ni
            nt += len(tf)
            ni += len(inf)
        self.state_t_vars, self.state_i_vars = nt, ni
        # bounds a restored int state must respect: NaN counts, window sizes
        # and insert ranks lie in [0, window]; tick indices are free
        self.state_i_max = []
        for i, (tf, inf) in fields.items():
            W = int(ops[i].get("window", 0))
            self.state_i_max += [-1 if f.startswith(("ix[", "idx[")) else W for f in inf]
        self.has_init = bool(fields)
        # rings of the buffers the stage touches
        decl = []
        for i, op in enumerate(ops):
            if op["k"] in ("Input", "Output") or (op["k"] == "WindowedTempOutput" and op.get("p", -1) < 0):
                if op.get("single_value"):
                    raise RuntimeError("single-value inputs are not supported in stream mode")
                sl = self.slot(op["buf"])
                decl.append(f"  {T}* __restrict__ r{i} = ({T}*)P.p[{sl}] + s;")
        loads, stores = [], []
        for i, (tf, inf) in fields.items():
            loads.append(f"  {self._state_decl(i)}")
            W = ops[i].get("window", 0)
            big_sl = ops[i]["k"] == "SkipListState" and W > 64
            for j, f in enumerate(tf):
                tgt = self._field(i, f)
                src = f"st[{toff[i] + j} * S]"
                loads.append(f"  {tgt} = {'(double)' if big_sl else ''}{src};")
                stores.append(f"  {src} = ({T}){tgt};")
            for j, f in enumerate(inf):
                tgt = self._field(i, f)
                src = f"si[{ioff[i] + j} * S]"
                loads.append(f"  {tgt} = {src};")
                stores.append(f"  {src} = {tgt};")
        # ops of one tick (CodegenCpp.py:189-307 with length 1)
        self.lines = []
        self.ring_ws = set()
        loops = self._loops()
        for i, op in enumerate(ops):
            if op.get("p", -1) >= 0:
                continue
            self._emit(i, loops)
        body = "\n".join(self.lines)
        ring_pos = "\n".join(f"  const int nm{W} = (int)(n % {W});" for W in sorted(self.ring_ws))
        pstruct = f"P_{self.kname}"
        nslots = max(1, len(self.slots))
        src = _SEG_HELPER + f"""
struct {pstruct} {{
  void* p[{nslots}];
  {T}* st;
  int32_t* si;
  const int32_t* seg_off;
  const int32_t* seg_stock0;
  const long long* seg_tick;
  const int32_t* cnt;
  int nseg;
  long long n_active, S;
}};

__global__ void __launch_bounds__(KUN_TS_THREADS) {self.kname}(const {pstruct} P) {{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int nseg = P.cnt ? P.cnt[0] : P.nseg;
  const long long n_active = P.cnt ? (long long)P.cnt[1] : P.n_active;
  if (i >= n_active) return;
  const int k = kun_segment(P.seg_off, nseg, i);
  const long long s = P.seg_stock0[k] + (i - P.seg_off[k]);
  const long long n = P.seg_tick[k];
  const long long S = P.S;
  const long long t = 0;  // the reference's row index within a one-row run
  (void)t;
  // ticks so far (capped) and this tick's row in each ring depth
  const int nc = n < (1LL << 30) ? (int)n : (1 << 30);
  (void)nc;
{ring_pos}
  {T}* __restrict__ st = P.st + s;
  int32_t* __restrict__ si = P.si + s;
  (void)st; (void)si;
{chr(10).join(decl)}
{chr(10).join(loads)}
{body}
{chr(10).join(stores)}
}}
"""
        init_src = ""
        if self.has_init:
            iv = []
            for i, (tf, inf) in fields.items():
                op = ops[i]
                k = op["k"]
                W = op.get("window", 0)
                for j, f in enumerate(tf):
                    val = f"kun::knan<{T}>()" if (k in ("ExpMovingAvg", "SkipListState")) else "0"
                    iv.append(f"  P.st[{toff[i] + j} * P.S + s] = {val};")
                for j, f in enumerate(inf):
                    val = str(W) if f == "nn" else "0"
                    iv.append(f"  P.si[{ioff[i] + j} * P.S + s] = {val};")
            init_src = f"""
__global__ void {self.kname}_initk(const {pstruct} P) {{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n_active) return;
  const long long s = P.seg_stock0[0] + i;
{chr(10).join(iv)}
}}
"""
        fill = "\n".join(f"  P.p[{sl}] = a->buffers[{bid}];" for bid, sl in self.slots.items())
        common = f"""  {pstruct} P;
{fill}
  P.st = ({T}*)a->state; P.si = (int32_t*)a->state_i;
  P.seg_off = a->seg_off; P.seg_stock0 = a->seg_stock0; P.seg_tick = (const long long*)a->seg_tick;
  P.nseg = a->nseg; P.n_active = a->n_active; P.S = a->num_stocks; P.cnt = a->seg_count;
  if (a->n_active <= 0) return 0;"""
        launch = f"""
extern "C" int {self.kname}_launch(const KunGpuStageArgs* a, void* stream) {{
{common}
  {self.kname}<<<(unsigned)((a->n_active + KUN_TS_THREADS - 1) / KUN_TS_THREADS), KUN_TS_THREADS, 0, (cudaStream_t)stream>>>(P);
  return (int)cudaGetLastError();
}}
"""
        if self.has_init:
            launch += f"""
extern "C" int {self.kname}_init(const KunGpuStageArgs* a, void* stream) {{
{common}
  {self.kname}_initk<<<(unsigned)((a->n_active + 127) / 128), 128, 0, (cudaStream_t)stream>>>(P);
  return (int)cudaGetLastError();
}}
"""
        return src + init_src, launch

    def _loops(self):
        ops = self.ops
        loops, prev = {}, None
        n = len(ops)
        for i, op in enumerate(ops):
            if op["k"] != "ForeachBackWindow":
                continue
            if op.get("p", -1) >= 0:
                raise RuntimeError("nested loops are not supported")
            body, reds = [], []
            if op.get("copy_prev_body") and prev is not None:
                body += loops[prev][0]
                reds += loops[prev][1]
            own = [j for j in range(n) if ops[j]["k"] in REDUCTIONS
                   and contraction.reduction_loop(ops, j) == i]
            body += [j for j in range(n) if ops[j].get("p", -1) == i]
            reds += own
            loops[i] = (body, reds, own)
            prev = i
        return loops

    def _emit(self, i: int, loops):
        ops, T = self.ops, self.T
        op = ops[i]
        k = op["k"]
        a = op["in"]
        ind = "  "
        fplan = self.fplan
        L = self.lines
        if k == "Input":
            L.append(f"{ind}const {T} v{i} = {self.cur_read(i)};")
        elif k in ("Output", "WindowedTempOutput"):
            L.append(f"{ind}{self.cur_read(i)} = {self.val(a[0])};")
            L.append(f"{ind}const {T} v{i} = {self.val(a[0])};")
        elif k == "ForeachBackWindow":
            body, reds, own = loops[i]
            w, seg = op["window"], op.get("segment_end", 0)
            for r in own:
                L.append(f"{ind}{self.reduction_decl(r)}")
            # unrolled so that the ring loads of several iterations are in
            # flight together: one thread walks the window alone
            L.append(f"{ind}#pragma unroll 8")
            L.append(f"{ind}for (int iter = {w - 1}; iter >= {seg}; --iter) {{")
            bind = ind + "  "
            for j in body:
                bo = ops[j]
                if bo["k"] == "IterValue":
                    L.append(f"{bind}const {T} v{j} = {self.window_read(bo['in'][1], 'iter', w - 1)};")
                elif bo["k"] == "WindowLoopIndex":
                    L.append(f"{bind}const {T} v{j} = ({T})({bo.get('loop_window', w)} - 1 - iter);")
                elif not self.emit_simple(j, bind, fplan):
                    raise RuntimeError(f"unsupported op in loop body: {bo['k']}")
            for r in reds:
                self.reduction_step(r, fplan, bind)
            L.append(f"{ind}}}")
        elif k in REDUCTIONS:
            pass
        elif k == "BackRef":
            L.append(f"{ind}const {T} v{i} = {self.window_read(a[0], op['window'])};")
        elif k == "FastWindowedSum":
            L.append(f"{ind}const {T} v{i} = fw{i}.step({self.window_read(a[0], op['window'])}, {self.val(a[0])});")
        elif k == "WindowedLinearRegression":
            shared = "true" if contraction.regression_shares_square(ops, i) else "false"
            L.append(f"{ind}lr{i}.template step<{shared}>({self.window_read(a[0], op['window'])}, {self.val(a[0])});")
        elif k == "WindowedLinearRegressionRSqaureImpl":
            L.append(f"{ind}const {T} v{i} = lr{a[0]}.rsq();")
        elif k == "WindowedLinearRegressionSlopeImpl":
            L.append(f"{ind}const {T} v{i} = lr{a[0]}.slope();")
        elif k == "WindowedLinearRegressionResiImpl":
            L.append(f"{ind}const {T} v{i} = lr{a[0]}.resi({self.val(a[1])});")
        elif k == "ExpMovingAvg":
            L.append(f"{ind}const {T} v{i} = ema{i}.step({self.val(a[0])});")
        elif k == "SkipListState":
            L.append(f"{ind}sl{i}.step({self.val(a[0])}, {self.val(a[1])}, 0);")
        elif k.startswith("SkipList"):
            W = ops[a[0]]["window"]
            if W <= 64:
                if k == "SkipListQuantile":
                    from .leveled import LeveledGen
                    expr = LeveledGen._quantile(self, i)
                    L.append(f"{ind}const {T} v{i} = {expr};")
                elif k == "SkipListMin":
                    L.append(f"{ind}const {T} v{i} = sl{a[0]}.vmin();")
                elif k == "SkipListMax":
                    L.append(f"{ind}const {T} v{i} = sl{a[0]}.vmax();")
                elif k == "SkipListArgMin":
                    L.append(f"{ind}const {T} v{i} = sl{a[0]}.argmin(0);")
                else:
                    L.append(f"{ind}const {T} v{i} = sl{a[0]}.rank({self.val(a[1])});")
            else:
                if k == "SkipListQuantile":
                    L.append(f"{ind}const {T} v{i} = sl{a[0]}.quantile<{T}>({self.lit(op['q'])});")
                elif k == "SkipListMin":
                    L.append(f"{ind}const {T} v{i} = sl{a[0]}.vmin<{T}>();")
                elif k == "SkipListMax":
                    L.append(f"{ind}const {T} v{i} = sl{a[0]}.vmax<{T}>();")
                elif k == "SkipListArgMin":
                    L.append(f"{ind}const {T} v{i} = sl{a[0]}.argmin<{T}>(0);")
                else:
                    L.append(f"{ind}const {T} v{i} = sl{a[0]}.rank<{T}>({self.val(a[1])});")
        elif k == "Accumulator":
            L.append(f"{ind}const {T} v{i} = acc{i};")
        elif k == "SetAccumulator":
            acc = a[0]
            L.append(f"{ind}acc{acc} = kun::ksel({self.val(a[1])}) ? {self.val(a[2])} : {self.val(acc)};")
            L.append(f"{ind}const {T} v{i} = acc{acc};")
        elif not self.emit_simple(i, ind, fplan):
            raise RuntimeError(f"unsupported op {k}")

    # --------------------------------------------------------------- xsec
    def gen_xsec(self):
        ops, T = self.ops, self.T
        kind = self.st["kind"]
        if kind == "generic":
            raise RuntimeError("a GenericCrossSectionalOp with its own C++ body is supported in batch "
                               "mode only, not in stream mode")
        xop = next(i for i, o in enumerate(ops) if o["k"] in ("Rank", "Scale", "DiffWithWeightedSum"))
        ins = [ops[j] for j in ops[xop]["in"]]
        outop = next(o for o in ops if o["k"] == "Output")
        in_slots = [self.slot(o["buf"]) for o in ins]
        out_slot = self.slot(outop["buf"])
        wins = [max(1, self.windows[o["buf"]]) for o in ins]
        wout = max(1, self.windows[outop["buf"]])
        pstruct = f"P_{self.kname}"
        nslots = len(self.slots)
        src = f"""
struct {pstruct} {{
  void* p[{nslots}];
}};
"""
        ring_args = ", ".join([f"(const {T}*)P.p[{sl}], {w}" for sl, w in zip(in_slots, wins)])
        fn = {"rank": "launch_rank_segments", "scale": "launch_scale_segments",
              "xsec": "launch_diffwsum_segments"}[kind]
        fill = "\n".join(f"  P.p[{sl}] = a->buffers[{bid}];" for bid, sl in self.slots.items())
        launch = f"""
extern "C" int {self.kname}_launch(const KunGpuStageArgs* a, void* stream) {{
  {pstruct} P;
{fill}
  if (a->n_active <= 0) return 0;
  return kun::{fn}<{T}>({ring_args}, ({T}*)P.p[{out_slot}], {wout}, a->num_stocks, a->seg_off,
      a->seg_stock0, (const long long*)a->seg_tick, a->nseg, a->max_seg_len, a->seg_count, (cudaStream_t)stream);
}}
"""
        return src, launch
