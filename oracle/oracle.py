"""Python driver of the CPU oracle (``oracle/kunoracle.c``) -- TEST INFRASTRUCTURE.

The oracle is the parity checker for the GPU backend: it interprets a module
spec (see ``kunquant_gb300/graph.py``) with the semantics of the reference's
CPU executor (``cpp/Kun/Runtime.cpp:311-352`` + the op templates in
``cpp/Kun/Ops.hpp``).  Only tests, the smoke check and the CPU-baseline leg of
``bench.py`` use it; the product never imports this module.

    from oracle.oracle import run_oracle
    outs = run_oracle(spec, {"open": o, ...}, cur_time=0, length=T)
"""
import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libkunoracle.so")

OPCODES = {n: i + 1 for i, n in enumerate([
    "Input", "Output", "WindowedTempOutput", "ConstantOp",
    "Add", "Sub", "Mul", "Div", "Max", "Min", "Or", "And",
    "GreaterThan", "GreaterEqual", "LessThan", "LessEqual", "Equals",
    "AddConst", "SubConst", "MulConst", "DivConst", "GreaterThanConst", "LessThanConst",
    "Sqrt", "Log", "Abs", "Sign", "Not", "Exp", "SetInfOrNanToValue",
    "Select", "ForeachBackWindow", "IterValue", "WindowLoopIndex",
    "ReduceAdd", "ReduceMul", "ReduceMin", "ReduceMax", "ReduceArgMax", "ReduceArgMin",
    "ReduceRank", "ReduceDecayLinear",
    "BackRef", "FastWindowedSum", "ExpMovingAvg", "WindowedLinearRegression",
    "WindowedLinearRegressionRSqaureImpl", "WindowedLinearRegressionSlopeImpl",
    "WindowedLinearRegressionResiImpl",
    "SkipListState", "SkipListQuantile", "SkipListRank", "SkipListMin", "SkipListMax",
    "SkipListArgMin", "Accumulator", "SetAccumulator", "ReturnFirstValue",
    "Rank", "Scale", "DiffWithWeightedSum"])}


class KOOp(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("nin", ctypes.c_int32), ("inp", ctypes.c_int32 * 3),
                ("parent", ctypes.c_int32), ("window", ctypes.c_int32),
                ("seg_end", ctypes.c_int32), ("copy_prev", ctypes.c_int32),
                ("buf", ctypes.c_int32), ("single_value", ctypes.c_int32),
                ("swap", ctypes.c_int32), ("loop_window", ctypes.c_int32),
                ("fast_log", ctypes.c_int32), ("fma_pos", ctypes.c_int32),
                ("fma_a", ctypes.c_int32), ("fma_b", ctypes.c_int32),
                ("unrolled", ctypes.c_int32), ("first_iter", ctypes.c_int32),
                ("shared_sq", ctypes.c_int32),
                ("fma_c", ctypes.c_char * 40), ("cval", ctypes.c_char * 40),
                ("qval", ctypes.c_char * 40)]


class KOStage(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("nops", ctypes.c_int32),
                ("ops", ctypes.POINTER(KOOp))]


_lock = threading.Lock()
_lib = None


def build(force=False):
    """Compile the oracle library into ``oracle/_build``."""
    src = os.path.join(HERE, "kunoracle.c")
    deps = [src, os.path.join(HERE, "kunoracle_impl.h"), os.path.join(HERE, "kunoracle.h")]
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(d) for d in deps)):
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-std=gnu11", "-fopenmp", "-ffp-contract=off",
                           "-fno-fast-math", "-shared", "-fPIC", src, "-o", tmp, "-lm"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            for name, ty in (("ko_run_f32", ctypes.c_float), ("ko_run_f64", ctypes.c_double)):
                fn = getattr(L, name)
                fn.restype = ctypes.c_int
                fn.argtypes = [ctypes.POINTER(KOStage), ctypes.c_int,
                               ctypes.POINTER(ctypes.POINTER(ty)), ctypes.POINTER(ctypes.c_int32),
                               ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                               ctypes.c_int]
            for name, ty in (("ko_logfast_f32", ctypes.c_float), ("ko_exp_f32", ctypes.c_float),
                             ("ko_logfast_f64", ctypes.c_double), ("ko_exp_f64", ctypes.c_double)):
                fn = getattr(L, name)
                fn.restype = None
                fn.argtypes = [ctypes.POINTER(ty), ctypes.POINTER(ty), ctypes.c_int64]
            L.ko_last_error.restype = ctypes.c_char_p
            _lib = L
        return _lib


def stage_order(spec):
    """Topological order of the stage DAG (dependency counts of
    ``cpp/Kun/Runtime.cpp:141-178``)."""
    stages = spec["stages"]
    pending = [s.get("pending", 0) for s in stages]
    ready = [i for i, p in enumerate(pending) if p == 0]
    order = []
    while ready:
        i = ready.pop(0)
        order.append(i)
        for d in stages[i].get("deps", []):
            pending[d] -= 1
            if pending[d] == 0:
                ready.append(d)
    if len(order) != len(stages):
        raise RuntimeError("cyclic stage graph")
    return order


UNROLL_MAX_TRIPS = int(os.environ.get("KO_UNROLL_MAX", "17"))
# approximate GIMPLE size of a back-window loop body, calibrated on loops the
# reference build does and does not unroll completely (GCC: at most 16 peeled
# iterations and ~200 insns after its 2/3 discount, i.e. trips * size <= 300)
_RED_SIZE = {"ReduceAdd": 4, "ReduceMul": 1, "ReduceMin": 3, "ReduceMax": 3, "ReduceArgMax": 6,
             "ReduceArgMin": 6, "ReduceRank": 7, "ReduceDecayLinear": 2}


def _loop_body_size(ops, loop, memo):
    if loop in memo:
        return memo[loop]
    size = 2.0
    prev = None
    for j in range(loop - 1, -1, -1):
        if ops[j]["k"] == "ForeachBackWindow":
            prev = j
            break
    if ops[loop].get("copy_prev_body") and prev is not None:
        size += _loop_body_size(ops, prev, memo) - 2.0
    for j, q in enumerate(ops):
        if q.get("p", -1) == loop:
            if q["k"] == "IterValue":
                size += 4.5 if ops[q["in"][1]]["k"] in ("Input", "Output") else 6.0
            else:
                size += 1.0
        elif q["k"] in _RED_SIZE:
            src = q["in"][0]
            lp = src if ops[src]["k"] == "ForeachBackWindow" else ops[src].get("p", -1)
            if lp == loop:
                size += _RED_SIZE[q["k"]]
    memo[loop] = size
    return size


def loop_unrolled(ops, loop):
    trips = ops[loop]["window"] - ops[loop].get("segment_end", 0)
    if trips > UNROLL_MAX_TRIPS:
        return False
    return trips * _loop_body_size(ops, loop, {}) <= 300
_ADDITIVE = {"Add", "Sub", "AddConst", "SubConst", "ReduceAdd"}
_BRANCHY_SOURCES = {"Input", "Output"}


def contraction_plan(ops):
    """Which products the reference build evaluates as fused multiply-adds.

    GCC (the reference's JIT compiler, ``KunQuant/jit/cfake.py:88-114``)
    contracts a multiplication into an FMA when every use of its result is an
    addition or subtraction in the same basic block.  In the generated stage
    code (``KunQuant/passes/CodegenCpp.py:189-307``) a basic block ends at
    every inner back-window loop and after every inlined template that
    branches on the time index (a windowed read of an input/output buffer).
    The body of each back-window loop is one block.  Returns
    {use op index: (input position, product op index)}.
    """
    n = len(ops)
    bb = [0] * n
    cur = 0
    for i, op in enumerate(ops):
        p = op.get("p", -1)
        if p >= 0:
            bb[i] = ("loop", p)
            continue
        k = op["k"]
        if k == "ForeachBackWindow":
            cur += 1
            bb[i] = cur
            cur += 1
            continue
        bb[i] = cur
        src_branchy = bool(op["in"]) and ops[op["in"][0]]["k"] in _BRANCHY_SOURCES
        if (k == "BackRef" or (k in ("FastWindowedSum", "WindowedLinearRegression") and src_branchy)
                or k.startswith("SkipList")):
            cur += 1
    # ReduceAdd's step lives in its loop body
    for i, op in enumerate(ops):
        if op["k"] == "ReduceAdd":
            src = op["in"][0]
            loop = src if ops[src]["k"] == "ForeachBackWindow" else ops[src].get("p", -1)
            bb[i] = ("loop", loop)
    users = [[] for _ in range(n)]
    for i, op in enumerate(ops):
        for j, v in enumerate(op["in"]):
            users[v].append((i, j))
    converted = set()
    plan = {}
    for i, op in enumerate(ops):
        if op["k"] not in ("Mul", "MulConst"):
            continue
        us = users[i]
        if not us:
            continue
        ok = True
        for (u, j) in us:
            k = ops[u]["k"]
            if k not in _ADDITIVE or u in converted or bb[u] != bb[i]:
                ok = False
                break
            if k == "ReduceAdd" and j != 0:
                ok = False
                break
            if k in ("Add", "Sub") and ops[u]["in"][0] == ops[u]["in"][1]:
                ok = False
                break
        if not ok:
            continue
        for (u, j) in us:
            plan[u] = (j, i)
            converted.add(u)
    return plan


def _encode_stage(spec, st):
    if st["kind"] == "generic":
        raise NotImplementedError("the oracle does not run GenericCrossSectionalOp C++ bodies; "
                                  "their parity is pinned on the reference's own outputs")
    ops = st["ops"]
    arr = (KOOp * len(ops))()
    fplan = contraction_plan(ops) if st["kind"] == "ts" else {}
    fast_log = 1 if spec.get("options", {}).get("fast_log", True) else 0
    last_loop_window = 0
    for i, op in enumerate(ops):
        k = op["k"]
        if k not in OPCODES:
            raise RuntimeError("oracle: unsupported op " + k)
        o = arr[i]
        o.kind = OPCODES[k]
        o.nin = len(op["in"])
        if o.nin > 3:
            raise RuntimeError("oracle: too many inputs for " + k)
        for j, v in enumerate(op["in"]):
            o.inp[j] = v
        o.parent = op.get("p", -1)
        o.window = op.get("window", 0)
        o.seg_end = op.get("segment_end", 0)
        o.copy_prev = 1 if op.get("copy_prev_body") else 0
        o.buf = op.get("buf", -1)
        o.single_value = 1 if op.get("single_value") else 0
        o.swap = 1 if op.get("swap") else 0
        o.fast_log = fast_log
        if k == "ForeachBackWindow":
            last_loop_window = op["window"]
        o.loop_window = last_loop_window
        o.fma_pos = -1
        if i in fplan:
            pos, prod = fplan[i]
            po = ops[prod]
            o.fma_pos = pos
            o.fma_a = po["in"][0]
            if po["k"] == "Mul":
                o.fma_b = po["in"][1]
            else:
                o.fma_b = -1
                o.fma_c = po["value"].encode()
        if k == "WindowedLinearRegression":
            o.shared_sq = 1 if sum(1 for q in ops if q["k"] == k and q["in"][0] == op["in"][0]) > 1 else 0
        if k == "ReduceAdd":
            src = op["in"][0]
            loop = src if ops[src]["k"] == "ForeachBackWindow" else ops[src].get("p", -1)
            lw = ops[loop]["window"]
            o.unrolled = 1 if loop_unrolled(ops, loop) else 0
            o.first_iter = lw - 1
        if "value" in op:
            o.cval = op["value"].encode()
        if "q" in op:
            o.qval = op["q"].encode()
    kind = {"ts": 0, "rank": 1, "scale": 2, "xsec": 3}[st["kind"]]
    return kind, arr


class OracleProgram:
    """A module spec flattened once for repeated oracle runs."""

    def __init__(self, spec):
        self.spec = spec
        self.dtype = np.float32 if spec["dtype"] == "float" else np.float64
        order = stage_order(spec)
        self.stages = (KOStage * len(order))()
        self._keep = []
        for j, si in enumerate(order):
            kind, arr = _encode_stage(spec, spec["stages"][si])
            self._keep.append(arr)
            self.stages[j].kind = kind
            self.stages[j].nops = len(arr)
            self.stages[j].ops = ctypes.cast(arr, ctypes.POINTER(KOOp))

    def run(self, inputs, cur_time=0, length=None, num_stocks=None, nthreads=None, outputs=None):
        """Inputs and outputs in the spec's layouts; the STs layout
        ([S/L][T][L], Module.hpp / LayoutMappers.hpp:19-22) is converted to
        and from [T][S] around the computation, which is layout-free."""
        spec = self.spec
        L = spec.get("blocking_len", 8)
        if spec.get("input_layout") == "STs":
            sv = set(spec.get("single_value_inputs", []))
            conv = {}
            for k, a in inputs.items():
                if k in sv or np.ndim(a) != 3:
                    conv[k] = a
                else:
                    nb, T_, Lb = a.shape
                    conv[k] = np.ascontiguousarray(np.asarray(a).transpose(1, 0, 2).reshape(T_, nb * Lb))
            inputs = conv
        if spec.get("output_layout") == "STs":
            ts = self._run_ts(inputs, cur_time, length, num_stocks, nthreads, None)
            out = {}
            for k, a in ts.items():
                T_, S_ = a.shape
                pad = (-S_) % L
                if pad:
                    a = np.concatenate([a, np.zeros((T_, pad), a.dtype)], axis=1)
                out[k] = np.ascontiguousarray(a.reshape(T_, -1, L).transpose(1, 0, 2))
            return out
        return self._run_ts(inputs, cur_time, length, num_stocks, nthreads, outputs)

    def _run_ts(self, inputs, cur_time=0, length=None, num_stocks=None, nthreads=None, outputs=None):
        spec = self.spec
        T = None
        S = num_stocks
        sv = set(spec.get("single_value_inputs", []))
        for b in spec["buffers"]:
            if b["kind"] == "INPUT" and b["name"] not in sv:
                a = inputs[b["name"]]
                T, S = a.shape[0], a.shape[1]
                break
        if length is None:
            length = T - cur_time
        if cur_time + length > T:
            raise ValueError("Bad parameter: length")
        bufs = []
        keep = []
        is_in = (ctypes.c_int32 * len(spec["buffers"]))()
        out = {}
        for b in spec["buffers"]:
            if b["kind"] == "INPUT":
                a = np.ascontiguousarray(inputs[b["name"]], dtype=self.dtype)
                is_in[b["id"]] = 1
            else:
                if outputs is not None and b["name"] in outputs:
                    a = outputs[b["name"]]
                else:
                    a = np.full((length, S), np.nan, dtype=self.dtype)
                if b["kind"] == "OUTPUT":
                    out[b["name"]] = a
            keep.append(a)
        ty = ctypes.c_float if self.dtype == np.float32 else ctypes.c_double
        ptrs = (ctypes.POINTER(ty) * len(keep))()
        for i, a in enumerate(keep):
            ptrs[i] = a.ctypes.data_as(ctypes.POINTER(ty))
        fn = lib().ko_run_f32 if self.dtype == np.float32 else lib().ko_run_f64
        nthreads = nthreads or min(os.cpu_count() or 1, 16)
        rc = fn(self.stages, len(self.stages), ptrs, is_in, S, T, cur_time, length, nthreads)
        if rc != 0:
            raise RuntimeError("oracle failed: " + lib().ko_last_error().decode())
        return out


def run_oracle(spec, inputs, cur_time=0, length=None, nthreads=None):
    return OracleProgram(spec).run(inputs, cur_time=cur_time, length=length, nthreads=nthreads)


def logfast(x):
    x = np.ascontiguousarray(x)
    y = np.empty_like(x)
    ty = ctypes.c_float if x.dtype == np.float32 else ctypes.c_double
    fn = lib().ko_logfast_f32 if x.dtype == np.float32 else lib().ko_logfast_f64
    fn(x.ctypes.data_as(ctypes.POINTER(ty)), y.ctypes.data_as(ctypes.POINTER(ty)), x.size)
    return y


def expk(x):
    x = np.ascontiguousarray(x)
    y = np.empty_like(x)
    ty = ctypes.c_float if x.dtype == np.float32 else ctypes.c_double
    fn = lib().ko_exp_f32 if x.dtype == np.float32 else lib().ko_exp_f64
    fn(x.ctypes.data_as(ctypes.POINTER(ty)), y.ctypes.data_as(ctypes.POINTER(ty)), x.size)
    return y
