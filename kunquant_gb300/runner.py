"""Python front of the GPU runtime, mirroring ``KunQuant.runner.KunRunner``
(``cpp/Python/PyBinding.cpp:146-596``): executors, ``Library``/``Module``,
``runGraph`` and ``StreamContext`` with the same argument names, defaults,
shape rules and error strings.

``runGraph`` accepts numpy arrays (host path: the runtime copies them to the
GPU and the outputs back) or torch CUDA tensors (device path: the graph is
enqueued on torch's current stream and the outputs are torch tensors).  There
is no CPU execution path: without the CUDA runtime library every call fails.
"""
import ctypes
import os
import threading
from typing import Dict, Optional

import numpy as np

from . import build as _build

_lib = None
_lock = threading.Lock()


class KunError(RuntimeError):
    pass


def _load_runtime():
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.runtime_path()
        if not os.path.exists(path):
            _build.build_runtime()
        L = ctypes.CDLL(path)
        vp, sz, cp, i32, i64 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_int, ctypes.c_int64
        sig = {
            "kunCreateSingleThreadExecutor": (vp, []),
            "kunCreateMultiThreadExecutor": (vp, [i32]),
            "kunDestoryExecutor": (None, [vp]),
            "kunLoadLibrary": (vp, [cp]),
            "kunGetModuleFromLibrary": (vp, [vp, cp]),
            "kunUnloadLibrary": (None, [vp]),
            "kunCreateBufferNameMap": (vp, []),
            "kunDestoryBufferNameMap": (None, [vp]),
            "kunSetBufferNameMap": (None, [vp, cp, vp]),
            "kunEraseBufferNameMap": (None, [vp, cp]),
            "kunRunGraph": (None, [vp, vp, vp, sz, sz, sz, sz]),
            "kunRunGraphEx": (i32, [vp, vp, vp, sz, sz, sz, sz, i32]),
            "kunExecutorSetStream": (i32, [vp, vp]),
            "kunExecutorClearStream": (i32, [vp]),
            "kunExecutorSynchronize": (i32, [vp]),
            "kunExecutorLastLaunchCount": (i64, [vp]),
            "kunExecutorSetProfiling": (i32, [vp, i32]),
            "kunExecutorSetGraphs": (i32, [vp, i32]),
            "kunExecutorStageTimes": (i32, [vp, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_float), i32]),
            "kunGetLastError": (cp, []),
            "kunModuleNumBuffers": (i32, [vp]),
            "kunModuleBufferName": (cp, [vp, i32]),
            "kunModuleBufferKind": (i32, [vp, i32]),
            "kunModuleBufferUnreliableCount": (i32, [vp, i32]),
            "kunModuleBufferWindow": (i32, [vp, i32]),
            "kunModuleInputLayout": (i32, [vp]),
            "kunModuleOutputLayout": (i32, [vp]),
            "kunModuleBlockingLen": (i32, [vp]),
            "kunModuleDtype": (i32, [vp]),
            "kunModuleNumStages": (i32, [vp]),
            "kunCreateStream": (vp, [vp, vp, sz]),
            "kunCreateStreamEx": (i32, [vp, vp, sz, vp, ctypes.POINTER(vp)]),
            "kunStreamSerializeStates": (i32, [vp, i32, vp, ctypes.POINTER(sz)]),
            "kunQueryBufferHandle": (sz, [vp, cp]),
            "kunStreamGetCurrentBuffer": (vp, [vp, sz]),
            "kunStreamPushData": (None, [vp, sz, vp]),
            "kunStreamRun": (None, [vp]),
            "kunDestoryStream": (None, [vp]),
            "kunStreamPushDataDevice": (i32, [vp, sz, vp]),
            "kunStreamGetCurrentBufferDevice": (vp, [vp, sz]),
            "kunStreamRunEx": (i32, [vp, i32]),
            "kunStreamCopyCurrentDevice": (i32, [vp, sz, vp]),
            "kunStreamTick": (i64, [vp]),
            "kunStreamBytesPerStock": (i64, [vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
        return L


def runtime():
    return _load_runtime()


def _err() -> str:
    return runtime().kunGetLastError().decode()


def _check(rc: int):
    if rc != 0:
        raise KunError(_err() or f"KunStatus {rc}")


_LAYOUTS = {0: "STs", 1: "TS", 2: "STREAM"}


class Executor:
    """A GPU execution context (replaces the CPU thread pool)."""

    def __init__(self, handle):
        if not handle:
            raise KunError("cannot create executor: " + _err())
        self.handle = handle

    def __del__(self):
        try:
            if self.handle and _lib is not None:
                _lib.kunDestoryExecutor(self.handle)
        except Exception:
            pass
        self.handle = None

    def synchronize(self):
        _check(runtime().kunExecutorSynchronize(self.handle))

    def last_launch_count(self) -> int:
        return int(runtime().kunExecutorLastLaunchCount(self.handle))

    def set_graphs(self, enable: bool):
        _check(runtime().kunExecutorSetGraphs(self.handle, 1 if enable else 0))

    def set_profiling(self, enable: bool):
        _check(runtime().kunExecutorSetProfiling(self.handle, 1 if enable else 0))

    def stage_times(self, cap: int = 4096):
        """[(stage id, ms)] of the last profiled run, in launch order."""
        ids = (ctypes.c_int32 * cap)()
        ms = (ctypes.c_float * cap)()
        n = runtime().kunExecutorStageTimes(self.handle, ids, ms, cap)
        if n < 0:
            raise KunError("profiling is not enabled")
        return [(int(ids[i]), float(ms[i])) for i in range(n)]


def createSingleThreadExecutor() -> Executor:
    return Executor(runtime().kunCreateSingleThreadExecutor())


def createMultiThreadExecutor(num_threads: int) -> Executor:
    return Executor(runtime().kunCreateMultiThreadExecutor(int(num_threads)))


class Module:
    def __init__(self, handle, lib: "Library"):
        self.handle = handle
        self._lib = lib  # keeps the library loaded (PyBinding.cpp:66-73)
        L = runtime()
        self.num_buffers = L.kunModuleNumBuffers(handle)
        self.buffers = []
        for i in range(self.num_buffers):
            self.buffers.append({
                "name": L.kunModuleBufferName(handle, i).decode(),
                "kind": L.kunModuleBufferKind(handle, i),
                "unreliable_count": L.kunModuleBufferUnreliableCount(handle, i),
                "window": L.kunModuleBufferWindow(handle, i),
            })
        self.input_layout = _LAYOUTS[L.kunModuleInputLayout(handle)]
        self.output_layout = _LAYOUTS[L.kunModuleOutputLayout(handle)]
        self.blocking_len = L.kunModuleBlockingLen(handle)
        self.dtype = np.float32 if L.kunModuleDtype(handle) == 0 else np.float64
        self.num_stages = L.kunModuleNumStages(handle)

    def getOutputNames(self):
        return [b["name"] for b in self.buffers if b["kind"] == 1]

    def getInputNames(self):
        return [b["name"] for b in self.buffers if b["kind"] == 0]

    def getOutputUnreliableCount(self) -> Dict[str, int]:
        return {b["name"]: b["unreliable_count"] for b in self.buffers if b["kind"] == 1}


class Library:
    def __init__(self, handle, path):
        self.handle = handle
        self.path = path

    @staticmethod
    def load(filename: str) -> "Library":
        h = runtime().kunLoadLibrary(os.fsencode(filename))
        if not h:
            raise KunError("Cannot load library")
        return Library(h, filename)

    @staticmethod
    def predefined(key: str) -> "Library":
        """Load (building if needed) a shipped Alpha101/Alpha158 library,
        e.g. ``alpha158_f32``."""
        return Library.load(_build.predefined_library(key))

    def getModule(self, name: str) -> Module:
        h = runtime().kunGetModuleFromLibrary(self.handle, name.encode())
        if not h:
            raise KunError("Module name not found")
        return Module(h, self)

    def __del__(self):
        # modules borrow the library: unloading is left to process exit
        pass


def _is_torch_cuda(x) -> bool:
    t = type(x)
    return t.__module__.startswith("torch") and getattr(x, "is_cuda", False)


def _check_contiguous(a, name, shape, dtype, torch_mode):
    if torch_mode:
        import torch
        want = torch.float32 if dtype == np.float32 else torch.float64
        if a.dtype != want:
            raise KunError(("Expecting float buffer at " if dtype == np.float32 else "Expecting double buffer at ") + name)
        got = tuple(a.shape)
        contiguous = a.is_contiguous()
    else:
        if a.dtype != dtype:
            raise KunError(("Expecting float buffer at " if dtype == np.float32 else "Expecting double buffer at ") + name)
        got = tuple(a.shape)
        contiguous = a.flags["C_CONTIGUOUS"]
    if got != tuple(shape):
        raise KunError(f"Bad shape at {name} expected {tuple(shape)} but got {got}")
    if any(s <= 0 for s in got):
        raise KunError("Bad dimension number at " + name)
    if not contiguous:
        raise KunError("Bad stride at " + name)


def runGraph(exec: Executor, mod: Module, inputs: dict, cur_time: int, length: int,
             outputs: Optional[dict] = None, skip_check: bool = False, num_stocks: int = -1):
    """Batch run (``cpp/Python/PyBinding.cpp:242-394``)."""
    if outputs is None:
        outputs = {}
    if not inputs:
        raise KunError("no inputs")
    torch_mode = any(_is_torch_cuda(v) for v in inputs.values())
    if torch_mode and not all(_is_torch_cuda(v) for v in inputs.values()):
        raise KunError("inputs must be all numpy arrays or all torch CUDA tensors")
    dtype = mod.dtype
    simd = mod.blocking_len
    known_S = known_T = known_N = 0
    for name, a in inputs.items():
        shape = tuple(a.shape)
        if name.startswith("__init"):
            if not skip_check:
                if len(shape) != 1:
                    raise KunError("Bad Init shape at " + name)
                if not known_N:
                    known_N = shape[0]
                _check_contiguous(a, name, (known_N,), dtype, torch_mode)
            continue
        if mod.input_layout == "STs":
            if len(shape) != 3:
                raise KunError("Bad STs shape at " + name)
            if known_S == 0:
                known_S, known_T = shape[0], shape[1]
                known_N = known_N or known_S * simd
            if not skip_check:
                _check_contiguous(a, name, (known_S, known_T, simd), dtype, torch_mode)
        elif mod.input_layout == "TS":
            if len(shape) != 2:
                raise KunError("Bad TS shape at " + name)
            if known_T == 0:
                known_T = shape[0]
                known_S = shape[1] // simd
                known_N = known_N or shape[1]
            if not skip_check:
                _check_contiguous(a, name, (known_T, known_N), dtype, torch_mode)
        else:
            raise KunError("Unknown layout at " + name)
    if num_stocks < 0:
        num_stocks = known_N
    if not skip_check:
        if length > known_T:
            raise KunError("Bad parameter: length")
        if mod.input_layout == "STs":
            if num_stocks > known_N or num_stocks <= known_N - simd:
                raise KunError("num_stocks does not match the shape of inputs")
        elif num_stocks != known_N:
            raise KunError("num_stocks does not match the shape of inputs")
    if mod.output_layout == "STs":
        out_shape = (known_S if known_S * simd >= num_stocks else (num_stocks + simd - 1) // simd, length, simd)
    else:
        out_shape = (length, num_stocks)
    L = runtime()
    m = L.kunCreateBufferNameMap()
    keep = []
    ret = {}
    try:
        for name, a in inputs.items():
            if torch_mode:
                L.kunSetBufferNameMap(m, name.encode(), ctypes.c_void_p(a.data_ptr()))
            else:
                a = np.ascontiguousarray(a)
                keep.append(a)
                L.kunSetBufferNameMap(m, name.encode(), a.ctypes.data_as(ctypes.c_void_p))
        for name in mod.getOutputNames():
            if name in outputs:
                o = outputs[name]
                if not skip_check:
                    _check_contiguous(o, name, out_shape, dtype, torch_mode)
            elif torch_mode:
                import torch
                dev = next(iter(inputs.values())).device
                o = torch.empty(out_shape, dtype=torch.float32 if dtype == np.float32 else torch.float64,
                                device=dev)
            else:
                o = np.empty(out_shape, dtype=dtype)
            ptr = o.data_ptr() if torch_mode else o.ctypes.data
            L.kunSetBufferNameMap(m, name.encode(), ctypes.c_void_p(ptr))
            ret[name] = o
        if torch_mode:
            import torch
            L.kunExecutorSetStream(exec.handle, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
            rc = L.kunRunGraphEx(exec.handle, mod.handle, m, num_stocks, known_T, cur_time, length, 0)
            L.kunExecutorClearStream(exec.handle)
        else:
            rc = L.kunRunGraphEx(exec.handle, mod.handle, m, num_stocks, known_T, cur_time, length, 1)
        _check(rc)
    finally:
        L.kunDestoryBufferNameMap(m)
    return ret


class _InitUnion(ctypes.Union):
    class _Mem(ctypes.Structure):
        _fields_ = [("buffer", ctypes.c_void_p), ("size", ctypes.c_size_t)]
    _fields_ = [("path", ctypes.c_char_p), ("memory", _Mem)]


class _StreamExtraArgs(ctypes.Structure):
    _fields_ = [("version", ctypes.c_size_t), ("init_kind", ctypes.c_int), ("init", _InitUnion)]


_KUN_INIT_NONE, _KUN_INIT_FILE, _KUN_INIT_MEMORY = 0, 1, 2


class StreamContext:
    """One stream session (``cpp/Python/PyBinding.cpp:508-596``): per tick,
    ``pushData`` one row of every input, ``run`` and read the outputs with
    ``getCurrentBuffer``.  ``init`` restores a ``serializeStates`` dump (a
    file name or bytes).  Numpy rows go through host memory; torch CUDA rows
    are pushed device to device (``pushData``) and ``getCurrentBufferDevice``
    returns the output row as a torch tensor without a copy to the host."""

    def __init__(self, exec: Executor, mod: Module, num_stocks: int, init=None):
        if mod.output_layout != "STREAM":
            raise KunError("Cannot run batch mode module via StreamContext")
        L = runtime()
        self._exec, self._mod, self.num_stocks = exec, mod, int(num_stocks)
        self.handle = None
        out = ctypes.c_void_p()
        if init is None:
            rc = L.kunCreateStreamEx(exec.handle, mod.handle, self.num_stocks, None, ctypes.byref(out))
        else:
            extra = _StreamExtraArgs()
            extra.version = 1
            if isinstance(init, str):
                extra.init_kind = _KUN_INIT_FILE
                path = os.fsencode(init)
                extra.init.path = path
            elif isinstance(init, (bytes, bytearray)):
                extra.init_kind = _KUN_INIT_MEMORY
                data = ctypes.create_string_buffer(bytes(init), len(init))
                extra.init.memory.buffer = ctypes.cast(data, ctypes.c_void_p)
                extra.init.memory.size = len(init)
            else:
                raise KunError("Bad type for init, expecting filename or bytes")
            rc = L.kunCreateStreamEx(exec.handle, mod.handle, self.num_stocks, ctypes.byref(extra),
                                     ctypes.byref(out))
        _check(rc)
        self.handle = out.value
        self._rows = {}

    def __del__(self):
        if getattr(self, "handle", None) and _lib is not None:
            _lib.kunDestoryStream(self.handle)
            self.handle = None

    def queryBufferHandle(self, name: str) -> int:
        h = runtime().kunQueryBufferHandle(self.handle, name.encode())
        if h == ctypes.c_size_t(-1).value:
            raise KunError("Cannot find the buffer name")
        return h

    def _check_handle(self, handle):
        if not (0 <= handle < self._mod.num_buffers):
            raise KunError("Bad buffer handle")

    def pushData(self, handle: int, data):
        self._check_handle(handle)
        dtype = self._mod.dtype
        if _is_torch_cuda(data):
            import torch
            want = torch.float32 if dtype == np.float32 else torch.float64
            if data.dtype != want or not data.is_contiguous():
                raise KunError("Bad input type to push, expecting float")
            if data.dim() != 1 or data.shape[0] != self.num_stocks:
                raise KunError("Bad dimension for input data to push")
            L = runtime()
            # order the device copy after torch's producer of `data`
            torch.cuda.current_stream().synchronize()
            _check(L.kunStreamPushDataDevice(self.handle, handle, ctypes.c_void_p(data.data_ptr())))
            return
        if not isinstance(data, np.ndarray) or data.dtype != dtype or not data.flags["C_CONTIGUOUS"]:
            raise KunError("Bad input type to push, expecting float")
        if data.ndim != 1 or data.shape[0] != self.num_stocks:
            raise KunError("Bad dimension for input data to push")
        runtime().kunStreamPushData(self.handle, handle, data.ctypes.data_as(ctypes.c_void_p))

    def run(self, synchronize: bool = True):
        _check(runtime().kunStreamRunEx(self.handle, 1 if synchronize else 0))

    def getCurrentBuffer(self, handle: int) -> np.ndarray:
        """The current row of a buffer, copied to the host (a fresh array)."""
        self._check_handle(handle)
        p = runtime().kunStreamGetCurrentBuffer(self.handle, handle)
        if not p:
            raise KunError(_err())
        ct = ctypes.c_float if self._mod.dtype == np.float32 else ctypes.c_double
        arr = np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ct)), shape=(self.num_stocks,))
        return arr.copy()

    def getCurrentBufferDevice(self, handle: int):
        """The current row of a buffer as a torch CUDA tensor (a copy made on
        the device, valid after later ticks)."""
        import torch
        self._check_handle(handle)
        L = runtime()
        p = L.kunStreamGetCurrentBufferDevice(self.handle, handle)
        if not p:
            raise KunError(_err())
        dt = torch.float32 if self._mod.dtype == np.float32 else torch.float64
        out = torch.empty(self.num_stocks, dtype=dt, device="cuda")
        _check(L.kunStreamCopyCurrentDevice(self.handle, handle, ctypes.c_void_p(out.data_ptr())))
        return out

    def tick(self) -> int:
        return runtime().kunStreamTick(self.handle)

    def serializeStates(self, fileNameOrNone=None):
        L = runtime()
        if isinstance(fileNameOrNone, str):
            n = ctypes.c_size_t(0)
            path = ctypes.create_string_buffer(os.fsencode(fileNameOrNone))
            rc = L.kunStreamSerializeStates(self.handle, _KUN_INIT_FILE, ctypes.cast(path, ctypes.c_void_p),
                                            ctypes.byref(n))
            if rc != 0:
                raise KunError("Failed to serialize states")
            return None
        n = ctypes.c_size_t(0)
        rc = L.kunStreamSerializeStates(self.handle, _KUN_INIT_MEMORY, None, ctypes.byref(n))
        if rc not in (0, 1):
            raise KunError("Failed to serialize states")
        buf = ctypes.create_string_buffer(n.value)
        rc = L.kunStreamSerializeStates(self.handle, _KUN_INIT_MEMORY, ctypes.cast(buf, ctypes.c_void_p),
                                        ctypes.byref(n))
        if rc != 0:
            raise KunError("Failed to serialize states")
        return buf.raw[:n.value]


def streamBytesPerStock(mod: Module) -> int:
    """Device bytes one stock of a stream module occupies (rings + states)."""
    return int(runtime().kunStreamBytesPerStock(mod.handle))


def _batch_maps(mod: Module, inputs_list, outputs_list, cur_time, length):
    """Buffer maps and shapes of a list of jobs (torch CUDA tensors, [T][S])."""
    import torch
    L = runtime()
    dt = torch.float32 if mod.dtype == np.float32 else torch.float64
    maps, S, TT, CT, LN, outs = [], [], [], [], [], []
    for j, inp in enumerate(inputs_list):
        if not inp or not all(_is_torch_cuda(v) for v in inp.values()):
            raise KunError("runGraphBatch takes torch CUDA tensors")
        T, n = next(iter(inp.values())).shape
        ln = (T - cur_time) if length is None else length
        o = dict(outputs_list[j]) if outputs_list else {}
        m = L.kunCreateBufferNameMap()
        maps.append(m)
        for k, v in inp.items():
            _check_contiguous(v, k, (T, n), mod.dtype, True)
            L.kunSetBufferNameMap(m, k.encode(), ctypes.c_void_p(v.data_ptr()))
        for k in mod.getOutputNames():
            if k not in o:
                o[k] = torch.empty((ln, n), dtype=dt, device=next(iter(inp.values())).device)
            L.kunSetBufferNameMap(m, k.encode(), ctypes.c_void_p(o[k].data_ptr()))
        outs.append(o)
        S.append(n), TT.append(T), CT.append(cur_time), LN.append(ln)
    arr = lambda xs, t: (t * len(xs))(*xs)  # noqa: E731
    return (maps, (ctypes.c_void_p * len(maps))(*maps), arr(S, ctypes.c_size_t), arr(TT, ctypes.c_size_t),
            arr(CT, ctypes.c_size_t), arr(LN, ctypes.c_size_t), outs)


def _batch_sigs(L):
    if not getattr(L, "_batch_sigs", False):
        vp, i32 = ctypes.c_void_p, ctypes.c_int
        szp = ctypes.POINTER(ctypes.c_size_t)
        L.kunRunGraphBatch.restype = i32
        L.kunRunGraphBatch.argtypes = [vp, vp, i32, ctypes.POINTER(vp), szp, szp, szp, szp, i32]
        L.kunExecutorTune.restype = i32
        L.kunExecutorTune.argtypes = [vp, vp, i32, ctypes.POINTER(vp), szp, szp, szp, szp, i32]
        L.kunExecutorTunedShape.restype = i32
        L.kunExecutorTunedShape.argtypes = [vp, vp, i32, ctypes.POINTER(ctypes.c_int32),
                                            ctypes.POINTER(ctypes.c_int32), i32]
        L.kunExecutorClearTuning.restype = i32
        L.kunExecutorClearTuning.argtypes = [vp]
        L._batch_sigs = True
    return L


def runGraphBatch(exec: Executor, mod: Module, inputs_list, cur_time: int = 0, length: Optional[int] = None,
                  outputs_list=None):
    """Run many universes of one module in one call (GPU extension): each
    element of ``inputs_list`` is one universe's inputs (torch CUDA tensors,
    [T][S], any S and T).  Returns the list of output dicts."""
    import torch
    L = _batch_sigs(runtime())
    maps, cmaps, S, TT, CT, LN, outs = _batch_maps(mod, inputs_list, outputs_list, cur_time, length)
    try:
        L.kunExecutorSetStream(exec.handle, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        rc = L.kunRunGraphBatch(exec.handle, mod.handle, len(maps), cmaps, S, TT, CT, LN, 1)
        L.kunExecutorClearStream(exec.handle)
        _check(rc)
    finally:
        for m in maps:
            L.kunDestoryBufferNameMap(m)
    return outs


def tune(exec: Executor, mod: Module, inputs_list, cur_time: int = 0, length: Optional[int] = None, reps: int = 2):
    """Autotune the launch shapes (time tile, threads per block) of every
    time-series stage of ``mod`` on these universes; the executor keeps them
    for later runs of the module.  Returns the number of stages tuned."""
    import torch
    L = _batch_sigs(runtime())
    maps, cmaps, S, TT, CT, LN, _ = _batch_maps(mod, inputs_list, None, cur_time, length)
    try:
        torch.cuda.synchronize()
        n = L.kunExecutorTune(exec.handle, mod.handle, len(maps), cmaps, S, TT, CT, LN, reps)
    finally:
        for m in maps:
            L.kunDestoryBufferNameMap(m)
    if n < 0:
        raise KunError(_err() or "tuning failed")
    return n


def tunedShape(exec: Executor, mod: Module, stage: int):
    """(time tiles, threads per block) chosen for one stage, or None."""
    L = _batch_sigs(runtime())
    t = (ctypes.c_int32 * 64)()
    b = (ctypes.c_int32 * 64)()
    n = L.kunExecutorTunedShape(exec.handle, mod.handle, stage, t, b, 64)
    if n <= 0:
        return None
    return list(t[:n]), list(b[:n])


_AGG_KINDS = ["sum", "min", "max", "first", "last", "count", "mean"]


def _to_device(a):
    """(torch CUDA tensor, was_numpy) of an array."""
    import torch
    if _is_torch_cuda(a):
        return a, False
    return torch.from_numpy(np.ascontiguousarray(a)).cuda(), True


def corrWith(exec: Executor, inputs, corr_with, outs, layout: str = "TS", rank_inputs: bool = False):
    """Cross-sectional correlation of every row of each input with the same
    row of ``corr_with`` (``cpp/Python/PyBinding.cpp:396-447``): ``outs[k][t]``.
    numpy arrays or torch CUDA tensors; fp32."""
    import torch
    if layout not in ("TS", "STs"):
        raise KunError("Unknown layout" + layout)
    if len(inputs) != len(outs):
        raise KunError("number of inputs and outputs should match")
    L = runtime()
    if not getattr(L, "_util_sigs", False):
        vp, sz, i32 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int
        L.kunCorrWith.restype = i32
        L.kunCorrWith.argtypes = [vp, i32, ctypes.POINTER(vp), vp, ctypes.POINTER(vp), sz, sz, i32, i32]
        L.kunAggregrate.restype = i32
        L.kunAggregrate.argtypes = [vp, i32, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp), sz, sz, i32]
        L._util_sigs = True
    y, _ = _to_device(corr_with)
    if y.dtype != torch.float32:
        raise KunError("Expecting float buffer at corr_with")
    if layout == "TS":
        T, S = y.shape
    else:
        nb, T, blk = y.shape
        S = nb * blk
    dev_in = []
    for i, a in enumerate(inputs):
        d, _ = _to_device(a)
        if tuple(d.shape) != tuple(y.shape) or d.dtype != torch.float32:
            raise KunError(f"Bad shape at buffer_{i}")
        dev_in.append(d.contiguous())
    dev_out = [torch.empty(T, dtype=torch.float32, device=y.device) for _ in outs]
    pin = (ctypes.c_void_p * len(dev_in))(*[d.data_ptr() for d in dev_in])
    pout = (ctypes.c_void_p * len(dev_out))(*[d.data_ptr() for d in dev_out])
    L.kunExecutorSetStream(exec.handle, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    rc = L.kunCorrWith(exec.handle, len(dev_in), pin, ctypes.c_void_p(y.contiguous().data_ptr()), pout, S, T,
                       1 if layout == "TS" else 0, 1 if rank_inputs else 0)
    L.kunExecutorClearStream(exec.handle)
    _check(rc)
    for o, d in zip(outs, dev_out):
        if _is_torch_cuda(o):
            o.copy_(d)
        else:
            o[...] = d.cpu().numpy()


def aggregrate(exec: Executor, inputs, labels, outs):
    """Per-stock reductions over runs of equal consecutive labels
    (``cpp/Python/PyBinding.cpp:449-506``; the reference's spelling): for
    input k ([T][S]) and labels k ([T]), ``outs[k]`` maps any of sum, min, max,
    first, last, count, mean to a [groups][S] array it fills."""
    import torch
    if len(inputs) != len(labels) or len(inputs) != len(outs):
        raise KunError("number of inputs, labels and outputs should match")
    if not inputs:
        return
    L = runtime()
    if not getattr(L, "_util_sigs", False):
        vp, sz, i32 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int
        L.kunCorrWith.restype = i32
        L.kunCorrWith.argtypes = [vp, i32, ctypes.POINTER(vp), vp, ctypes.POINTER(vp), sz, sz, i32, i32]
        L.kunAggregrate.restype = i32
        L.kunAggregrate.argtypes = [vp, i32, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp), sz, sz, i32]
        L._util_sigs = True
    first, _ = _to_device(inputs[0])
    dt = first.dtype
    if dt not in (torch.float32, torch.float64):
        raise KunError("aggregrate takes float or double buffers")
    T, S = first.shape
    keep, pin, plab, pout, back = [], [], [], [], []
    for k, (a, lab, o) in enumerate(zip(inputs, labels, outs)):
        d, _ = _to_device(a)
        lb, _ = _to_device(lab)
        if tuple(d.shape) != (T, S) or d.dtype != dt or lb.dtype != dt or tuple(lb.shape) != (T,):
            raise KunError(f"Bad shape at buffer_{k}")
        d, lb = d.contiguous(), lb.contiguous()
        keep += [d, lb]
        pin.append(d.data_ptr())
        plab.append(lb.data_ptr())
        row = [None] * 7
        for name, arr in o.items():
            if name not in _AGG_KINDS:
                raise KunError("Unknown aggregration kind: " + name)
            dev = arr if _is_torch_cuda(arr) else torch.empty(tuple(arr.shape), dtype=dt, device=d.device)
            if dev.shape[1] != S:
                raise KunError(f"Bad shape at output_{name}{_AGG_KINDS.index(name)}")
            keep.append(dev)
            row[_AGG_KINDS.index(name)] = dev.data_ptr()
            if not _is_torch_cuda(arr):
                back.append((arr, dev))
        pout += row
    vp = ctypes.c_void_p
    L.kunExecutorSetStream(exec.handle, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    rc = L.kunAggregrate(exec.handle, len(pin), (vp * len(pin))(*pin), (vp * len(plab))(*plab),
                         (vp * len(pout))(*pout), S, T, 0 if dt == torch.float32 else 1)
    L.kunExecutorClearStream(exec.handle)
    _check(rc)
    for arr, dev in back:
        arr[...] = dev.cpu().numpy()
