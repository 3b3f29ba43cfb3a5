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
