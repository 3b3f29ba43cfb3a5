"""Serving pool: many stream sessions of one stream module on one GPU.

The reference serves each stream with its own ``StreamContext``
(``cpp/Python/PyBinding.cpp:508-596``).  Here sessions of different universe
sizes share one device store (``kun_serve.cu``): each keeps its window and
order-statistic state resident in a column range of the pool; a request loop
in the runtime batches every tick submitted before a step into one graph
launch (continuous batching).  Admission is by device memory: a pool is sized
by an HBM budget, and ``open`` waits until a session slot and a free column
range of the requested size exist.

    pool = ServePool(ex, mod, hbm_budget_bytes=4 << 30, max_sessions=256)
    s = pool.open(1200)                    # admitted (or waits for room)
    s.inputs["close"][:] = row             # pinned host views, one per input
    out = s.tick()                         # {name: view of the output row}
    pool.close(s)
"""
import ctypes
import threading
import weakref
from typing import Dict, List, Optional

import numpy as np

from . import runner

KUN_OUT_OF_MEMORY = 4
KUN_TIMEOUT = 5


def _lib():
    L = runner.runtime()
    if not getattr(L, "_serve_sigs", False):
        vp, sz, i32, i64 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_int64
        p64 = ctypes.POINTER(ctypes.c_int64)
        sig = {
            "kunCreateServePool": (i32, [vp, vp, sz, i32, i32, ctypes.POINTER(vp)]),
            "kunDestroyServePool": (None, [vp]),
            "kunServeOpen": (i32, [vp, sz, p64]),
            "kunServeClose": (i32, [vp, i64]),
            "kunServeStep": (i32, [vp, i32, p64, vp, vp]),
            "kunServeStart": (i32, [vp, i32]),
            "kunServeStop": (i32, [vp]),
            "kunServeSubmit": (i32, [vp, i32, p64]),
            "kunServeWait": (i32, [vp, i64, i64, i32]),
            "kunServeTakeLatencies": (i32, [vp, ctypes.POINTER(ctypes.c_float), i32,
                                            ctypes.POINTER(ctypes.c_int32), i32, ctypes.POINTER(ctypes.c_int)]),
            "kunServeHostInputs": (vp, [vp]),
            "kunServeHostOutputs": (vp, [vp]),
            "kunServeSessionTick": (i64, [vp, i64]),
            "kunServeSessionStocks": (i64, [vp, i64]),
            "kunServeSessionColumn": (i64, [vp, i64]),
            "kunServeFreeStocks": (i32, [vp, p64, p64]),
            "kunServePoolBytes": (i64, [vp, sz]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        L._serve_sigs = True
    return L


def pool_bytes(mod: runner.Module, capacity_stocks: int) -> int:
    """Device bytes of a pool of ``capacity_stocks`` columns."""
    return int(_lib().kunServePoolBytes(mod.handle, capacity_stocks))


class Session:
    """One stream session of a pool: ``inputs``/``outputs`` are views of its
    columns in the pool's pinned host tables, one 1-D array per buffer."""

    def __init__(self, pool: "ServePool", sid: int, num_stocks: int, column: int):
        self.pool, self.id, self.num_stocks, self.column = pool, sid, num_stocks, column
        sl = slice(column, column + num_stocks)
        self.inputs = {n: pool._in_table[i, sl] for i, n in enumerate(pool.input_names)}
        self.outputs = {n: pool._out_table[i, sl] for i, n in enumerate(pool.output_names)}
        self._submitted = 0

    @property
    def ticks(self) -> int:
        return int(_lib().kunServeSessionTick(self.pool.handle, self.id))

    def submit(self, rows: Optional[Dict[str, np.ndarray]] = None):
        """Write ``rows`` (name -> row of num_stocks values; omit to use what
        was written into ``inputs``) and queue the tick."""
        if rows:
            for k, v in rows.items():
                self.inputs[k][:] = v
        done = self.ticks
        arr = (ctypes.c_int64 * 1)(self.id)
        runner._check(_lib().kunServeSubmit(self.pool.handle, 1, arr))
        self._submitted = done + 1

    def wait(self, timeout_ms: int = -1) -> Dict[str, np.ndarray]:
        """Wait for the submitted tick; returns the output views (valid until
        this session's next tick)."""
        rc = _lib().kunServeWait(self.pool.handle, self.id, self._submitted, timeout_ms)
        runner._check(rc)
        return self.outputs

    def tick(self, rows: Optional[Dict[str, np.ndarray]] = None, timeout_ms: int = -1):
        self.submit(rows)
        return self.wait(timeout_ms)


class ServePool:
    """A serving pool over one stream module (see the module docstring).

    Size it with ``capacity_stocks`` or with ``hbm_budget_bytes`` (the pool's
    device footprint, from ``pool_bytes``).  ``batch_window_us`` delays each
    step to let more ticks join it."""

    def __init__(self, exec: runner.Executor, mod: runner.Module, capacity_stocks: Optional[int] = None,
                 hbm_budget_bytes: Optional[int] = None, max_sessions: int = 256,
                 max_session_stocks: int = 8192, batch_window_us: int = 0, start: bool = True):
        if mod.output_layout != "STREAM":
            raise runner.KunError("Cannot run batch mode module via StreamContext")
        L = _lib()
        if capacity_stocks is None:
            if hbm_budget_bytes is None:
                raise runner.KunError("give capacity_stocks or hbm_budget_bytes")
            per = pool_bytes(mod, 1)
            capacity_stocks = int(hbm_budget_bytes // per)
        self.capacity = int(capacity_stocks)
        self.mod, self._exec = mod, exec
        self.input_names = mod.getInputNames()
        self.output_names = mod.getOutputNames()
        h = ctypes.c_void_p()
        runner._check(L.kunCreateServePool(exec.handle, mod.handle, self.capacity, max_sessions,
                                           max_session_stocks, ctypes.byref(h)))
        self.handle = h.value
        ct = ctypes.c_float if mod.dtype == np.float32 else ctypes.c_double
        nin, nout = len(self.input_names), len(self.output_names)
        self._in_table = np.ctypeslib.as_array(ctypes.cast(L.kunServeHostInputs(self.handle), ctypes.POINTER(ct)),
                                               shape=(max(1, nin), self.capacity))
        self._out_table = np.ctypeslib.as_array(
            ctypes.cast(L.kunServeHostOutputs(self.handle), ctypes.POINTER(ct)), shape=(max(1, nout), self.capacity))
        self._room = threading.Condition()
        # sessions hold their pool; the pool only tracks them weakly
        self.sessions = weakref.WeakValueDictionary()
        self.running = False
        if start:
            self.start(batch_window_us)

    def start(self, batch_window_us: int = 0):
        runner._check(_lib().kunServeStart(self.handle, batch_window_us))
        self.running = True

    def stop(self):
        if self.handle and self.running:
            _lib().kunServeStop(self.handle)
            self.running = False

    def shutdown(self):
        """Stop the loop and free the pool's device and pinned memory; the
        sessions' views must not be used afterwards."""
        if getattr(self, "handle", None) and runner._lib is not None:
            self.stop()
            runner._lib.kunDestroyServePool(self.handle)
            self.handle = None

    def __del__(self):
        self.shutdown()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.shutdown()

    def try_open(self, num_stocks: int) -> Optional[Session]:
        """Admit a session now, or None when no slot or column range fits."""
        L = _lib()
        sid = ctypes.c_int64()
        rc = L.kunServeOpen(self.handle, num_stocks, ctypes.byref(sid))
        if rc == KUN_OUT_OF_MEMORY:
            return None
        runner._check(rc)
        s = Session(self, sid.value, num_stocks, int(L.kunServeSessionColumn(self.handle, sid.value)))
        self.sessions[s.id] = s
        return s

    def open(self, num_stocks: int, timeout: Optional[float] = None) -> Session:
        """Admit a session, waiting for a close to free room if needed."""
        with self._room:
            s = self.try_open(num_stocks)
            while s is None:
                if not self._room.wait(timeout):
                    raise runner.KunError(f"no room for a session of {num_stocks} stocks")
                s = self.try_open(num_stocks)
            return s

    def close(self, s: Session):
        runner._check(_lib().kunServeClose(self.handle, s.id))
        self.sessions.pop(s.id, None)
        with self._room:
            self._room.notify_all()

    def free_stocks(self):
        t, l = ctypes.c_int64(), ctypes.c_int64()
        _lib().kunServeFreeStocks(self.handle, ctypes.byref(t), ctypes.byref(l))
        return t.value, l.value

    def submit_all(self, sessions: List[Session]):
        """Queue one tick of each session (inputs already written)."""
        for s in sessions:
            s._submitted = s.ticks + 1
        arr = (ctypes.c_int64 * len(sessions))(*[s.id for s in sessions])
        runner._check(_lib().kunServeSubmit(self.handle, len(sessions), arr))

    def step(self, sessions: List[Session], device_inputs=None, device_outputs=None):
        """Without the request loop: advance ``sessions`` by one tick now.
        ``device_inputs``/``device_outputs``: optional torch CUDA tables
        [num_inputs][capacity] / [num_outputs][capacity]."""
        arr = (ctypes.c_int64 * len(sessions))(*[s.id for s in sessions])
        din = ctypes.c_void_p(device_inputs.data_ptr()) if device_inputs is not None else None
        dout = ctypes.c_void_p(device_outputs.data_ptr()) if device_outputs is not None else None
        runner._check(_lib().kunServeStep(self.handle, len(sessions), arr, din, dout))

    def take_latencies(self, cap: int = 1 << 20):
        """(tick latencies in microseconds, sessions per step) recorded by the
        loop since the last call."""
        lat = (ctypes.c_float * cap)()
        steps = (ctypes.c_int32 * cap)()
        ns = ctypes.c_int()
        n = _lib().kunServeTakeLatencies(self.handle, lat, cap, steps, cap, ctypes.byref(ns))
        return np.frombuffer(lat, np.float32, n).copy(), np.frombuffer(steps, np.int32, ns.value).copy()
