"""Restoring a stream from a KUNGPUS1 dump checks every value a kernel would
use as an index or a loop bound before any device work: a forged dump is
refused with the reference's error text (cpp/Kun/Runtime.cpp:418,456).  These
run without a GPU: the dump is parsed before the executor is looked at, so a
NULL executor reaches the parser and nothing is launched."""
import ctypes
import struct

import numpy as np

from kunquant_gb300 import runner as kr


class _Stage(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char_p), ("kind", ctypes.c_int32), ("num_in", ctypes.c_int32),
                ("in_bufs", ctypes.c_void_p), ("num_out", ctypes.c_int32), ("out_bufs", ctypes.c_void_p),
                ("num_deps", ctypes.c_int32), ("deps", ctypes.c_void_p), ("pending", ctypes.c_int32),
                ("num_scratch", ctypes.c_int32), ("state_bytes_per_stock", ctypes.c_int64),
                ("launch", ctypes.c_void_p), ("num_kernels", ctypes.c_int32),
                ("state_t_vars", ctypes.c_int32), ("state_i_vars", ctypes.c_int32), ("init", ctypes.c_void_p),
                ("state_i_max", ctypes.POINTER(ctypes.c_int32)), ("kernel_info", ctypes.c_void_p),
                ("prepare", ctypes.c_void_p), ("launch_group", ctypes.c_void_p)]


class _Module(ctypes.Structure):
    _fields_ = [("abi", ctypes.c_uint64), ("name", ctypes.c_char_p), ("num_stages", ctypes.c_int32),
                ("stages", ctypes.POINTER(_Stage)), ("num_buffers", ctypes.c_int32), ("buffers", ctypes.c_void_p),
                ("input_layout", ctypes.c_int32), ("output_layout", ctypes.c_int32),
                ("blocking_len", ctypes.c_int32), ("dtype", ctypes.c_int32), ("aligned", ctypes.c_int32)]


class _Extra(ctypes.Structure):
    _fields_ = [("version", ctypes.c_size_t), ("init_kind", ctypes.c_int), ("buffer", ctypes.c_char_p),
                ("size", ctypes.c_size_t)]


def _module():
    mod = kr.Library.predefined("alpha158_stream_f32").getModule("alpha158_stream")
    return mod, ctypes.cast(mod.handle, ctypes.POINTER(_Module)).contents


def _dump(mod, desc, S, tick=0, int_value=None):
    """A well-formed dump of a fresh stream (NaN rings, zero states) for S
    stocks; `int_value` overwrites every bounded int32 state."""
    out = [b"KUNGPUS1", struct.pack("<IIqqII", 1, desc.dtype, S, tick, desc.num_buffers, desc.num_stages),
           desc.name.ljust(64, b"\0")]
    for b in mod.buffers:
        w = b["window"]
        out.append(struct.pack("<ii", w, w - 1))
        out.append(np.full((w, S), np.nan, np.float32).tobytes())
    for s in range(desc.num_stages):
        st = desc.stages[s]
        out.append(struct.pack("<ii", st.state_t_vars, st.state_i_vars))
        out.append(np.zeros((st.state_t_vars, S), np.float32).tobytes())
        ints = np.zeros((st.state_i_vars, S), np.int32)
        if int_value is not None:
            for v in range(st.state_i_vars):
                if st.state_i_max[v] >= 0:
                    ints[v] = int_value
        out.append(ints.tobytes())
    return b"".join(out)


def _restore(mod, blob, S):
    L = kr.runtime()
    fn = L.kunCreateStreamEx
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(_Extra),
                   ctypes.POINTER(ctypes.c_void_p)]
    extra = _Extra(1, 2, blob, len(blob))  # KUN_API_VERSION, KUN_INIT_MEMORY
    out = ctypes.c_void_p()
    rc = fn(None, mod.handle, S, ctypes.byref(extra), ctypes.byref(out))
    return rc, L.kunGetLastError().decode(), out.value


def test_module_declares_state_bounds():
    mod, desc = _module()
    bounded = 0
    for s in range(desc.num_stages):
        st = desc.stages[s]
        if st.state_i_vars:
            mx = [st.state_i_max[v] for v in range(st.state_i_vars)]
            assert all(m >= -1 for m in mx)
            bounded += sum(m >= 0 for m in mx)
    assert bounded > 0


def test_well_formed_dump_passes_the_parser():
    mod, desc = _module()
    rc, msg, h = _restore(mod, _dump(mod, desc, 8), 8)
    # parsed and accepted; it stops only at the missing executor
    assert h is None and "null executor" in msg, (rc, msg)


def test_out_of_range_state_is_refused():
    mod, desc = _module()
    big = max(b["window"] for b in mod.buffers) + 1000
    for value in (big, -1):
        rc, msg, h = _restore(mod, _dump(mod, desc, 8, int_value=value), 8)
        assert h is None and msg == "Failed to deserialize state buffer", (value, rc, msg)


def test_negative_tick_is_refused():
    mod, desc = _module()
    rc, msg, h = _restore(mod, _dump(mod, desc, 8, tick=-5), 8)
    assert h is None and msg == "Failed to read initial stream buffer", (rc, msg)


def test_truncated_dump_is_refused():
    mod, desc = _module()
    blob = _dump(mod, desc, 8)
    rc, msg, h = _restore(mod, blob[:len(blob) - 3], 8)
    assert h is None and msg == "Failed to deserialize state buffer", (rc, msg)
    rc, msg, h = _restore(mod, blob[:40], 8)
    assert h is None and msg == "Failed to read initial stream buffer", (rc, msg)
