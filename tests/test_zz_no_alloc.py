"""kunRunGraphNoAlloc: the batch run whose temporaries and scratch live in a
static device array of libkungpu.so.  Its outputs must equal kunRunGraphEx's
bit for bit, on two calls in a row; oversize runs are refused with a clear
message.  The file is named so that pytest collects it last: it must pass
alone and after every other test."""
import ctypes
import os
import re

import numpy as np
import pytest

from kunquant_gb300 import runner as kr
from kunquant_gb300 import synth
from tests.parity import compare_exact

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SCRATCH_BYTES = 64 << 20


def _no_alloc_fn():
    L = kr.runtime()
    fn = L.kunRunGraphNoAlloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_size_t] * 4 + [ctypes.c_void_p]
    return L, fn


def test_no_alloc_source_allocates_nothing():
    src = open(os.path.join(REPO, "kunquant_gb300", "csrc", "kun_noalloc.cu")).read()
    code = re.sub(r"//[^\n]*", "", re.sub(r"/\*.*?\*/", "", src, flags=re.S))
    # no device allocation of any kind (cudaMalloc* covers the async, host,
    # managed and pool forms)
    for call in ("cudaMalloc", "cudaFree", "cuMemAlloc", "cuMemFree", "cuMemCreate", "cudaHostAlloc",
                 "torch", "cublas"):
        assert call not in code, call
    assert "static __device__ __align__(256)" in code
    assert "cudaGetSymbolAddress" in code


def _check_twice(key, module, S, T, cur_time, seed):
    """Two no-alloc calls in a row on fresh output buffers, each equal bit
    for bit to kunRunGraphEx; the second call changes no device memory."""
    import torch
    mod = kr.Library.predefined(key).getModule(module)
    data = synth.ohlcv(S, T, seed=seed, nan_frac=0.005)
    dev_in = {k: torch.from_numpy(v).cuda() for k, v in data.items() if k in mod.getInputNames()}
    L, run_no_alloc = _no_alloc_fn()
    length = T - cur_time

    # existing entry point, device buffers, own executor
    ex = kr.createSingleThreadExecutor()
    want = kr.runGraph(ex, mod, dev_in, cur_time, length)
    torch.cuda.synchronize()
    want = {k: v.cpu().numpy() for k, v in want.items()}

    stream = torch.cuda.current_stream()
    for call in range(2):
        outs = {k: torch.full((length, S), float("nan"), device="cuda") for k in mod.getOutputNames()}
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        m = L.kunCreateBufferNameMap()
        try:
            for k, v in list(dev_in.items()) + list(outs.items()):
                L.kunSetBufferNameMap(m, k.encode(), ctypes.c_void_p(v.data_ptr()))
            rc = run_no_alloc(mod.handle, m, S, T, cur_time, length, ctypes.c_void_p(stream.cuda_stream))
        finally:
            L.kunDestoryBufferNameMap(m)
        assert rc == 0, L.kunGetLastError().decode()
        stream.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        if call == 1:
            # the first call may load the module's kernels; the second finds
            # everything in place and takes no device memory
            assert free_after == free_before, (free_before, free_after)
        got = {k: v.cpu().numpy() for k, v in outs.items()}
        bad = compare_exact(got, want)
        assert not bad, f"{key} call {call}: differs from kunRunGraphEx: {bad}"


@pytest.mark.gpu
def test_no_alloc_matches_run_graph_twice():
    _check_twice("alpha158_f32", "alpha158", 128, 200, 0, seed=7)


@pytest.mark.gpu
def test_no_alloc_alpha101_rank_and_scratch_with_offset():
    # Alpha101: cross-sectional Rank/Scale stages, per-stage scratch slots and
    # a run that starts at cur_time > 0
    _check_twice("alpha101_f32", "alpha101", 96, 260, 50, seed=8)


@pytest.mark.gpu
def test_no_alloc_rejects_oversize_runs():
    import torch
    mod = kr.Library.predefined("alpha158_f32").getModule("alpha158")
    L, run_no_alloc = _no_alloc_fn()
    m = L.kunCreateBufferNameMap()
    try:
        # 5000 stocks x 2500 days: one [T][S] slot alone is 50 MB
        rc = run_no_alloc(mod.handle, m, 5000, 2500, 0, 2500,
                          ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    finally:
        L.kunDestoryBufferNameMap(m)
    assert rc == 4  # KUN_OUT_OF_MEMORY
    msg = L.kunGetLastError().decode()
    assert f"the static scratch holds {SCRATCH_BYTES} bytes" in msg, msg
