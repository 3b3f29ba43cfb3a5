"""Serving pool: sessions of different sizes batched into one step per tick.

Every session's outputs must equal (bit for bit) the same session run alone
through its own StreamContext, whether it is stepped alone or in a mix with
sessions that join late, leave early, or reuse the columns of closed ones."""
import threading

import numpy as np
import pytest

from kunquant_gb300 import runner as kr
from kunquant_gb300 import serve
from tests import golden_util as G
from tests.parity import compare_exact


def _module(name):
    if name == "alpha101_stream":
        return kr.Library.predefined("alpha101_stream_f32").getModule(name)
    from kunquant_gb300 import build
    spec = G.load(name)[0]
    return kr.Library.load(build.build_module_library([spec], "kun_serve_" + name)).getModule(spec["name"])


def _data(mod, S, T, seed):
    rng = np.random.default_rng(seed)
    out = {}
    for k in mod.getInputNames():
        x = (rng.random((T, S)) * 10 + 1).astype(mod.dtype)
        x[rng.random((T, S)) < 0.01] = np.nan
        out[k] = x
    return out


def _alone(ex, mod, data):
    T, S = next(iter(data.values())).shape
    ctx = kr.StreamContext(ex, mod, S)
    hin = {k: ctx.queryBufferHandle(k) for k in data}
    hout = {k: ctx.queryBufferHandle(k) for k in mod.getOutputNames()}
    out = {k: np.empty((T, S), mod.dtype) for k in hout}
    for t in range(T):
        for k, h in hin.items():
            ctx.pushData(h, np.ascontiguousarray(data[k][t]))
        ctx.run()
        for k, h in hout.items():
            out[k][t] = ctx.getCurrentBuffer(h)
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["stream_misc_f32", "alpha101_stream"])
def test_pool_mix_equals_alone(name):
    mod = _module(name)
    ex = kr.createSingleThreadExecutor()
    T = 60
    sizes = [24, 7, 61, 130, 3]
    data = [_data(mod, S, T, seed=100 + i) for i, S in enumerate(sizes)]
    want = [_alone(ex, mod, d) for d in data]
    # sessions 0-2 from tick 0; session 3 joins at tick 10; session 1 leaves
    # at tick 30 and session 4 takes its columns
    pool = serve.ServePool(ex, mod, capacity_stocks=300, max_sessions=8, max_session_stocks=256, start=False)
    got = [{k: np.full((T, S), np.nan, mod.dtype) for k in mod.getOutputNames()} for S in sizes]
    live = {i: pool.try_open(sizes[i]) for i in (0, 1, 2)}
    clock = {i: 0 for i in live}
    for step in range(T + 40):
        if step == 10:
            live[3] = pool.try_open(sizes[3]); clock[3] = 0
        if step == 30:
            pool.close(live.pop(1))
            live[4] = pool.try_open(sizes[4]); clock[4] = 0
            assert live[4] is not None
        active = [i for i in live if clock[i] < T]
        if not active:
            break
        for i in active:
            for k in mod.getInputNames():
                live[i].inputs[k][:] = data[i][k][clock[i]]
        pool.step([live[i] for i in active])
        for i in active:
            for k in mod.getOutputNames():
                got[i][k][clock[i]] = live[i].outputs[k]
            clock[i] += 1
    for i in (0, 2, 3, 4):
        assert clock[i] == T
        assert not compare_exact(got[i], want[i]), f"session {i} differs from its StreamContext run"
    # session 1 ran 30 ticks before it left
    head = {k: v[:30] for k, v in got[1].items()}
    assert not compare_exact(head, {k: v[:30] for k, v in want[1].items()})
    pool.shutdown()


@pytest.mark.gpu
def test_pool_rank_size_classes():
    """Sessions on both sides of the small-segment Rank threshold (1024
    stocks: 128-thread blocks below, 1024-thread blocks with the radix sort
    above) in one step, each equal to its StreamContext run alone."""
    mod = _module("alpha101_stream")
    ex = kr.createSingleThreadExecutor()
    T = 40
    sizes = [1024, 1025, 40, 3000, 700]
    data = [_data(mod, S, T, seed=300 + i) for i, S in enumerate(sizes)]
    want = [_alone(ex, mod, d) for d in data]
    pool = serve.ServePool(ex, mod, capacity_stocks=sum(sizes), max_sessions=8, max_session_stocks=3000,
                           start=False)
    sess = [pool.try_open(S) for S in sizes]
    got = [{k: np.empty((T, S), mod.dtype) for k in mod.getOutputNames()} for S in sizes]
    for t in range(T):
        for i, se in enumerate(sess):
            for k in mod.getInputNames():
                se.inputs[k][:] = data[i][k][t]
        pool.step(sess[::-1])
        for i, se in enumerate(sess):
            for k in mod.getOutputNames():
                got[i][k][t] = se.outputs[k]
    for i in range(len(sizes)):
        assert not compare_exact(got[i], want[i]), f"session of {sizes[i]} stocks differs from its StreamContext run"
    pool.shutdown()


@pytest.mark.gpu
def test_pool_request_loop_threads():
    """Ticks submitted from several client threads through the request loop
    give the same outputs as the sessions run alone."""
    mod = _module("stream_misc_f32")
    ex = kr.createSingleThreadExecutor()
    T, sizes = 40, [16, 33, 5, 64]
    data = [_data(mod, S, T, seed=7 + i) for i, S in enumerate(sizes)]
    want = [_alone(ex, mod, d) for d in data]
    pool = serve.ServePool(ex, mod, capacity_stocks=200, max_sessions=8, max_session_stocks=128)
    sessions = [pool.open(S) for S in sizes]
    got = [{k: np.empty((T, S), mod.dtype) for k in mod.getOutputNames()} for S in sizes]
    errors = []

    def client(i):
        try:
            s = sessions[i]
            for t in range(T):
                out = s.tick({k: data[i][k][t] for k in mod.getInputNames()}, timeout_ms=20000)
                for k, v in out.items():
                    got[i][k][t] = v
        except Exception as e:  # surfaced below
            errors.append(e)

    th = [threading.Thread(target=client, args=(i,)) for i in range(len(sizes))]
    for t in th:
        t.start()
    for t in th:
        t.join(60)
    assert not errors, errors
    for i in range(len(sizes)):
        assert not compare_exact(got[i], want[i]), f"session {i}"
    lat, steps = pool.take_latencies()
    assert len(lat) == T * len(sizes)
    assert steps.sum() == T * len(sizes)
    pool.shutdown()


@pytest.mark.gpu
def test_pool_admission_by_columns():
    mod = _module("stream_misc_f32")
    ex = kr.createSingleThreadExecutor()
    pool = serve.ServePool(ex, mod, capacity_stocks=100, max_sessions=4, max_session_stocks=100)
    a = pool.open(60)
    b = pool.open(40)
    assert pool.try_open(1) is None          # no columns left
    assert pool.free_stocks() == (0, 0)
    admitted = []

    def waiter():
        admitted.append(pool.open(50, timeout=30))

    t = threading.Thread(target=waiter)
    t.start()
    pool.close(a)                            # frees 60 columns: the waiter gets in
    t.join(30)
    assert admitted and admitted[0].num_stocks == 50
    pool.close(b)
    pool.close(admitted[0])
    assert pool.free_stocks() == (100, 100)  # ranges merged back
    with pytest.raises(kr.KunError):
        pool.try_open(101)
    pool.shutdown()


@pytest.mark.gpu
def test_pool_budget_sizing():
    mod = _module("alpha101_stream")
    per = serve.pool_bytes(mod, 1)
    assert per > 1000
    ex = kr.createSingleThreadExecutor()
    pool = serve.ServePool(ex, mod, hbm_budget_bytes=per * 500, max_sessions=4, max_session_stocks=500,
                           start=False)
    assert pool.capacity == 500
    pool.shutdown()
