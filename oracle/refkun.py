"""Run the reference KunQuant CPU executor (built by ``oracle/build_ref.py``)
on the predefined graphs -- TEST INFRASTRUCTURE, this container only.

Used to pin the oracle restatement and to generate the golden fixtures under
``tests/golden``.  Needs the reference sources (``$KUN_REFERENCE_ROOT``,
default the ``reference`` folder beside this repository); it is never imported on the product path and
never on the GPU machine.
"""
import dataclasses
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
JIT_DIR = os.path.join(HERE, "_ref", "jit")

_libs = {}


def available():
    from oracle import build_ref
    return build_ref.available()


def _setup():
    from oracle import build_ref
    build_ref.import_reference()
    if REPO not in sys.path:
        sys.path.insert(0, REPO)


def compile_predefined(key: str):
    """Compile one entry of ``export_predefined.CONFIGS`` with the reference JIT
    (cached under ``oracle/_ref/jit``) and return the loaded module."""
    _setup()
    if key in _libs:
        return _libs[key]
    from KunQuant.jit import cfake
    from KunQuant.Driver import KunCompilerConfig
    from KunQuant.runner import KunRunner as kr
    from kunquant_gb300.graphs.export_predefined import CONFIGS
    builder, modname, kw = CONFIGS[key]
    os.makedirs(JIT_DIR, exist_ok=True)
    libpath = os.path.join(JIT_DIR, key, key + ".so")
    if os.path.exists(libpath):
        lib = kr.Library.load(libpath)
    else:
        cfg = KunCompilerConfig(**{k: (dict(v) if isinstance(v, dict) else v) for k, v in kw.items()})
        lib = cfake.compileit([(modname, builder(), cfg)], key,
                              cfake.CppCompilerConfig(machine=cfake.X64CPUFlags()),
                              tempdir=JIT_DIR, keep_files=True, load=True)
    mod = lib.getModule(modname)
    _libs[key] = (lib, mod)
    return _libs[key]


def run_batch(key: str, inputs: dict, cur_time=0, length=None, threads=1):
    """runGraph of the reference on [T][S] inputs; returns {name: [length][S]}."""
    lib, mod = compile_predefined(key)
    from KunQuant.runner import KunRunner as kr
    a0 = next(iter(inputs.values()))
    T = a0.shape[1] if a0.ndim == 3 else a0.shape[0]  # [S/L][T][L] or [T][S]
    if length is None:
        length = T - cur_time
    ex = kr.createSingleThreadExecutor() if threads == 1 else kr.createMultiThreadExecutor(threads)
    out = kr.runGraph(ex, mod, {k: np.ascontiguousarray(v) for k, v in inputs.items()},
                      cur_time, length)
    return {k: np.asarray(v) for k, v in out.items()}


def run_stream(key: str, inputs: dict, num_ticks=None):
    """Drive the reference StreamContext tick by tick; returns {name: [T][S]}."""
    lib, mod = compile_predefined(key)
    return run_stream_module(mod, inputs, num_ticks)


def run_stream_module(mod, inputs: dict, num_ticks=None):
    """run_stream for a module compiled by compile_function."""
    from KunQuant.runner import KunRunner as kr
    T, S = next(iter(inputs.values())).shape
    num_ticks = num_ticks or T
    ex = kr.createSingleThreadExecutor()
    ctx = kr.StreamContext(ex, mod, S)
    hin = {k: ctx.queryBufferHandle(k) for k in inputs}
    names = mod.getOutputNames()
    hout = {k: ctx.queryBufferHandle(k) for k in names}
    res = {k: np.empty((num_ticks, S), dtype=next(iter(inputs.values())).dtype) for k in names}
    for t in range(num_ticks):
        for k, h in hin.items():
            ctx.pushData(h, np.ascontiguousarray(inputs[k][t]))
        ctx.run()
        for k, h in hout.items():
            res[k][t] = ctx.getCurrentBuffer(h)
    return res


def compile_function(key: str, build, modname: str, **cfg_kw):
    """Compile an arbitrary front-end graph (``build()`` returns a Function)
    with the reference JIT; returns (spec, module).  The spec is exported from
    a second, identical build so both sides see the same pass pipeline."""
    _setup()
    from KunQuant.jit import cfake
    from KunQuant.Driver import KunCompilerConfig
    from KunQuant.runner import KunRunner as kr
    from kunquant_gb300.graph import export_function
    import copy
    spec = export_function(build(), modname, **copy.deepcopy(cfg_kw))
    if key not in _libs:
        os.makedirs(JIT_DIR, exist_ok=True)
        libpath = os.path.join(JIT_DIR, key, key + ".so")
        if os.path.exists(libpath):
            lib = kr.Library.load(libpath)
        else:
            cfg = KunCompilerConfig(**copy.deepcopy(cfg_kw))
            lib = cfake.compileit([(modname, build(), cfg)], key,
                                  cfake.CppCompilerConfig(machine=cfake.X64CPUFlags()),
                                  tempdir=JIT_DIR, keep_files=True, load=True)
        _libs[key] = (lib, lib.getModule(modname))
    return spec, _libs[key][1]


def run_module(mod, inputs: dict, cur_time=0, length=None, threads=1):
    from KunQuant.runner import KunRunner as kr
    a0 = next(iter(inputs.values()))
    T = a0.shape[1] if a0.ndim == 3 else a0.shape[0]  # [S/L][T][L] or [T][S]
    if length is None:
        length = T - cur_time
    ex = kr.createSingleThreadExecutor() if threads == 1 else kr.createMultiThreadExecutor(threads)
    out = kr.runGraph(ex, mod, {k: np.ascontiguousarray(v) for k, v in inputs.items()},
                      cur_time, length)
    return {k: np.asarray(v) for k, v in out.items()}
