"""Compile front door with the reference's signature
(``KunQuant/jit/cfake.py:174``):

    lib = cfake.compileit([("alpha101", f, cfake.KunCompilerConfig(...))],
                          "mylib", cfake.CppCompilerConfig())
    mod = lib.getModule("alpha101")

The functions go through KunQuant's own front end and passes
(``graph.export_function``, which runs ``KunQuant/Driver.py:91-245``), then the
CUDA code generator, and are compiled for sm_103a into one shared library
that ``runner.Library`` loads.  A reference script needs only its imports
changed: ``from kunquant_gb300 import cfake`` and
``from kunquant_gb300 import runner as kr``.

``CppCompilerConfig`` and the CPU flag classes are accepted for source
compatibility; their CPU settings (``machine``, ``opt_level`` ...) do not
apply to a GPU build.  ``GpuCompilerConfig`` is the GPU form: the target arch
and the number of parallel compile jobs.
"""
import dataclasses
import os
import shutil
import tempfile
from dataclasses import dataclass, field
from typing import List, Optional, Tuple, Union

from . import build as _build
from . import graph as _graph
from . import runner as _runner

try:  # the reference front end's config, when the front end is importable
    from KunQuant.Driver import KunCompilerConfig  # noqa: F401
except ImportError:  # same fields (KunQuant/Driver.py:15-23)
    @dataclass
    class KunCompilerConfig:
        partition_factor: int = 3
        dtype: str = "float"
        blocking_len: int = None
        input_layout: str = "STs"
        output_layout: str = "STs"
        allow_unaligned: Union[bool, None] = None
        split_source: int = 0
        options: dict = field(default_factory=dict)


@dataclass
class X64CPUFlags:
    """Accepted for source compatibility; a GPU build has no CPU flags."""
    avx512: bool = False
    avx512dq: bool = False
    avx512vl: bool = False


@dataclass
class NativeCPUFlags:
    """Accepted for source compatibility; a GPU build has no CPU flags."""


@dataclass
class GpuCompilerConfig:
    """Target of the generated CUDA: `arch` as in sm_<arch> (only "103a" is
    supported) and the number of translation units compiled at once."""
    arch: str = "103a"
    jobs: Optional[int] = None


@dataclass
class CppCompilerConfig:
    """The reference's compiler config, accepted in place of a
    GpuCompilerConfig; only `other_flags` has no CPU-only meaning and it is
    ignored too (the GPU flags are fixed by the code generator)."""
    opt_level: int = 3
    machine: object = field(default_factory=NativeCPUFlags)
    for_each: object = None
    other_flags: Tuple[str, ...] = ()
    fast_linker_threads: int = 0


def _config_kwargs(cfg) -> dict:
    if dataclasses.is_dataclass(cfg):
        d = dataclasses.asdict(cfg)
    else:
        d = dict(vars(cfg))
    keys = ("partition_factor", "dtype", "blocking_len", "input_layout", "output_layout", "allow_unaligned",
            "split_source", "options")
    return {k: d[k] for k in keys if k in d}


def compileit(func: List[Tuple[str, object, object]], libname: str, compiler_config=None,
              tempdir: str = None, keep_files: bool = False, load: bool = True) -> Union["_runner.Library", str]:
    """Compile `(module name, Function, KunCompilerConfig)` triples into one
    library named `libname`.  Returns the loaded ``runner.Library`` (``load``)
    or the library's path.  Same arguments and rules as the reference: with
    ``keep_files`` the generated sources stay in ``tempdir/libname`` (and
    ``tempdir`` is required); otherwise they go to a temporary folder that
    is removed once the library is loaded."""
    if keep_files and not tempdir:
        raise RuntimeError("if keep_files=True, tempdir should not be empty")
    gpu = compiler_config if isinstance(compiler_config, GpuCompilerConfig) else GpuCompilerConfig()
    if gpu.arch != _build.ARCH:
        raise RuntimeError(f"this build targets sm_{_build.ARCH}, not sm_{gpu.arch}")
    specs = []
    for name, f, cfg in func:
        specs.append(_graph.export_function(f, name, **_config_kwargs(cfg)))
    if keep_files:
        out_dir = os.path.join(tempdir, libname)
        os.makedirs(out_dir, exist_ok=True)
    else:
        out_dir = tempfile.mkdtemp(dir=tempdir)
    try:
        path = _build.build_module_library(specs, libname, out_dir=out_dir, jobs=gpu.jobs)
        if not load:
            if keep_files:
                return path
            # the caller gets a library file that outlives the sources
            final = os.path.join(tempfile.mkdtemp(dir=tempdir), os.path.basename(path))
            shutil.copy2(path, final)
            return final
        return _runner.Library.load(path)
    finally:
        if not keep_files:
            shutil.rmtree(out_dir, ignore_errors=True)
