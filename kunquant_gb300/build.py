"""Builds the native parts in-tree (``kunquant_gb300/_build``) for sm_103a:

* ``libkungpu.so`` -- the runtime behind ``include/kun_gpu.h``;
* module libraries -- generated from module specs by ``codegen.py``.

Compilation is content-addressed: a library is rebuilt only when its sources
or the compiler flags change.  Translation units are compiled in parallel.
"""
import hashlib
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from typing import Dict, Iterable, List

from . import codegen
from .graph import predefined_spec

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(REPO, "include")
BUILD = os.path.join(HERE, "_build")
ARCH = os.environ.get("KUN_CUDA_ARCH", "103a")

NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")
COMMON_FLAGS = ["-gencode", f"arch=compute_{ARCH},code=sm_{ARCH}", "-O3", "-lineinfo", "-std=c++17",
                "-Xcompiler", "-fPIC,-fvisibility=hidden", f"-I{CSRC}", f"-I{INCLUDE}"]
# the factor arithmetic must not be contracted except where the templates
# call kfma() explicitly (see contraction.py)
MODULE_FLAGS = COMMON_FLAGS + ["-fmad=false"]

# built by build_all() (the bench times the slide and plain forms beside the
# headline); the other forms (the fast-stat, compensated, fp64-sum and STs
# builds, alpha101_slide_f32) are built on first use by predefined_library()
PREDEFINED = ["alpha101_f32", "alpha158_f32", "alpha101_f64", "alpha158_f64", "alpha101_stream_f32",
              "alpha158_stream_f32", "alpha158_slide_f32", "alpha158_plain_f32"]


def _hash(paths: Iterable[str], extra: str) -> str:
    h = hashlib.sha256(extra.encode())
    for p in sorted(paths):
        with open(p, "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:20]


def _run(cmd: List[str]):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout[-6000:])
    return r.stdout


def _headers() -> List[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(INCLUDE, "kun_gpu.h"))
    return hs


def _stamp_ok(lib: str, digest: str) -> bool:
    st = lib + ".stamp"
    return os.path.exists(lib) and os.path.exists(st) and open(st).read().strip() == digest


def _write_stamp(lib: str, digest: str):
    with open(lib + ".stamp", "w") as f:
        f.write(digest)


def runtime_path() -> str:
    return os.path.join(BUILD, "libkungpu.so")


def build_runtime(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(CSRC, f) for f in ("kun_runtime.cu", "kun_stream.cu", "kun_serve.cu", "kun_batch.cu",
                                            "kun_util.cu", "kun_noalloc.cu")]
    srcs = [s for s in srcs if os.path.exists(s)]
    lib = runtime_path()
    digest = _hash(srcs + _headers(), " ".join(COMMON_FLAGS) + ARCH)
    if not force and _stamp_ok(lib, digest):
        return lib
    objs = []

    def cc(src):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        _run([NVCC] + COMMON_FLAGS + ["-c", src, "-o", obj])
        return obj

    with ThreadPoolExecutor(len(srcs)) as ex:
        objs = list(ex.map(cc, srcs))
    tmp = lib + ".tmp"
    _run([NVCC, "-shared", "-gencode", f"arch=compute_{ARCH},code=sm_{ARCH}"] + objs + ["-o", tmp, "-ldl"])
    os.replace(tmp, lib)
    _write_stamp(lib, digest)
    return lib


def build_module_library(specs: List[dict], libname: str, out_dir: str = None, force: bool = False,
                         jobs: int = None) -> str:
    """Generate and compile one library holding the given module specs."""
    out_dir = out_dir or os.path.join(BUILD, libname)
    os.makedirs(out_dir, exist_ok=True)
    srcs: List[str] = []
    for spec in specs:
        srcs += codegen.generate_module(spec, out_dir, tag=spec["name"])
    lib = os.path.join(out_dir, f"lib{libname}.so")
    digest = _hash(srcs + _headers(), " ".join(MODULE_FLAGS) + ARCH)
    if not force and _stamp_ok(lib, digest):
        return lib

    def cc(src):
        obj = src[:-3] + ".o"
        _run([NVCC] + MODULE_FLAGS + ["-c", src, "-o", obj])
        return obj

    jobs = jobs or max(1, min(len(srcs), os.cpu_count() or 4))
    with ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(cc, srcs))
    tmp = lib + ".tmp"
    _run([NVCC, "-shared", "-gencode", f"arch=compute_{ARCH},code=sm_{ARCH}"] + objs + ["-o", tmp])
    os.replace(tmp, lib)
    _write_stamp(lib, digest)
    return lib


def predefined_library(key: str, force: bool = False) -> str:
    return build_module_library([predefined_spec(key)], "kun_" + key, force=force)


def build_all(keys: List[str] = None, force: bool = False) -> Dict[str, str]:
    out = {"runtime": build_runtime(force)}
    keys = keys or PREDEFINED
    for k in keys:
        out[k] = predefined_library(k, force)
    return out
