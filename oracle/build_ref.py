"""Build recipe for ``oracle/_ref``: the reference KunQuant CPU runtime, compiled
from its own sources where they lie, used only as a checker.

This is test infrastructure.  It never runs on the product path: only the
fixture generator under ``tests/golden/`` and the CPU-side parity tests use it.

What it builds (all outputs go to ``oracle/_ref/`` and nothing else):

* ``oracle/_ref/py/KunQuant/runner/libKunRuntime.so`` -- the reference
  ``KunRuntime`` (``cpp/Kun/*.cpp`` + ``cpp/KunSIMD/cpu/tables.cpp``), compiled
  with the flags of the reference ``CMakeLists.txt:21-27`` (``-std=c++11``,
  ``-mavx2 -mfma`` on x86_64).
* ``oracle/_ref/py/KunQuant/runner/KunRunner<ext>`` -- the pybind11 binding
  ``cpp/Python/PyBinding.cpp`` (pybind11 from the local Python install, because
  the reference's ``3rdparty/pybind11`` submodule is empty).
* A two-file shadow package (``oracle/_ref/py/KunQuant/__init__.py`` and
  ``.../runner/__init__.py``) whose ``__path__`` chains to the reference's own
  ``KunQuant`` package, so ``import KunQuant.jit.cfake`` works unchanged and
  its JIT includes the reference headers and links the runtime built here.

The reference's own cmake build is not used: it needs the missing pybind11
submodule.  The recipe is ~20 s on 8 cores.  Usage::

    python oracle/build_ref.py            # build if missing
    python oracle/build_ref.py --force    # rebuild
"""
import os
import platform
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference checkout: $KUN_REFERENCE_ROOT, by default the "reference"
# folder beside this repository
REF_ROOT = os.environ.get("KUN_REFERENCE_ROOT",
                          os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))
OUT = os.path.join(HERE, "_ref")
PYROOT = os.path.join(OUT, "py")
RUNNER_DIR = os.path.join(PYROOT, "KunQuant", "runner")


def _arch_flags():
    m = platform.machine().lower()
    if m in ("x86_64", "amd64"):
        return ["-mavx2", "-mfma"]
    return []


def runner_ext():
    return sysconfig.get_config_var("EXT_SUFFIX")


def built():
    return (os.path.exists(os.path.join(RUNNER_DIR, "libKunRuntime.so"))
            and os.path.exists(os.path.join(RUNNER_DIR, "KunRunner" + runner_ext())))


def available():
    return os.path.isdir(os.path.join(REF_ROOT, "cpp", "Kun"))


def _shadow_package():
    os.makedirs(RUNNER_DIR, exist_ok=True)
    ref_pkg = os.path.join(REF_ROOT, "KunQuant")
    with open(os.path.join(PYROOT, "KunQuant", "__init__.py"), "w") as f:
        f.write("# generated by oracle/build_ref.py: chains to the reference package\n"
                f"__path__.append({ref_pkg!r})\n")
    with open(os.path.join(RUNNER_DIR, "__init__.py"), "w") as f:
        f.write("# generated by oracle/build_ref.py\n"
                "from . import KunRunner\n"
                "import os\n"
                "example_projects_path = os.path.dirname(__file__)\n")


def build(force=False):
    if not available():
        raise RuntimeError("reference sources not found at " + REF_ROOT)
    if built() and not force:
        _shadow_package()
        return
    _shadow_package()
    cpp = os.path.join(REF_ROOT, "cpp")
    objdir = os.path.join(OUT, "obj")
    os.makedirs(objdir, exist_ok=True)
    srcs = [os.path.join(cpp, "Kun", f) for f in sorted(os.listdir(os.path.join(cpp, "Kun")))
            if f.endswith(".cpp")]
    srcs.append(os.path.join(cpp, "KunSIMD", "cpu", "tables.cpp"))
    common = ["g++", "-O3", "-std=c++11", "-fPIC", "-fvisibility=hidden",
              "-fvisibility-inlines-hidden", "-pthread", "-I" + cpp] + _arch_flags()

    def cc(src):
        obj = os.path.join(objdir, os.path.basename(src) + ".o")
        subprocess.check_call(common + ["-DKUN_CORE_LIB=1", "-c", src, "-o", obj])
        return obj

    with ThreadPoolExecutor(os.cpu_count() or 4) as ex:
        objs = list(ex.map(cc, srcs))
    lib = os.path.join(RUNNER_DIR, "libKunRuntime.so")
    subprocess.check_call(["g++", "-shared", "-pthread"] + objs + ["-o", lib, "-ldl"])
    import pybind11
    binding = os.path.join(RUNNER_DIR, "KunRunner" + runner_ext())
    subprocess.check_call(
        ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fvisibility=hidden", "-pthread",
         "-I" + cpp, "-I" + pybind11.get_include(),
         "-I" + sysconfig.get_paths()["include"]] + _arch_flags() +
        [os.path.join(cpp, "Python", "PyBinding.cpp"), "-o", binding,
         "-L" + RUNNER_DIR, "-lKunRuntime", "-Wl,-rpath,$ORIGIN"])


def import_reference():
    """Put the reference front end + the runtime built here on ``sys.path``
    and return the ``KunQuant`` package."""
    build()
    if PYROOT not in sys.path:
        sys.path.insert(0, PYROOT)
    import KunQuant  # noqa: F401
    return KunQuant


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print("built", OUT)
