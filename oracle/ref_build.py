"""Recipe that builds the reference's own eSRRF/SRRF CPU path into ``oracle/_ref``.

TEST INFRASTRUCTURE ONLY.  Nothing in ``nanopyx_gb300`` imports this module;
only ``tests/``, ``__graft_entry__`` (build/smoke) and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` use what it produces, as the checker
and as the timed CPU baseline.

Two stages, so that the compiled reference can also be produced on a machine
that has no copy of the reference tree:

``stage()``  (needs the reference tree and Cython)
    Cythonizes the hot-path ``.pyx`` files where they lie in the reference tree
    and gathers everything the C compiler needs into ``oracle/_ref/stage``:
    the generated C, the reference's helper C files they link against, and the
    three pure-Python modules they import.  ``oracle/_ref`` is git-ignored: the
    staged tree is a build intermediate and is never committed.

``compile_staged()``  (needs gcc, numpy and the Python headers)
    Compiles the staged tree into extension modules under
    ``oracle/_ref/pkg/nanopyx/core/transform`` with the reference's own flags
    (``-O3 -march=native -fopenmp``, ``setup.py:202-206``), and writes the
    small stub modules that replace the un-vendored ``liquid_engine`` package
    (it only dispatches ``run`` to ``_run_<runtype>``; no arithmetic).

``load()`` puts ``oracle/_ref/pkg`` on ``sys.path`` and returns the modules.

Reference files used (paths inside the reference project):
    src/nanopyx/core/transform/_le_esrrf.pyx
    src/nanopyx/core/transform/_le_interpolation_catmull_rom.pyx
    src/nanopyx/core/transform/_le_roberts_cross_gradients.pyx
    src/nanopyx/core/transform/_le_radial_gradient_convergence.pyx
    src/nanopyx/core/transform/_le_radiality.pyx
    src/nanopyx/core/transform/mpcorrector.pyx
    src/nanopyx/core/transform/{__interpolation_tools__,interpolation,sr_temporal_correlations}.py
    src/include/{_c_interpolation_catmull_rom,_c_gradients,
                 _c_sr_radial_gradient_convergence,_c_sr_radiality}.{c,h}
"""
from __future__ import annotations

import concurrent.futures as _cf
import os
import platform
import shutil
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")
STAGE = os.path.join(REF_OUT, "stage")
PKG = os.path.join(REF_OUT, "pkg")
# The reference checkout: $NANOPYX_REFERENCE_ROOT, else a directory named
# `reference` beside this repository's root (the layout the recipe is used
# with); without either, only an already staged tree can be compiled.
REFERENCE_ROOT = os.environ.get("NANOPYX_REFERENCE_ROOT") or os.path.join(
    os.path.dirname(os.path.dirname(HERE)), "reference")

PYX_MODULES = [
    "_le_interpolation_catmull_rom",
    "_le_roberts_cross_gradients",
    "_le_radial_gradient_convergence",
    "_le_radiality",
    "_le_esrrf",
    "mpcorrector",
]
# helper C files each extension links (from its `cdef extern from` lines)
C_DEPS = {
    "_le_interpolation_catmull_rom": ["_c_interpolation_catmull_rom"],
    "_le_roberts_cross_gradients": ["_c_gradients"],
    "_le_radial_gradient_convergence": ["_c_sr_radial_gradient_convergence"],
    "_le_radiality": ["_c_sr_radiality", "_c_interpolation_catmull_rom", "_c_gradients"],
    "_le_esrrf": [],
    "mpcorrector": [],
}
PY_MODULES = ["__interpolation_tools__", "interpolation", "sr_temporal_correlations"]

_STUB_LIQUID = '''"""Stand-in for the un-vendored ``liquid_engine`` dispatcher (no arithmetic)."""
import time


class LiquidEngine:
    def __init__(self, clear_benchmarks=False, testing=False, verbose=True, **kwargs):
        self._last_runtype = None
        self._last_time = None

    def _run(self, *args, run_type=None, **kwargs):
        name = "_run_" + (run_type or "threaded").lower()
        fn = getattr(self, name)
        t0 = time.perf_counter()
        out = fn(*args, **kwargs)
        self._last_time = time.perf_counter() - t0
        self._last_runtype = name[5:]
        return out

    def benchmark(self, *args, **kwargs):
        t0 = time.perf_counter()
        out = self._run_threaded(*args, **kwargs)
        return [[time.perf_counter() - t0, "Threaded", out]]
'''
_STUB_OPENCL = "cl = None\ncl_array = None\n_fastest_device = None\n"


def _ref_paths():
    tr = os.path.join(REFERENCE_ROOT, "src", "nanopyx", "core", "transform")
    inc = os.path.join(REFERENCE_ROOT, "src", "include")
    return tr, inc


def reference_present() -> bool:
    tr, inc = _ref_paths()
    return os.path.isfile(os.path.join(tr, "_le_esrrf.pyx")) and os.path.isdir(inc)


def staged() -> bool:
    return all(os.path.isfile(os.path.join(STAGE, "gen", m + ".c")) for m in PYX_MODULES)


def stage() -> None:
    """Cythonize the reference's hot-path modules into ``oracle/_ref/stage``."""
    tr, inc = _ref_paths()
    gen = os.path.join(STAGE, "gen")
    csrc = os.path.join(STAGE, "csrc")
    pysrc = os.path.join(STAGE, "py")
    for d in (gen, csrc, pysrc):
        os.makedirs(d, exist_ok=True)

    def cy(mod):
        out = os.path.join(gen, mod + ".c")
        src = os.path.join(tr, mod + ".pyx")
        if os.path.isfile(out) and os.path.getmtime(out) >= os.path.getmtime(src):
            return
        subprocess.run([sys.executable, "-m", "cython", "-3",
                        "--module-name", "nanopyx.core.transform." + mod,
                        "-I", inc, "-o", out, src], check=True)

    with _cf.ThreadPoolExecutor(len(PYX_MODULES)) as ex:
        list(ex.map(cy, PYX_MODULES))
    for deps in C_DEPS.values():
        for d in deps:
            for ext in (".c", ".h"):
                shutil.copyfile(os.path.join(inc, d + ext), os.path.join(csrc, d + ext))
    for m in PY_MODULES:
        shutil.copyfile(os.path.join(tr, m + ".py"), os.path.join(pysrc, m + ".py"))


def _arch_flags():
    if platform.machine() in ("aarch64", "arm64"):
        return [["-mcpu=native"], []]
    return [["-march=native"], []]


def compile_staged(jobs: int | None = None) -> None:
    """Compile the staged tree with gcc into ``oracle/_ref/pkg``."""
    import numpy

    gen = os.path.join(STAGE, "gen")
    csrc = os.path.join(STAGE, "csrc")
    pysrc = os.path.join(STAGE, "py")
    tdir = os.path.join(PKG, "nanopyx", "core", "transform")
    os.makedirs(tdir, exist_ok=True)
    for d, body in ((os.path.join(PKG, "nanopyx"), ""),
                    (os.path.join(PKG, "nanopyx", "core"), ""),
                    (tdir, "")):
        with open(os.path.join(d, "__init__.py"), "w") as f:
            f.write(body)
    with open(os.path.join(PKG, "nanopyx", "__liquid_engine__.py"), "w") as f:
        f.write(_STUB_LIQUID)
    with open(os.path.join(PKG, "nanopyx", "__opencl__.py"), "w") as f:
        f.write(_STUB_OPENCL)
    for m in PY_MODULES:
        shutil.copyfile(os.path.join(pysrc, m + ".py"), os.path.join(tdir, m + ".py"))

    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    incs = ["-I", sysconfig.get_paths()["include"], "-I", numpy.get_include(), "-I", csrc]

    def build(mod):
        out = os.path.join(tdir, mod + suffix)
        srcs = [os.path.join(gen, mod + ".c")] + [os.path.join(csrc, d + ".c") for d in C_DEPS[mod]]
        if os.path.isfile(out) and all(os.path.getmtime(out) >= os.path.getmtime(s) for s in srcs):
            return
        last = None
        for arch in _arch_flags():
            cmd = (["gcc", "-O3", *arch, "-fopenmp", "-fPIC", "-shared", "-w",
                    "-DNPY_NO_DEPRECATED_API=NPY_1_7_API_VERSION"] + incs + srcs +
                   ["-o", out, "-lm", "-fopenmp"])
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode == 0:
                return
            last = r.stderr
        raise RuntimeError(f"gcc failed for {mod}:\n{last}")

    with _cf.ThreadPoolExecutor(jobs or min(8, os.cpu_count() or 1)) as ex:
        list(ex.map(build, PYX_MODULES))


def build() -> bool:
    """Stage (when the reference tree is present) and compile. Returns success."""
    if reference_present():
        stage()
    if not staged():
        return False
    compile_staged()
    return True


def available() -> bool:
    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    tdir = os.path.join(PKG, "nanopyx", "core", "transform")
    return all(os.path.isfile(os.path.join(tdir, m + suffix)) for m in PYX_MODULES)


def load():
    """Import the compiled reference modules; returns a namespace dict."""
    if not available():
        raise RuntimeError("oracle/_ref is not built (run oracle.ref_build.build())")
    if PKG not in sys.path:
        sys.path.insert(0, PKG)
    import importlib

    t = "nanopyx.core.transform."
    mods = {m: importlib.import_module(t + m)
            for m in PYX_MODULES + ["sr_temporal_correlations", "interpolation"]}
    return {
        "CRShiftAndMagnify": mods["_le_interpolation_catmull_rom"].ShiftAndMagnify,
        "GradientRobertsCross": mods["_le_roberts_cross_gradients"].GradientRobertsCross,
        "RadialGradientConvergence": mods["_le_radial_gradient_convergence"].RadialGradientConvergence,
        "Radiality": mods["_le_radiality"].Radiality,
        "eSRRF_ST": mods["_le_esrrf"].eSRRF,
        "macro_pixel_corrector": mods["mpcorrector"].macro_pixel_corrector,
        "calculate_eSRRF_temporal_correlations":
            mods["sr_temporal_correlations"].calculate_eSRRF_temporal_correlations,
        "calculate_SRRF_temporal_correlations":
            mods["sr_temporal_correlations"].calculate_SRRF_temporal_correlations,
        "fht_space_interpolation": mods["interpolation"].fht_space_interpolation,
    }


if __name__ == "__main__":
    ok = build()
    print("oracle/_ref built" if ok else "oracle/_ref: nothing staged and no reference tree")
