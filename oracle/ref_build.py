"""Recipe that builds the reference's own eSRRF/SRRF CPU path into ``oracle/_ref``.

TEST INFRASTRUCTURE ONLY.  Nothing in ``nanopyx_gb300`` imports this module;
only ``tests/``, ``__graft_entry__`` (build/smoke) and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` use what it produces, to check results
and as the timed CPU baseline.

Two stages, so that the compiled reference can also be produced on a machine
that has no copy of the reference tree:

``stage()``  (needs the reference tree and Cython)
    Cythonizes the reference's ``.pyx`` files for this path where they lie in
    the reference tree and gathers everything the C compiler needs into
    ``oracle/_ref/stage``: the generated C, the reference's helper C files they
    link against, and the pure-Python modules they import.  ``oracle/_ref`` is
    git-ignored: the staged tree is a build intermediate and is never committed.

``compile_staged()``  (needs gcc, numpy and the Python headers)
    Compiles the staged tree into extension modules under
    ``oracle/_ref/pkg/nanopyx/core/<package>`` with the reference's own flags
    (``-O3 -march=native -fopenmp``, ``setup.py:202-206``), and writes the
    small stub modules that replace the un-vendored ``liquid_engine`` package
    (it only dispatches ``run`` to ``_run_<runtype>``; no arithmetic) and the
    plotting / progress-bar imports (``matplotlib.pyplot``, ``tqdm``) of the
    sweep-scoring modules, which the returned numbers never touch.

``load()`` puts ``oracle/_ref/pkg`` on ``sys.path`` and returns the modules.

Reference files used (paths inside the reference project):
    src/nanopyx/core/transform/_le_esrrf.pyx
    src/nanopyx/core/transform/_le_interpolation_catmull_rom.pyx
    src/nanopyx/core/transform/_le_roberts_cross_gradients.pyx
    src/nanopyx/core/transform/_le_radial_gradient_convergence.pyx
    src/nanopyx/core/transform/_le_radiality.pyx
    src/nanopyx/core/transform/mpcorrector.pyx
    src/nanopyx/core/transform/_le_esrrf3d.pyx
    src/nanopyx/core/transform/{_interpolation,error_map,edges,normalize}.pyx
    src/nanopyx/core/transform/{__interpolation_tools__,interpolation,
                                sr_temporal_correlations,padding}.py
    src/nanopyx/core/analysis/{pearson_correlation,ccm_helper_functions,frc,decorr}.pyx
    src/nanopyx/core/analysis/parameter_sweep.py
    src/nanopyx/core/utils/{math,array}.pyx, src/nanopyx/core/utils/timeit.py
    src/nanopyx/core/generate/mask.pyx
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

# (package under nanopyx/core, module, helper C files it links from its
# `cdef extern from` lines)
PYX_SPECS = [
    ("transform", "_le_interpolation_catmull_rom", ["_c_interpolation_catmull_rom"]),
    ("transform", "_le_roberts_cross_gradients", ["_c_gradients"]),
    ("transform", "_le_radial_gradient_convergence", ["_c_sr_radial_gradient_convergence"]),
    ("transform", "_le_radiality", ["_c_sr_radiality", "_c_interpolation_catmull_rom", "_c_gradients"]),
    ("transform", "_le_esrrf", []),
    ("transform", "mpcorrector", []),
    # eSRRF-3D
    ("transform", "_le_esrrf3d", ["_c_gradients", "_c_sr_radial_gradient_convergence"]),
    # the parameter sweep's scoring: ErrorMap (RSP), FIRECalculator (FRC),
    # DecorrAnalysis and what they cimport
    ("transform", "_interpolation", ["_c_interpolation_catmull_rom"]),
    ("transform", "error_map", []),
    ("transform", "edges", []),
    ("transform", "normalize", []),
    ("analysis", "pearson_correlation", []),
    ("analysis", "ccm_helper_functions", []),
    ("analysis", "frc", []),
    ("analysis", "decorr", []),
    ("utils", "math", []),
    ("utils", "array", []),
    ("generate", "mask", []),
]
PYX_MODULES = [m for _, m, _ in PYX_SPECS]
PY_SPECS = [
    ("transform", "__interpolation_tools__"),
    ("transform", "interpolation"),
    ("transform", "sr_temporal_correlations"),
    ("transform", "padding"),
    ("analysis", "parameter_sweep"),
    ("utils", "timeit"),
]
PACKAGES = ("transform", "analysis", "utils", "generate")

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
# plotting and progress bars of the sweep/FRC/decorrelation modules: imported
# at module level by the reference, never used by the numbers it returns
_STUB_PYPLOT = ("def __getattr__(name):\n"
                "    raise RuntimeError('plotting is not available in the compiled reference')\n")
_STUB_TQDM = (
    '"""No-op progress bar standing in for tqdm."""\n\n\n'
    "class tqdm:\n"
    "    def __init__(self, *args, **kwargs):\n"
    "        pass\n\n"
    "    def __enter__(self):\n"
    "        return self\n\n"
    "    def __exit__(self, *exc):\n"
    "        return False\n\n"
    "    def update(self, n=1):\n"
    "        pass\n")


def _core():
    return os.path.join(REFERENCE_ROOT, "src", "nanopyx", "core")


def _ref_paths():
    tr = os.path.join(_core(), "transform")
    inc = os.path.join(REFERENCE_ROOT, "src", "include")
    return tr, inc


def reference_present() -> bool:
    tr, inc = _ref_paths()
    return os.path.isfile(os.path.join(tr, "_le_esrrf.pyx")) and os.path.isdir(inc)


def staged() -> bool:
    return all(os.path.isfile(os.path.join(STAGE, "gen", m + ".c")) for m in PYX_MODULES)


def stage() -> None:
    """Cythonize the reference's modules into ``oracle/_ref/stage``."""
    _, inc = _ref_paths()
    src_root = os.path.join(REFERENCE_ROOT, "src")
    gen = os.path.join(STAGE, "gen")
    csrc = os.path.join(STAGE, "csrc")
    pysrc = os.path.join(STAGE, "py")
    for d in (gen, csrc, pysrc):
        os.makedirs(d, exist_ok=True)

    def cy(spec):
        pkg, mod, _ = spec
        out = os.path.join(gen, mod + ".c")
        src = os.path.join(_core(), pkg, mod + ".pyx")
        if os.path.isfile(out) and os.path.getmtime(out) >= os.path.getmtime(src):
            return
        subprocess.run([sys.executable, "-m", "cython", "-3",
                        "--module-name", f"nanopyx.core.{pkg}.{mod}",
                        "-I", inc, "-I", src_root, "-o", out, src], check=True)

    with _cf.ThreadPoolExecutor(min(8, len(PYX_SPECS))) as ex:
        list(ex.map(cy, PYX_SPECS))
    for _, _, deps in PYX_SPECS:
        for d in deps:
            for ext in (".c", ".h"):
                shutil.copyfile(os.path.join(inc, d + ext), os.path.join(csrc, d + ext))
    for pkg, m in PY_SPECS:
        shutil.copyfile(os.path.join(_core(), pkg, m + ".py"), os.path.join(pysrc, m + ".py"))


def _arch_flags():
    if platform.machine() in ("aarch64", "arm64"):
        return [["-mcpu=native"], []]
    return [["-march=native"], []]


def _write(path, body):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as f:
        f.write(body)


def compile_staged(jobs: int | None = None) -> None:
    """Compile the staged tree with gcc into ``oracle/_ref/pkg``."""
    import numpy

    gen = os.path.join(STAGE, "gen")
    csrc = os.path.join(STAGE, "csrc")
    pysrc = os.path.join(STAGE, "py")
    core = os.path.join(PKG, "nanopyx", "core")
    _write(os.path.join(PKG, "nanopyx", "__init__.py"), "")
    _write(os.path.join(core, "__init__.py"), "")
    for pkg in PACKAGES:
        _write(os.path.join(core, pkg, "__init__.py"), "")
    _write(os.path.join(PKG, "nanopyx", "__liquid_engine__.py"), _STUB_LIQUID)
    _write(os.path.join(PKG, "nanopyx", "__opencl__.py"), _STUB_OPENCL)
    _write(os.path.join(PKG, "matplotlib", "__init__.py"), "")
    _write(os.path.join(PKG, "matplotlib", "pyplot.py"), _STUB_PYPLOT)
    _write(os.path.join(PKG, "tqdm", "__init__.py"), _STUB_TQDM)
    pkg_of = dict((m, p) for p, m in PY_SPECS)
    for m, pkg in pkg_of.items():
        shutil.copyfile(os.path.join(pysrc, m + ".py"), os.path.join(core, pkg, m + ".py"))

    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    incs = ["-I", sysconfig.get_paths()["include"], "-I", numpy.get_include(), "-I", csrc]

    def build(spec):
        pkg, mod, deps = spec
        out = os.path.join(core, pkg, mod + suffix)
        srcs = [os.path.join(gen, mod + ".c")] + [os.path.join(csrc, d + ".c") for d in deps]
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
        list(ex.map(build, PYX_SPECS))


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
    core = os.path.join(PKG, "nanopyx", "core")
    return all(os.path.isfile(os.path.join(core, p, m + suffix)) for p, m, _ in PYX_SPECS)


def load():
    """Import the compiled reference modules; returns a namespace dict."""
    if not available():
        raise RuntimeError("oracle/_ref is not built (run oracle.ref_build.build())")
    if PKG not in sys.path:
        sys.path.insert(0, PKG)
    import importlib

    names = [(p, m) for p, m, _ in PYX_SPECS] + [
        ("transform", "sr_temporal_correlations"), ("transform", "interpolation"),
        ("analysis", "parameter_sweep")]
    mods = {m: importlib.import_module(f"nanopyx.core.{p}.{m}") for p, m in names}
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
        "dht_interpolation": mods["_interpolation"].fht_space_interpolation,
        "ErrorMap": mods["error_map"].ErrorMap,
        "FIRECalculator": mods["frc"].FIRECalculator,
        "DecorrAnalysis": mods["decorr"].DecorrAnalysis,
        "ParameterSweep": mods["parameter_sweep"].ParameterSweep,
        "pearson_correlation": mods["pearson_correlation"].pearson_correlation,
        "eSRRF3D_ST": mods["_le_esrrf3d"].eSRRF3D,
    }


if __name__ == "__main__":
    ok = build()
    print("oracle/_ref built" if ok else "oracle/_ref: nothing staged and no reference tree")
