"""Batched eSRRF: uneven stacks and parameter sweeps in persistent launches.

``EsrrfBatch`` plans many independent reconstructions -- different H, W, T,
magnification, radius, sensitivity and correlation -- and runs them as one
persistent kernel launch per kernel class (magnification, window half-width),
every CTA taking (stack, tile, timepoint, frame-chunk) units from a shared
work list, followed by the temporal finalisation and macro-pixel correction
of every item.  The launch sequence can be captured into a CUDA graph once and
replayed (``graph=True``).

A sensitivity sweep at one radius is a single item with up to four
sensitivities: the RGC map is evaluated once per frame and raised to each
sensitivity in the epilogue, so a 4 x 4 (radius x sensitivity) grid costs four
RGC passes instead of the sixteen full eSRRF runs of the reference sweep
(``src/nanopyx/core/analysis/parameter_sweep.py:33-37``).

Two autotuners cache their choices per GPU and kernel key (magnification,
window J) in ``~/.cache/nanopyx_gb300/autotune.json``: ``tune_tiling`` times a
batch under each kernel's tilings (the default, and one producer warp group
fewer for magnifications 2, 4, 5) and ``tune_frames_per_unit`` times one
reconstruction at several work-unit sizes.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import threading
import warnings

import numpy as np
import torch

from . import _native as N
from ._device import check_image, get_plan, require_cuda, workspace

__all__ = ["EsrrfBatch", "SweepGrid", "esrrf_batch", "sweep_batch", "tune_frames_per_unit",
           "tune_tiling"]

_CACHE_PATH = os.path.join(os.path.expanduser("~"), ".cache", "nanopyx_gb300", "autotune.json")
_cache_lock = threading.Lock()


def _corr_mask(corr):
    names = [corr] if isinstance(corr, str) else list(corr)
    if not names or any(n not in N.CORR_BITS for n in names):
        raise ValueError("Type of correlation must be AVG, VAR or TAC2")
    m = 0
    for n in names:
        m |= N.CORR_BITS[n]
    return names, m


class EsrrfBatch:
    """A fixed set of eSRRF reconstructions run as persistent batched launches.

    ``add(stack, ...)`` registers one reconstruction (a (T, H, W) float32 CUDA
    tensor or NumPy array, copied to the device once) and returns its index;
    ``run()`` executes everything and returns the list of outputs, each
    (n_outputs, n_timepoints, H*m, W*m) on the device (outputs follow the
    requested correlation order, or the sensitivity order for a sweep item).
    """

    def __init__(self, device=None, tiles=None):
        self.device = device if device is not None else require_cuda()
        # tile variant per (magnification, window J): explicit choices, else the
        # autotuner's cached ones, else 0 (the default tiling)
        self.tiles = dict(tiles or {})
        self._specs = []
        self._handle = None
        self._ws = None
        self._graph = None
        self.outputs = []

    def add(self, stack, magnification: int = 5, radius: float = 1.5, sensitivity=1,
            frames_per_timepoint: int = 0, temporal_correlation="AVG",
            doIntensityWeighting: bool = True, macro_pixel_correction: bool = True,
            frames_per_unit: int = 0) -> int:
        if self._handle is not None:
            raise RuntimeError("batch already planned")
        if isinstance(stack, torch.Tensor):
            t = check_image(stack).to(self.device).contiguous()
        else:
            t = torch.from_numpy(np.ascontiguousarray(check_image(stack))).to(self.device)
        T, H, W = t.shape
        sens_list = list(sensitivity) if isinstance(sensitivity, (list, tuple)) else None
        if sens_list is not None:
            if not 1 <= len(sens_list) <= 4:
                raise ValueError("a sweep item takes 1 to 4 sensitivities")
            names, mask = _corr_mask("AVG")
            if temporal_correlation != "AVG":
                raise ValueError("sensitivity sweeps are AVG only")
            plan_s = sens_list[0]
        else:
            names, mask = _corr_mask(temporal_correlation)
            plan_s = sensitivity
        m = int(magnification)
        fpt = T if frames_per_timepoint == 0 or frames_per_timepoint > T else int(frames_per_timepoint)
        n_tp = T // fpt + (1 if T % fpt else 0)
        order = [b for b in ("AVG", "VAR", "TAC2") if mask & N.CORR_BITS[b]]
        n_out = len(sens_list) if sens_list is not None else len(order)
        out = torch.empty((n_out, n_tp, H * m, W * m), dtype=torch.float32, device=self.device)
        plan = get_plan(H, W, m, radius, plan_s, doIntensityWeighting)
        self._specs.append(dict(stack=t, plan=plan, T=T, fpt=fpt, mask=mask, names=names,
                                order=order, sens=sens_list, mpc=bool(macro_pixel_correction),
                                out=out, fpu=int(frames_per_unit), key=(m, float(radius))))
        return len(self._specs) - 1

    # -- planning -----------------------------------------------------------
    def _items(self):
        arr = (N.EsrrfItem * len(self._specs))()
        for it, sp in zip(arr, self._specs):
            it.plan = sp["plan"].handle
            it.d_in = sp["stack"].data_ptr()
            it.T = sp["T"]
            it.frames_per_timepoint = sp["fpt"]
            it.corr_mask = sp["mask"]
            it.macro_pixel_correction = 1 if sp["mpc"] else 0
            sens = sp["sens"] or []
            it.n_sens = len(sens)
            for k, v in enumerate(sens):
                it.sens[k] = float(v)
            it.frames_per_unit = sp["fpu"] or _cached_fpu(sp["key"])
            it.d_out = sp["out"].data_ptr()
        return arr

    def kernel_keys(self):
        """The (magnification, window J) kernel keys of the batch's items."""
        return sorted({_kernel_key(*sp["key"]) for sp in self._specs})

    def plan(self):
        if not self._specs:
            raise ValueError("empty batch")
        L = N.lib()
        items = self._items()
        # the plans are shared with other calls: set each item's tiling only for
        # the batch's creation and binding, which fix it in the batch's kernel
        # classes and work lists, then restore the default
        chosen = {}
        for sp in self._specs:
            k = _kernel_key(*sp["key"])
            v = self.tiles.get(k, _cached_tile(k))
            chosen[k] = v if L.nx_esrrf_plan_set_tile_variant(sp["plan"].handle, v) == N.NX_OK else 0
        try:
            h = C.c_void_p()
            N.check(L.nx_esrrf_batch_create(C.byref(h), C.cast(items, C.c_void_p),
                                            len(self._specs)), "eSRRF batch")
            self._handle = h
            self._ws = workspace(L.nx_esrrf_batch_workspace_bytes(h), self.device)
            N.check(L.nx_esrrf_batch_bind(h, self._ws.data_ptr(), self._ws.numel(),
                                          torch.cuda.current_stream(self.device).cuda_stream),
                    "eSRRF batch")
        finally:
            for sp in self._specs:
                L.nx_esrrf_plan_set_tile_variant(sp["plan"].handle, 0)
        self.tiling = chosen
        self.outputs = [sp["out"] for sp in self._specs]
        return self

    def launch(self, stream=None):
        """Issue the batch on ``stream`` (default: current); capturable."""
        if self._handle is None:
            self.plan()
        s = stream if stream is not None else torch.cuda.current_stream(self.device).cuda_stream
        N.check(N.lib().nx_esrrf_batch_launch(self._handle, s), "eSRRF batch")

    def capture(self):
        """Capture the launch sequence into a CUDA graph (after one eager run)."""
        if self._handle is None:
            self.plan()
        side = torch.cuda.Stream(self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(side):
            self.launch(side.cuda_stream)  # warm-up: kernel attributes, lazy loading
        torch.cuda.current_stream(self.device).wait_stream(side)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.launch(torch.cuda.current_stream(self.device).cuda_stream)
        self._graph = g
        return self

    def run(self, graph: bool = False, check: bool = True):
        if graph:
            if self._graph is None:
                self.capture()
            self._graph.replay()
        else:
            self.launch()
        if check:
            N.check(N.lib().nx_workspace_status(
                self._ws.data_ptr(), torch.cuda.current_stream(self.device).cuda_stream),
                "eSRRF batch")
        outs = []
        for sp in self._specs:
            o = sp["out"]
            if sp["sens"] is None:
                o = o[[sp["order"].index(n) for n in sp["names"]]]
            outs.append(o)
        return outs

    def __del__(self):
        try:
            if self._handle is not None:
                N.lib().nx_esrrf_batch_destroy(self._handle)
        except Exception:
            pass


def esrrf_batch(stacks, params, graph: bool = False):
    """Run ``eSRRF`` on every stack with its own keyword arguments in one batch.

    ``params`` is a list of dicts with the keyword arguments of ``EsrrfBatch.add``.
    Returns the list of device outputs (see ``EsrrfBatch``).
    """
    b = EsrrfBatch()
    for st, kw in zip(stacks, params):
        b.add(st, **kw)
    return b.run(graph=graph)


class SweepGrid:
    """The (sensitivity x radius) AVG reconstruction grid of one stack, planned
    once and run as often as needed (``run(graph=True)`` replays one CUDA graph).

    One batch item per radius and group of up to four sensitivities: the RGC
    map of a radius is evaluated once per frame and raised to each sensitivity
    in the epilogue.  ``run`` returns a device tensor
    (len(sensitivities), len(radii), n_tp, H*m, W*m).
    """

    def __init__(self, stack, magnification: int, sensitivities, radii,
                 frames_per_timepoint: int = 0, doIntensityWeighting: bool = True,
                 macro_pixel_correction: bool = False, frames_per_unit: int = 0,
                 tiles=None, plan: bool = True):
        self.batch = b = EsrrfBatch(tiles=tiles)
        t = stack if isinstance(stack, torch.Tensor) else torch.from_numpy(
            np.ascontiguousarray(check_image(stack)))
        t = check_image(t).to(b.device).contiguous()
        self.sens, self.radii = list(sensitivities), list(radii)
        self.groups = [self.sens[i:i + 4] for i in range(0, len(self.sens), 4)]
        self.index = {}
        for r in self.radii:
            for g in self.groups:
                self.index[(float(r), tuple(g))] = b.add(
                    t, magnification, r, list(g), frames_per_timepoint, "AVG",
                    doIntensityWeighting, macro_pixel_correction, frames_per_unit)
        if plan:
            b.plan()

    def run(self, graph: bool = False, check: bool = True):
        outs = self.batch.run(graph=graph, check=check)
        rows = []
        for si in range(len(self.sens)):
            g = self.groups[si // 4]
            rows.append(torch.stack([outs[self.index[(float(r), tuple(g))]][si % 4]
                                     for r in self.radii]))
        return torch.stack(rows)


def sweep_batch(stack, magnification: int, sensitivities, radii, frames_per_timepoint: int = 0,
                doIntensityWeighting: bool = True, macro_pixel_correction: bool = False,
                graph: bool = False):
    """The (sensitivity x radius) AVG reconstruction grid in one batch (see
    ``SweepGrid``).  Returns a device tensor
    (len(sensitivities), len(radii), n_tp, H*m, W*m).
    """
    return SweepGrid(stack, magnification, sensitivities, radii, frames_per_timepoint,
                     doIntensityWeighting, macro_pixel_correction).run(graph=graph)


# ---------------------------------------------------------------------------
# autotuner: frames per work unit
# ---------------------------------------------------------------------------
# bumped whenever the kernels' tiling or unit structure changes, so that tunings
# made with an older build are not reused
TUNE_LAYOUT = "ws3"


def _gpu_key():
    p = torch.cuda.get_device_properties(torch.cuda.current_device())
    return f"{p.name}/{p.multi_processor_count}/{TUNE_LAYOUT}"


def _load_cache():
    try:
        with open(_CACHE_PATH) as f:
            return json.load(f)
    except Exception:
        return {}


def _kernel_key(m, r):
    """(magnification, window half-width J = int(2 R)): what selects a kernel."""
    return int(m), int(np.float32(2.0) * np.float32(r))


def _cached_fpu(key) -> int:
    m, J = _kernel_key(*key)
    return int(_load_cache().get(_gpu_key(), {}).get(f"m{m}_J{J}", 0))


def _cached_tile(kernel_key) -> int:
    m, J = kernel_key
    return int(_load_cache().get(_gpu_key(), {}).get(f"m{m}_J{J}_tile", 0))


def _store_fpu(gpu_key: str, magnification: int, J: int, fpu: int) -> bool:
    """Record a tuned frames-per-unit; False (and a warning) if the cache is not writable."""
    return _store(gpu_key, f"m{int(magnification)}_J{int(J)}", int(fpu))


def _store(gpu_key: str, name: str, value: int) -> bool:
    """Record one tuned value; False (and a warning) if the cache is not writable."""
    with _cache_lock:
        data = _load_cache()
        data.setdefault(gpu_key, {})[name] = int(value)
        try:
            os.makedirs(os.path.dirname(_CACHE_PATH), exist_ok=True)
            tmp = f"{_CACHE_PATH}.{os.getpid()}.tmp"
            with open(tmp, "w") as f:
                json.dump(data, f, indent=1, sort_keys=True)
            os.replace(tmp, _CACHE_PATH)  # atomic: concurrent tuners never see a torn file
        except OSError as e:
            warnings.warn(f"autotune cache not written ({e})")
            return False
    return True


def tune_frames_per_unit(stack, magnification: int = 5, radius: float = 1.5,
                         candidates=(8, 16, 32, 64, 0), repeats: int = 3,
                         temporal_correlation="AVG", save: bool = True):
    """Time one reconstruction at several frames-per-unit sizes; cache the best.

    ``0`` means the built-in heuristic.  Returns (best, {candidate: ms}).
    """
    times = {}
    for c in candidates:
        b = EsrrfBatch()
        b.add(stack, magnification, radius, 1, 0, temporal_correlation, frames_per_unit=c)
        b.plan()
        b.run(check=False)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(repeats):
            b.run(check=False)
        e1.record()
        torch.cuda.synchronize()
        times[c] = e0.elapsed_time(e1) / repeats
    best = min(times, key=times.get)
    if save:
        J = int(np.float32(2.0) * np.float32(radius))
        _store_fpu(_gpu_key(), magnification, J, best)
    return best, times


def _time_batch(b, repeats):
    b.run(check=False)  # plan, warm-up
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(repeats):
        b.run(check=False)
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / repeats


def tune_tiling(build, repeats: int = 2, save: bool = True):
    """Autotuner of the kernels' tiling for one batch.

    ``build(tiles)`` returns an unplanned ``EsrrfBatch`` of the workload with
    the given {(magnification, J): tile variant} choices.  Every kernel key
    with a second tiling (magnifications 2, 4, 5: one producer warp group
    fewer) is timed on the whole batch under both, the others held at their
    current choice; the faster is kept and, with ``save``, cached per GPU (later
    batches pick it up).  Returns {"m{m}_J{J}": {"variant": v, "ms": {v: ms}}}.
    """
    base = build({})
    keys = base.kernel_keys()
    choice = {k: 0 for k in keys}
    t0 = _time_batch(build(dict(choice)), repeats)
    report = {}
    for k in keys:
        trial = dict(choice)
        trial[k] = 1
        probe = build(trial)
        probe.plan()
        if probe.tiling.get(k, 0) != 1:  # no second tiling for this key
            report[f"m{k[0]}_J{k[1]}"] = {"variant": 0, "ms": {0: t0}}
            continue
        t1 = _time_batch(probe, repeats)
        report[f"m{k[0]}_J{k[1]}"] = {"variant": 1 if t1 < t0 else 0, "ms": {0: t0, 1: t1}}
        if t1 < t0:
            choice[k], t0 = 1, t1
    if save:
        for (m, J), v in choice.items():
            _store(_gpu_key(), f"m{m}_J{J}_tile", v)
    return report
