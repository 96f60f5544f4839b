"""User-level methods: ``eSRRF``, ``SRRF``, ``Workflow`` and the parameter sweep.

Drop-ins for (paths inside the reference project):

* ``eSRRF`` -- ``src/nanopyx/methods/esrrf/eSRRF_workflow.py:12-121``
* ``SRRF`` -- ``src/nanopyx/methods/srrf/SRRF_workflow.py:9-76``
* ``Workflow`` -- ``src/nanopyx/methods/workflow.py:4-139``
* ``esrrf_parameter_sweep`` -- the reconstruction grid of
  ``src/nanopyx/core/analysis/parameter_sweep.py:17-97`` (one eSRRF run per
  (sensitivity, radius) pair).  Its QnR scoring (ErrorMap, FRC, decorrelation)
  is not part of this engine.

``eSRRF`` runs the whole timepoint loop on the device: one fused kernel per
call produces every timepoint's temporal correlation(s), then the macro-pixel
correction runs on the device too; only the final images come back.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _native as N
from ._device import check_image, get_plan, stream_ptr, to_device_stack, workspace
from .transform import (GradientRobertsCross, Radiality, ShiftAndMagnify,  # noqa: F401
                        macro_pixel_corrector)

__all__ = ["eSRRF", "eSRRF3D", "SRRF", "Workflow", "ESRRFAccumulator", "esrrf_parameter_sweep",
           "esrrf_device"]


def _corr_list(temporal_correlation):
    names = [temporal_correlation] if isinstance(temporal_correlation, str) else list(
        temporal_correlation)
    if not names or any(n not in N.CORR_BITS for n in names):
        raise ValueError("Type of correlation must be AVG, VAR or TAC2")
    return names


def esrrf_device(stack: torch.Tensor, magnification: int = 5, radius: float = 1.5,
                 sensitivity: float = 1, frames_per_timepoint: int = 0,
                 temporal_correlation="AVG", doIntensityWeighting: bool = True,
                 macro_pixel_correction: bool = True, check_status: bool = True):
    """eSRRF on a resident (T, H, W) float32 CUDA tensor.

    Returns a (n_corr, n_timepoints, H*m, W*m) CUDA tensor, correlations in the
    order requested.  Asynchronous on the current stream unless ``check_status``.
    """
    names = _corr_list(temporal_correlation)
    mask = 0
    for n in names:
        mask |= N.CORR_BITS[n]
    T, H, W = stack.shape
    if T < 1:
        raise ValueError("eSRRF needs at least one frame")
    fpt = T if frames_per_timepoint == 0 or frames_per_timepoint > T else int(frames_per_timepoint)
    if fpt < 0:
        raise ValueError("frames_per_timepoint must be >= 0")
    n_tp = T // fpt + (1 if T % fpt else 0)
    m = int(magnification)
    plan = get_plan(H, W, m, radius, sensitivity, doIntensityWeighting)
    L = N.lib()
    ws = workspace(L.nx_esrrf_workspace_bytes(plan.handle, T, fpt, mask), stack.device)
    order = [b for b in ("AVG", "VAR", "TAC2") if mask & N.CORR_BITS[b]]
    out = torch.empty((len(order), n_tp, H * m, W * m), dtype=torch.float32, device=stack.device)
    N.check(L.nx_esrrf_run(plan.handle, stack.data_ptr(), T, fpt, mask,
                           1 if macro_pixel_correction else 0, out.data_ptr(), ws.data_ptr(),
                           ws.numel(), stream_ptr()), "eSRRF")
    if check_status:
        N.check(L.nx_workspace_status(ws.data_ptr(), stream_ptr()), "eSRRF")
    idx = [order.index(n) for n in names]
    if idx != list(range(len(order))):
        out = out[idx]
    return out


def eSRRF(image, magnification: int = 5, radius: float = 1.5, sensitivity: float = 1,
          frames_per_timepoint: int = 0, temporal_correlation="AVG", use_fht: bool = False,
          doIntensityWeighting: bool = True, macro_pixel_correction: bool = True,
          pad_edges: bool = False, _force_run_type=None):
    """eSRRF reconstruction (reference signature and semantics).

    ``temporal_correlation`` may also be a sequence of names; the result is then
    a tuple with one squeezed array per name, computed in a single pass.
    ``pad_edges`` only acts with ``use_fht=True``, as in the reference.
    """
    names = _corr_list(temporal_correlation)
    if use_fht:
        return _esrrf_fht(image, magnification, radius, sensitivity, frames_per_timepoint, names,
                          isinstance(temporal_correlation, str), doIntensityWeighting,
                          macro_pixel_correction, pad_edges)
    if isinstance(image, torch.Tensor) and image.is_cuda:
        st = to_device_stack(image)
        out = esrrf_device(st.t, magnification, radius, sensitivity, frames_per_timepoint,
                           names, doIntensityWeighting, macro_pixel_correction)
        parts = [torch.squeeze(out[i]) for i in range(len(names))]
    else:
        img = check_image(image.numpy() if isinstance(image, torch.Tensor) else image)
        res = _esrrf_host(np.ascontiguousarray(img), magnification, radius, sensitivity,
                          frames_per_timepoint, names, doIntensityWeighting,
                          macro_pixel_correction)
        parts = [np.squeeze(res[i]) for i in range(len(names))]
    return parts[0] if isinstance(temporal_correlation, str) else tuple(parts)


def _esrrf_fht(image, magnification, radius, sensitivity, frames_per_timepoint, names, single,
               iw, mpc, pad_edges):
    """eSRRF() with use_fht=True: per timepoint the Fourier-path eSRRF_ST stack,
    then the temporal correlation and the macro-pixel correction of each name
    (eSRRF_workflow.py:76-121), all on the device."""
    from .transform import _esrrf_st_fht, calculate_eSRRF_temporal_correlations, \
        macro_pixel_corrector

    on_dev = isinstance(image, torch.Tensor) and image.is_cuda
    st = to_device_stack(image)
    x = st.t
    T = x.shape[0]
    fpt = T if frames_per_timepoint == 0 or frames_per_timepoint > T else int(frames_per_timepoint)
    m = int(magnification)
    res = {n: [] for n in names}
    for a in range(0, T, fpt):
        rgc = _esrrf_st_fht(x[a:a + fpt].contiguous(), m, radius, sensitivity, iw, pad_edges)
        for n in names:
            tc = calculate_eSRRF_temporal_correlations(rgc, n)
            res[n].append(macro_pixel_corrector(tc[None], m)[0] if mpc else tc)
    parts = []
    for n in names:
        o = torch.squeeze(torch.stack(res[n]))
        parts.append(o if on_dev else o.cpu().numpy())
    return parts[0] if single else tuple(parts)


def upload_segments(T: int, fpt: int):
    """Frame ranges uploaded per timepoint by the host-buffer eSRRF path.

    A timepoint goes up whole when there are at least three (one segment
    overlaps the previous timepoint's compute), else in quarters; the first
    timepoint starts with a head of ~1/5 of its frames so that the device
    starts early.  Returns, per timepoint, a list of (first, end) frame indices
    that tile [0, T).
    """
    n_tp = T // fpt + (1 if T % fpt else 0)
    nseg = 1 if n_tp >= 3 else min(4, fpt)
    seg_len = -(-fpt // nseg)
    head = fpt // 5 if nseg == 1 and fpt >= 10 else seg_len
    segs = []
    for tp in range(n_tp):
        a0, a1 = tp * fpt, min(T, (tp + 1) * fpt)
        cuts = [a0 + head] if tp == 0 and head < seg_len else []
        cuts += list(range(a0 + seg_len, a1, seg_len)) + [a1]
        segs.append(list(zip([a0] + cuts[:-1], cuts)))
    return segs


def _esrrf_host(arr: np.ndarray, magnification, radius, sensitivity, frames_per_timepoint,
                names, doIntensityWeighting, macro_pixel_correction) -> np.ndarray:
    """eSRRF with host buffers, copies overlapped with compute.

    The stack is uploaded in segments (a timepoint, or a quarter of it when
    there are fewer than three timepoints): host threads copy a segment into
    one of two pinned buffers, a copy stream moves it to the device, and the
    compute stream folds it into its timepoint's device-resident accumulator
    while the next segment is staged.  Each finished timepoint goes back the
    same way (device -> pinned on the copy stream, pinned -> result by the host
    threads) while the next computes.  Same arithmetic as ``esrrf_device``.
    Returns (n_corr, n_timepoints, H*m, W*m) float32.
    """
    from ._device import require_cuda
    from ._hostio import par_copy, pinned

    dev = require_cuda()
    T, H, W = arr.shape
    if T < 1:
        raise ValueError("eSRRF needs at least one frame")
    fpt = T if frames_per_timepoint == 0 or frames_per_timepoint > T else int(frames_per_timepoint)
    if fpt < 0:
        raise ValueError("frames_per_timepoint must be >= 0")
    n_tp = T // fpt + (1 if T % fpt else 0)
    m = int(magnification)
    mask = 0
    for n in names:
        mask |= N.CORR_BITS[n]
    order = [b for b in ("AVG", "VAR", "TAC2") if mask & N.CORR_BITS[b]]
    sel = [order.index(n) for n in names]
    L = N.lib()
    plan = get_plan(H, W, m, radius, sensitivity, doIntensityWeighting)
    comp = torch.cuda.current_stream(dev)
    cp = torch.cuda.Stream(dev)   # host -> device
    cpo = torch.cuda.Stream(dev)  # device -> host (never queues behind an upload)
    segs = upload_segments(T, fpt)
    max_seg = max(sb - sa for tsegs in segs for sa, sb in tsegs)
    ws_push = workspace(max(L.nx_esrrf_push_workspace_bytes(plan.handle, n)
                            for n in {sb - sa for tsegs in segs for sa, sb in tsegs}), dev)
    ws_fin = workspace(256 + L.nx_macro_pixel_workspace_bytes(3, m), dev)
    acc = [torch.empty(L.nx_esrrf_accum_bytes(plan.handle), dtype=torch.uint8, device=dev)
           for _ in range(2)]
    outs = [torch.empty((len(order), H * m, W * m), dtype=torch.float32, device=dev)
            for _ in range(2)]
    seg_dev = [torch.empty((max_seg, H, W), dtype=torch.float32, device=dev) for _ in range(2)]
    seg_pin = [pinned((max_seg, H, W)) for _ in range(2)]
    out_pin = [pinned((len(order), H * m, W * m)) for _ in range(2)]
    seg_free = [None, None]  # event: the H2D copy out of seg_pin[i] has finished
    seg_used = [None, None]  # event: the push reading seg_dev[i] has finished
    res = np.empty((len(names), n_tp, H * m, W * m), dtype=np.float32)
    done = [None, None]
    back = [None, None]

    def fetch(tp):
        # device -> pinned on the download stream once timepoint tp is finalised
        k = tp & 1
        cpo.wait_event(done[k])
        with torch.cuda.stream(cpo):
            out_pin[k].copy_(outs[k], non_blocking=True)
            back[k] = cpo.record_event()

    def drain(tp):
        k = tp & 1
        back[k].synchronize()
        src = out_pin[k].numpy()
        for i, si in enumerate(sel):
            par_copy(res[i, tp], src[si])

    pending = None
    iseg = 0
    for tp in range(n_tp):
        k = tp & 1
        before = 0
        for sa, sb in segs[tp]:
            j = iseg & 1
            iseg += 1
            if seg_free[j] is not None:
                seg_free[j].synchronize()
            par_copy(seg_pin[j].numpy()[: sb - sa], arr[sa:sb])
            with torch.cuda.stream(cp):
                # seg_dev[j] is free once the push two segments ago has run
                if seg_used[j] is not None:
                    cp.wait_event(seg_used[j])
                seg_dev[j][: sb - sa].copy_(seg_pin[j][: sb - sa], non_blocking=True)
                seg_free[j] = cp.record_event()
            comp.wait_event(seg_free[j])
            N.check(L.nx_esrrf_accum_push(plan.handle, seg_dev[j].data_ptr(), sb - sa, before,
                                          acc[k].data_ptr(), ws_push.data_ptr(), ws_push.numel(),
                                          comp.cuda_stream), "eSRRF push")
            seg_used[j] = comp.record_event()
            before += sb - sa
        if pending is not None:
            drain(pending)  # outs / out_pin of pending & 1 are free again after this
        N.check(L.nx_esrrf_accum_finalize(plan.handle, acc[k].data_ptr(), before, mask,
                                          1 if macro_pixel_correction else 0,
                                          outs[k].data_ptr(), ws_fin.data_ptr(),
                                          ws_fin.numel(), comp.cuda_stream), "eSRRF finalize")
        done[k] = comp.record_event()
        fetch(tp)
        pending = tp
    drain(pending)
    N.check(L.nx_workspace_status(ws_push.data_ptr(), comp.cuda_stream), "eSRRF")
    return res


def SRRF(image, magnification: int = 5, ringRadius: float = 0.5, border: int = 0,
         radialityPositivityConstraint: bool = True, doIntensityWeighting: bool = True,
         macro_pixel_correction: bool = True, _force_run_type=None):
    """SRRF per-frame radiality stack (T, H*m, W*m), macro-pixel corrected per frame.

    One fused pass per frame block: the magnified intensity is formed inside the
    radiality kernel instead of being materialised (the reference's two-step
    CRShiftAndMagnify -> Radiality workflow, SRRF_workflow.py:50-67).
    """
    st = to_device_stack(image)
    T, h, w = st.shape
    m = int(magnification)
    L = N.lib()
    out = torch.empty((T, h * m, w * m), dtype=torch.float32, device=st.t.device)
    ws = workspace(L.nx_srrf_workspace_bytes(T, h, w, m), st.t.device)
    N.check(L.nx_srrf(st.ptr(), T, h, w, m, float(ringRadius), int(border),
                      1 if radialityPositivityConstraint else 0, 1 if doIntensityWeighting else 0,
                      1 if macro_pixel_correction else 0, out.data_ptr(), ws.data_ptr(),
                      ws.numel(), stream_ptr()), "SRRF")
    return st.out(out)


class Workflow:
    """Sequential op chain with ``PREV_RETURN_VALUE_<i>_<j>`` argument wiring."""

    def __init__(self, *args):
        self._methods = []
        self._return_values = []
        for arg in args:
            if isinstance(arg, tuple) and len(arg) == 3:
                self._methods.append((arg[0], arg[1], arg[2]))
            else:
                raise TypeError("Each arg must be a tuple of 3 items (fn, args, kwargs)")

    @staticmethod
    def _resolve(v, values):
        if isinstance(v, str) and "PREV_RETURN_VALUE" in v:
            idx = [int(i) for i in v.split("_") if i.isdigit()]
            return values[idx[0]][idx[1]]
        return v

    def run(self, _force_run_type=None):
        fn = None
        for fn, args, kwargs in self._methods:
            sane_args = [self._resolve(a, self._return_values) for a in args]
            kw = {k: self._resolve(v, self._return_values) for k, v in kwargs.items()}
            kw["run_type"] = _force_run_type
            rv = fn.run(*sane_args, **kw)
            self._return_values.append(rv if isinstance(rv, tuple) else (rv,))
        return self._return_values[-1], fn._last_runtype, fn._last_time

    def calculate(self, _force_run_type=None):
        output, _, _ = self.run(_force_run_type=_force_run_type)
        return output


def esrrf_parameter_sweep(img, magnification: int = 2, sensitivities=(1, 2), radii=(1, 1.5),
                          temporal_correlation: str = "AVG", frames_per_timepoint: int = 0,
                          doIntensityWeighting: bool = True, macro_pixel_correction: bool = False,
                          graph: bool = False):
    """Reconstruction grid of the eSRRF parameter sweep.

    Returns an array (len(sensitivities), len(radii), n_timepoints, H*m, W*m)
    (squeezed over timepoints when there is one).  The whole grid runs as one
    batch (``nanopyx_gb300.engine.sweep_batch``): one RGC pass per radius serves
    up to four sensitivities; the reference runs a full, independent eSRRF_ST
    per (sensitivity, radius) pair (parameter_sweep.py:35-37).
    """
    if temporal_correlation != "AVG":
        raise ValueError("the batched sweep computes AVG reconstructions")
    from .engine import sweep_batch

    from_numpy = not (isinstance(img, torch.Tensor) and img.is_cuda)
    res = sweep_batch(img if isinstance(img, torch.Tensor) else np.asarray(img), magnification,
                      sensitivities, radii, frames_per_timepoint, doIntensityWeighting,
                      macro_pixel_correction, graph=graph)
    if res.shape[2] == 1:
        res = res[:, :, 0]
    return res.cpu().numpy() if from_numpy else res


class ESRRFAccumulator:
    """Device-resident temporal state of one eSRRF reconstruction.

    Frame blocks are pushed as they arrive (``push``); the per-pixel streaming
    moments (first value, running mean, M2, lag-1 co-moment, last value) stay
    on the device between pushes, so a reconstruction
    over many blocks never holds its per-frame stack anywhere.  ``finalize``
    returns the requested correlations (each (H*m, W*m)), macro-pixel corrected
    if asked, with the same arithmetic as ``eSRRF`` over one timepoint.
    """

    def __init__(self, H: int, W: int, magnification: int = 5, radius: float = 1.5,
                 sensitivity: float = 1, doIntensityWeighting: bool = True, device=None):
        from ._device import require_cuda

        self.device = device if device is not None else require_cuda()
        self.H, self.W, self.m = int(H), int(W), int(magnification)
        self.plan = get_plan(H, W, magnification, radius, sensitivity, doIntensityWeighting)
        L = N.lib()
        self.state = torch.empty(L.nx_esrrf_accum_bytes(self.plan.handle), dtype=torch.uint8,
                                 device=self.device)
        self.frames = 0
        self._ws = None

    def _workspace(self, nbytes):
        if self._ws is None or self._ws.numel() < nbytes:
            self._ws = workspace(nbytes, self.device)
        return self._ws

    def push(self, block) -> None:
        """Add a (T_block, H, W) block (NumPy or CUDA tensor) to the state."""
        st = to_device_stack(block)
        T, H, W = st.shape
        if (H, W) != (self.H, self.W):
            raise ValueError("block frame size does not match the accumulator")
        L = N.lib()
        ws = self._workspace(L.nx_esrrf_push_workspace_bytes(self.plan.handle, T))
        N.check(L.nx_esrrf_accum_push(self.plan.handle, st.ptr(), T, self.frames,
                                      self.state.data_ptr(), ws.data_ptr(), ws.numel(),
                                      stream_ptr()), "eSRRF push")
        self._keep = st.t  # the input must outlive the asynchronous push
        self.frames += T

    def finalize_device(self, temporal_correlation="AVG", macro_pixel_correction: bool = True):
        names = _corr_list(temporal_correlation)
        mask = 0
        for n in names:
            mask |= N.CORR_BITS[n]
        if self.frames < 1:
            raise ValueError("no frames were pushed")
        order = [b for b in ("AVG", "VAR", "TAC2") if mask & N.CORR_BITS[b]]
        out = torch.empty((len(order), self.H * self.m, self.W * self.m), dtype=torch.float32,
                          device=self.device)
        L = N.lib()
        ws = self._workspace(256 + L.nx_macro_pixel_workspace_bytes(3, self.m))
        N.check(L.nx_esrrf_accum_finalize(self.plan.handle, self.state.data_ptr(), self.frames,
                                          mask, 1 if macro_pixel_correction else 0,
                                          out.data_ptr(), ws.data_ptr(), ws.numel(),
                                          stream_ptr()), "eSRRF finalize")
        return out[[order.index(n) for n in names]]

    def finalize(self, temporal_correlation="AVG", macro_pixel_correction: bool = True):
        out = self.finalize_device(temporal_correlation, macro_pixel_correction)
        N.check(N.lib().nx_workspace_status(self._ws.data_ptr(), stream_ptr()), "eSRRF")
        res = out.cpu().numpy()
        return res[0] if isinstance(temporal_correlation, str) else tuple(res)


def eSRRF3D(img, magnification_xy=2, magnification_z=2, radius: float = 1.5,
            PSF_ratio: float = 2.8, voxel_ratio: float = 4.0, sensitivity: float = 1,
            frames_per_timepoint: int = 0, mode: str = "average", doIntensityWeighting: bool = True,
            macro_pixel_correction: bool = True, _force_run_type=None):
    """eSRRF-3D of a (T, S, H, W) stack (methods/esrrf_3d/eSRRF3D_workflow.py:8-107):
    per timepoint of ``frames_per_timepoint`` frames an eSRRF3D_ST volume
    (S*mz, H*mxy, W*mxy), macro-pixel corrected slice by slice; returns
    (n_timepoints, S*mz, H*mxy, W*mxy) float32 (NumPy in, NumPy out; CUDA
    tensor in, CUDA tensor out)."""
    from .transform import eSRRF3D_ST, macro_pixel_corrector

    T = img.shape[0]
    if frames_per_timepoint == 0 or frames_per_timepoint > T:
        frames_per_timepoint = T
    n_tp = T // frames_per_timepoint + (1 if T % frames_per_timepoint else 0)
    on_dev = isinstance(img, torch.Tensor) and img.is_cuda
    outs = []
    for i in range(n_tp):
        v = eSRRF3D_ST(verbose=False).run(
            img[frames_per_timepoint * i:frames_per_timepoint * (i + 1)],
            magnification_xy=magnification_xy, magnification_z=magnification_z, radius=radius,
            PSF_ratio=PSF_ratio, voxel_ratio=voxel_ratio, sensitivity=sensitivity, mode=mode,
            doIntensityWeighting=doIntensityWeighting)
        if v is None:
            raise ValueError("eSRRF3D: radius or radius_z too large for the volume")
        if macro_pixel_correction:
            v = macro_pixel_corrector(v, magnification=magnification_xy)
        outs.append(v)
    if on_dev:
        return torch.stack([o if isinstance(o, torch.Tensor) else torch.as_tensor(o) for o in outs])
    return np.stack([np.asarray(o, dtype=np.float32) for o in outs]).astype(np.float32)
