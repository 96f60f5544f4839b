"""The Liquid-Engine ops of the eSRRF / SRRF path, on the GB300 CUDA path.

Drop-ins for (paths inside the reference project):

* ``ShiftAndMagnify`` (exported as ``CRShiftAndMagnify``)
  -- ``src/nanopyx/core/transform/_le_interpolation_catmull_rom.pyx:17``
* ``GradientRobertsCross`` -- ``.../_le_roberts_cross_gradients.pyx:16``
* ``RadialGradientConvergence`` -- ``.../_le_radial_gradient_convergence.pyx:16``
* ``Radiality`` -- ``.../_le_radiality.pyx:27``
* ``eSRRF_ST`` -- ``.../_le_esrrf.pyx:21`` (class ``eSRRF``)
* ``calculate_eSRRF_temporal_correlations`` /
  ``calculate_SRRF_temporal_correlations``
  -- ``src/nanopyx/core/transform/sr_temporal_correlations.py:4-75``
* ``macro_pixel_corrector`` -- ``src/nanopyx/core/transform/mpcorrector.pyx:7``

Ownership follows the reference: inputs are never modified; NumPy in gives
NumPy out; a CUDA tensor in gives a CUDA tensor out (computed on the current
stream).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _native as N
from ._device import (DeviceStack, check_image, get_fht_plan, get_plan, require_cuda,
                      stream_ptr, to_device_stack, workspace)
from .liquid import LiquidEngine

__all__ = ["ShiftAndMagnify", "CRShiftAndMagnify", "GradientRobertsCross",
           "RadialGradientConvergence", "Radiality", "eSRRF_ST", "value2array",
           "calculate_eSRRF_temporal_correlations", "calculate_SRRF_temporal_correlations",
           "macro_pixel_corrector", "check_image", "fht_space_interpolation"]


def value2array(v, n_frames: int) -> np.ndarray:
    """Reference ``value2array`` (``__interpolation_tools__.py:30-40``)."""
    if type(v) in (int, float) or np.isscalar(v):
        v = np.ones(n_frames, dtype=np.float32) * np.float32(v)
    return np.asarray(v, dtype=np.float32)


def _ptr(t: torch.Tensor) -> int:
    return t.data_ptr()


def _empty(shape, like: DeviceStack) -> torch.Tensor:
    return torch.empty(shape, dtype=torch.float32, device=like.t.device)


class ShiftAndMagnify(LiquidEngine):
    """Catmull-Rom shift and magnify (``row = i / mag - shift``, pixel-centre taps)."""

    _designation = "ShiftMagnify_catmull_rom"

    def run(self, image, shift_row, shift_col, magnification_row, magnification_col,
            run_type=None):
        return self._run(image, shift_row, shift_col, magnification_row, magnification_col,
                         run_type=run_type)

    def benchmark(self, image, shift_row, shift_col, magnification_row, magnification_col):
        return super().benchmark(image, shift_row, shift_col, magnification_row,
                                 magnification_col)

    def _run_cuda(self, image, shift_row, shift_col, magnification_row, magnification_col):
        img = to_device_stack(image)
        T, H, W = img.shape
        mr = np.float32(magnification_row)
        mc = np.float32(magnification_col)
        rowsM = int(np.float32(H) * mr)
        colsM = int(np.float32(W) * mc)
        sr = torch.from_numpy(value2array(shift_row, T).copy()).to(img.t.device)
        sc = torch.from_numpy(value2array(shift_col, T).copy()).to(img.t.device)
        if sr.numel() != T or sc.numel() != T:
            raise ValueError("shift arrays must have one value per frame")
        out = _empty((T, rowsM, colsM), img)
        N.check(N.lib().nx_cr_shift_magnify(img.ptr(), T, H, W, _ptr(sr), _ptr(sc), float(mr),
                                            float(mc), _ptr(out), stream_ptr()),
                "ShiftAndMagnify")
        return img.out(out)


CRShiftAndMagnify = ShiftAndMagnify


class GradientRobertsCross(LiquidEngine):
    """Roberts-Cross gradients with top/left clamp; returns (gradient_col, gradient_row)."""

    _designation = "GradientRobertsCross"

    def run(self, image, run_type=None):
        return self._run(image, run_type=run_type)

    def benchmark(self, image):
        return super().benchmark(image)

    def _run_cuda(self, image):
        img = to_device_stack(image)
        T, H, W = img.shape
        gc = _empty((T, H, W), img)
        gr = _empty((T, H, W), img)
        N.check(N.lib().nx_roberts_cross(img.ptr(), T, H, W, _ptr(gc), _ptr(gr), stream_ptr()),
                "GradientRobertsCross")
        return img.out(gc), img.out(gr)


class RadialGradientConvergence(LiquidEngine):
    """RGC on 2m-magnified gradients and the m-magnified image."""

    _designation = "RadialGradientConvergence"

    def run(self, gradient_col_interp, gradient_row_interp, image_interp, magnification: int = 5,
            radius: float = 1.5, sensitivity: float = 1, doIntensityWeighting: bool = True,
            pad_edges: bool = False, run_type=None):
        return self._run(gradient_col_interp, gradient_row_interp, image_interp, magnification,
                         radius, sensitivity, doIntensityWeighting, pad_edges=pad_edges,
                         run_type=run_type)

    def benchmark(self, gradient_col_interp, gradient_row_interp, image_interp,
                  magnification: int = 5, radius: float = 1.5, sensitivity: float = 1,
                  doIntensityWeighting: bool = True, pad_edges: bool = False):
        return super().benchmark(gradient_col_interp, gradient_row_interp, image_interp,
                                 magnification, radius, sensitivity, doIntensityWeighting,
                                 pad_edges=pad_edges)

    def _run_cuda(self, gci, gri, image_interp, magnification=5, radius=1.5, sensitivity=1,
                  doIntensityWeighting=True, pad_edges=False):
        gc = to_device_stack(gci)
        gr = to_device_stack(gri)
        im = to_device_stack(image_interp)
        T, rowsM, colsM = im.shape
        if gc.shape != (T, 2 * rowsM, 2 * colsM) or gr.shape != gc.shape:
            raise ValueError("gradient images must be (T, 2*rowsM, 2*colsM) of the magnified image")
        out = _empty((T, rowsM, colsM), im)
        N.check(N.lib().nx_rgc(gc.ptr(), gr.ptr(), im.ptr(), T, rowsM, colsM, int(magnification),
                               float(np.float32(radius)), float(np.float32(sensitivity)),
                               1 if doIntensityWeighting else 0, 1 if pad_edges else 0,
                               _ptr(out), stream_ptr()),
                "RadialGradientConvergence")
        return im.out(out)


class Radiality(LiquidEngine):
    """SRRF radiality over a 12-point ring of radius ringRadius * magnification."""

    _designation = "Radiality"

    def run(self, image, image_interp, magnification: int = 5, ringRadius: float = 0.5,
            border: int = 0, radialityPositivityConstraint: bool = True,
            doIntensityWeighting: bool = True, run_type=None):
        return self._run(image, image_interp, magnification, ringRadius, border,
                         radialityPositivityConstraint, doIntensityWeighting, run_type=run_type)

    def benchmark(self, image, image_interp, magnification: int = 5, ringRadius: float = 0.5,
                  border: int = 0, radialityPositivityConstraint: bool = True,
                  doIntensityWeighting: bool = True):
        return super().benchmark(image, image_interp, magnification, ringRadius, border,
                                 radialityPositivityConstraint, doIntensityWeighting)

    def _run_cuda(self, image, image_interp, magnification=5, ringRadius=0.5, border=0,
                  radialityPositivityConstraint=True, doIntensityWeighting=True):
        img = to_device_stack(image)
        imi = to_device_stack(image_interp)
        T, h, w = img.shape
        m = int(magnification)
        if imi.shape != (T, h * m, w * m):
            raise ValueError("image_interp must be (T, h*m, w*m)")
        out = _empty((T, h * m, w * m), img)
        nb = N.lib().nx_radiality_workspace_bytes(T, h, w)
        ws = workspace(nb, img.t.device)
        N.check(N.lib().nx_radiality(img.ptr(), imi.ptr(), T, h, w, m, float(ringRadius),
                                     int(border), 1 if radialityPositivityConstraint else 0,
                                     1 if doIntensityWeighting else 0, _ptr(out), _ptr(ws),
                                     ws.numel(), stream_ptr()),
                "Radiality")
        return img.out(out)


class eSRRF_ST(LiquidEngine):
    """eSRRF single task: per-frame RGC maps (T, H*m, W*m) from one fused kernel.

    ``use_fht=True`` follows the reference's Fourier path (``_le_esrrf.pyx:
    183-188``): FHT-magnified intensity (x m) and gradients (x 2m), then RGC,
    which honours ``pad_edges``; on the default path ``pad_edges`` has no
    effect, as in the reference (``_le_esrrf.pyx:194`` does not forward it).
    """

    _designation = "eSRRF_ST"

    def run(self, image, magnification: int = 5, radius: float = 1.5, sensitivity: float = 1,
            use_fht: bool = False, doIntensityWeighting: bool = True, pad_edges: bool = False,
            run_type=None):
        return self._run(image, magnification=magnification, radius=radius,
                         sensitivity=sensitivity, use_fht=use_fht,
                         doIntensityWeighting=doIntensityWeighting, pad_edges=pad_edges,
                         run_type=run_type)

    def benchmark(self, image, magnification: int = 5, radius: float = 1.5,
                  sensitivity: float = 1, use_fht: bool = False,
                  doIntensityWeighting: bool = True, pad_edges: bool = False):
        return super().benchmark(image, magnification=magnification, radius=radius,
                                 sensitivity=sensitivity, use_fht=use_fht,
                                 doIntensityWeighting=doIntensityWeighting, pad_edges=pad_edges)

    def _run_cuda(self, image, magnification=5, radius=1.5, sensitivity=1, use_fht=False,
                  doIntensityWeighting=True, pad_edges=False):
        if use_fht:
            img = to_device_stack(image)
            return img.out(_esrrf_st_fht(img.t, int(magnification), radius, sensitivity,
                                         doIntensityWeighting, pad_edges))
        img = to_device_stack(image)
        T, H, W = img.shape
        m = int(magnification)
        plan = get_plan(H, W, m, radius, sensitivity, doIntensityWeighting)
        out = _empty((T, H * m, W * m), img)
        L = N.lib()
        ws = workspace(L.nx_esrrf_st_workspace_bytes(plan.handle, T), img.t.device)
        N.check(L.nx_esrrf_st(plan.handle, img.ptr(), T, _ptr(out), _ptr(ws), ws.numel(),
                              stream_ptr()), "eSRRF_ST")
        N.check(L.nx_workspace_status(_ptr(ws), stream_ptr()), "eSRRF_ST")
        return img.out(out)


def _fht_device(t: torch.Tensor, magnification: int, variant: int = 0) -> torch.Tensor:
    """(T, H, W) CUDA float32 -> (T, H*m, W*m) Fourier interpolation
    (variant 0: interpolation.py, 1: _interpolation.pyx)."""
    T, H, W = t.shape
    m = int(magnification)
    out = torch.empty((T, H * m, W * m), dtype=torch.float32, device=t.device)
    if T == 0:
        return out
    plan = get_fht_plan(H, W, m, variant)
    L = N.lib()
    ws = workspace(L.nx_fht_workspace_bytes(plan.handle, T), t.device)
    N.check(L.nx_fht_interpolate(plan.handle, _ptr(t), T, _ptr(out), _ptr(ws), ws.numel(),
                                 stream_ptr()), "FHT interpolation")
    return out


def fht_space_interpolation(image, magnification: int = 2, doMirrorPadding: bool = True,
                            tile_size: int = 0, overlap: int = 16):
    """Fourier interpolation of a 2-D image or (T, H, W) stack, the reference's
    ``fht_space_interpolation`` (interpolation.py:250-290): mirror padding,
    zero-padded spectrum, rescale onto each frame's [min, max]; frames over 256
    px a side in Hann-blended 256-pixel tiles.  NumPy in -> NumPy out, CUDA
    tensor in -> CUDA tensor out."""
    if not doMirrorPadding or int(tile_size) not in (0, 256) or int(overlap) != 16:
        raise NotImplementedError("the Fourier interpolation supports the default mirror "
                                  "padding, 256-pixel tiles and 16-pixel overlap")
    if isinstance(image, torch.Tensor):
        t = image.to(torch.float32)
        on_dev = t.is_cuda
        t = t.to(require_cuda()).contiguous()
    else:
        t = torch.from_numpy(np.ascontiguousarray(np.asarray(image, dtype=np.float32))).to(
            require_cuda())
        on_dev = False
    if t.ndim not in (2, 3):
        raise ValueError("Input must be 2-D or 3-D array")
    out = _fht_device(t[None] if t.ndim == 2 else t, int(magnification))
    if t.ndim == 2:
        out = out[0]
    return out if on_dev else out.cpu().numpy()


def _esrrf_st_fht(x: torch.Tensor, m: int, radius, sensitivity, iw, pad_edges) -> torch.Tensor:
    """eSRRF_ST on the Fourier path, in frame chunks that keep the 2m-magnified
    gradients (2 x 4 m^2 H W floats per frame) near 2 GB."""
    T, H, W = x.shape
    out = torch.empty((T, H * m, W * m), dtype=torch.float32, device=x.device)
    per_frame = 4 * (8 * m * m + 4) * H * W
    chunk = max(1, min(T, (2 << 30) // max(per_frame, 1)))
    L = N.lib()
    s = stream_ptr()
    for a in range(0, T, chunk):
        xb = x[a:a + chunk].contiguous()
        n = xb.shape[0]
        mag = _fht_device(xb, m)
        gc = torch.empty_like(xb)
        gr = torch.empty_like(xb)
        N.check(L.nx_roberts_cross(_ptr(xb), n, H, W, _ptr(gc), _ptr(gr), s), "Roberts-Cross")
        gci = _fht_device(gc, 2 * m)
        gri = _fht_device(gr, 2 * m)
        N.check(L.nx_rgc(_ptr(gci), _ptr(gri), _ptr(mag), n, H * m, W * m, m, float(radius),
                         float(sensitivity), 1 if iw else 0, 1 if pad_edges else 0,
                         _ptr(out[a:a + n]), s), "RadialGradientConvergence")
    return out


# ---------------------------------------------------------------------------
# temporal correlations
# ---------------------------------------------------------------------------
def _stack3(im) -> DeviceStack:
    if isinstance(im, torch.Tensor):
        t = im.to(torch.float32)
        if t.ndim != 3:
            raise AssertionError("input must be a 3-D (T, H, W) stack")
        return DeviceStack(t.contiguous().to(require_cuda()) if not t.is_cuda else t.contiguous(),
                           not t.is_cuda)
    a = np.array(im, dtype="float32")
    if a.ndim != 3:
        raise AssertionError("input must be a 3-D (T, H, W) stack")
    return DeviceStack(torch.from_numpy(np.ascontiguousarray(a)).to(require_cuda()), True)


def calculate_eSRRF_temporal_correlations(im, correlation: str):
    """AVG / VAR / TAC2 over axis 0 (numpy float32 order)."""
    if correlation not in N.CORR_BITS:
        raise ValueError("Type of correlation must be AVG, VAR or TAC2")
    st = _stack3(im)
    T = st.shape[0]
    out = torch.empty(st.shape[1:], dtype=torch.float32, device=st.t.device)
    N.check(N.lib().nx_temporal_correlation(st.ptr(), T, out.numel(), N.CORR_BITS[correlation],
                                            _ptr(out), stream_ptr()),
            "temporal correlation")
    return st.out(out)


def calculate_SRRF_temporal_correlations(im, order: int = 1, do_integrate_lag_times: bool = 0):
    """Orders 0 (max), 1 (mean), -1 (pairwise product sum), 2/3/4 (ACRF, with
    or without lag-time integration; the flag only applies to orders 2-4, as in
    sr_temporal_correlations.py:31-41,111-202).  Raises IndexError at the frame
    counts where the reference's lag-time binning indexes past its input."""
    st = _stack3(im)
    assert order <= 4
    if order < -1:
        raise ValueError("order must be -1, 0, 1, 2, 3 or 4")
    T = st.shape[0]
    out = torch.empty(st.shape[1:], dtype=torch.float32, device=st.t.device)
    L = N.lib()
    if do_integrate_lag_times == 1 and order >= 2:
        ws = workspace(L.nx_srrf_acrf_workspace_bytes(T, out.numel()), st.t.device)
        N.check(L.nx_srrf_acrf_integrated(st.ptr(), T, out.numel(), int(order), _ptr(out),
                                          _ptr(ws), ws.numel(), stream_ptr()),
                "ACRF with lag-time integration")
        return st.out(out)
    N.check(L.nx_srrf_temporal_correlation(st.ptr(), T, out.numel(), int(order), _ptr(out),
                                           stream_ptr()),
            "SRRF temporal correlation")
    return st.out(out)


def macro_pixel_corrector(img, magnification: int):
    """Per-slice macro-pixel correction; returns a corrected float32 copy."""
    if isinstance(img, torch.Tensor):
        t = img.to(torch.float32)
        src_np = not t.is_cuda
        t = t.to(require_cuda()).contiguous().clone()
    else:
        a = np.asarray(img).astype(np.float32)
        src_np = True
        t = torch.from_numpy(np.ascontiguousarray(a)).to(require_cuda())
    if t.ndim != 3:
        raise ValueError("Buffer has wrong number of dimensions (expected 3)")
    S, rowsM, colsM = t.shape
    m = int(magnification)
    ws = workspace(N.lib().nx_macro_pixel_workspace_bytes(S, m), t.device)
    N.check(N.lib().nx_macro_pixel_correct(_ptr(t), S, rowsM, colsM, m, _ptr(ws), ws.numel(),
                                           stream_ptr()),
            "macro_pixel_corrector")
    return t.cpu().numpy() if src_np else t


class eSRRF3D_ST(LiquidEngine):
    """eSRRF-3D single task (``_le_esrrf3d.pyx:26-140``): a (T, S, H, W) stack
    (or one (S, H, W) volume) -> (S*mz, H*mxy, W*mxy), the frames' RGC-3D
    mean (``mode="average"``) or standard deviation (``mode="std"``).  Like the
    reference, an oversized radius prints a warning and returns None."""

    _designation = "eSRRF_3D"

    def run(self, image, magnification_xy: int = 2, magnification_z: int = 2,
            radius: float = 1.5, PSF_ratio: float = 2.8, voxel_ratio: float = 4.0,
            sensitivity: float = 1, mode: str = "average", doIntensityWeighting: bool = True,
            run_type=None):
        radius_z = radius * PSF_ratio / voxel_ratio
        shape = tuple(image.shape)
        if len(shape) == 3:
            shape = (1,) + shape
        if len(shape) != 4:
            print("Warning:image must either be 3D or 4D. If 3D, it will be reshaped to 4D.")
            return None
        if radius > shape[2] / 2 or radius * 2 > shape[3] / 2:
            print("Warning: Radius is too big for the image. The radius must be smaller than "
                  "half the number of columns and half number of rows of the image.")
            return None
        if radius_z > shape[1] / 2:
            print("Warning: Radius_z is too big for the image. The radius_z must be smaller "
                  "than half of number of Z planes. Radius_z is automatically calculated from "
                  "radius * PSF_ratio / voxel_ratio.")
            return None
        if mode not in ("average", "std"):
            raise ValueError("mode must be 'average' or 'std'")
        return self._run(image, magnification_xy=magnification_xy,
                         magnification_z=magnification_z, radius=radius, radius_z=radius_z,
                         sensitivity=sensitivity, mode=mode,
                         doIntensityWeighting=doIntensityWeighting, run_type=run_type)

    def _run_cuda(self, image, magnification_xy=2, magnification_z=2, radius=1.5, radius_z=1.05,
                  sensitivity=1, mode="average", doIntensityWeighting=True):
        if isinstance(image, torch.Tensor):
            t = image.to(torch.float32)
            from_np = not t.is_cuda
            t = t.to(require_cuda()).contiguous()
        else:
            t = torch.from_numpy(np.ascontiguousarray(np.asarray(image, dtype=np.float32))).to(
                require_cuda())
            from_np = True
        if t.ndim == 3:
            t = t[None]
        T, S, H, W = t.shape
        mxy, mz = int(magnification_xy), int(magnification_z)
        out = torch.empty((S * mz, H * mxy, W * mxy), dtype=torch.float32, device=t.device)
        md = 1 if mode == "std" else 0
        L = N.lib()
        ws = workspace(L.nx_esrrf3d_workspace_bytes(S, H, W, mxy, mz, md), t.device)
        N.check(L.nx_esrrf3d_st(_ptr(t), T, S, H, W, mxy, mz, float(radius), float(radius_z),
                                float(sensitivity), md, 1 if doIntensityWeighting else 0,
                                _ptr(out), _ptr(ws), ws.numel(), stream_ptr()), "eSRRF3D")
        return out.cpu().numpy() if from_np else out
