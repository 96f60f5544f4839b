"""Device plumbing: input normalisation, streams, workspaces and plan cache.

PyTorch is used only for device memory (its caching allocator), streams and
host<->device copies; every computation goes through the native library.
"""
from __future__ import annotations

import collections
import ctypes as C
import threading

import numpy as np
import torch

from . import _native as N

__all__ = ["check_image", "DeviceStack", "to_device_stack", "stream_ptr", "workspace",
           "get_plan", "require_cuda"]


def require_cuda() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("nanopyx_gb300 needs a CUDA device (sm_103a); there is no CPU path")
    N.lib()
    return torch.device("cuda", torch.cuda.current_device())


def check_image(image):
    """Reference ``check_image`` (``core/transform/__interpolation_tools__.py:4-27``).

    NumPy in: ``np.asarray``, 2-D or 3-D, cast to float32, 2-D -> (1, H, W).
    Torch tensors are accepted too (kept on their device, cast to float32).
    """
    if isinstance(image, torch.Tensor):
        if image.ndim not in (2, 3):
            raise ValueError("Image must be 2D and 3D (sequence of 2D images)")
        if image.dtype != torch.float32:
            image = image.to(torch.float32)
        if image.ndim == 2:
            image = image.reshape(1, image.shape[0], image.shape[1])
        return image
    image = np.asarray(image)
    if type(image) is not np.ndarray:
        raise TypeError("Image must be of type np.ndarray")
    if image.ndim != 2 and image.ndim != 3:
        raise ValueError("Image must be 2D and 3D (sequence of 2D images)")
    if image.dtype != np.float32:
        image = image.astype(np.float32, copy=False)
    if image.ndim == 2:
        image = image.reshape((1, image.shape[0], image.shape[1]))
    return image


class DeviceStack:
    """A (T, H, W) float32 C-contiguous CUDA tensor plus where it came from."""

    __slots__ = ("t", "from_numpy")

    def __init__(self, t: torch.Tensor, from_numpy: bool):
        self.t = t
        self.from_numpy = from_numpy

    @property
    def shape(self):
        return tuple(self.t.shape)

    def ptr(self) -> int:
        return self.t.data_ptr()

    def out(self, t: torch.Tensor):
        """Return a result in the caller's flavour (NumPy in -> NumPy out)."""
        if self.from_numpy:
            return t.cpu().numpy()
        return t


def to_device_stack(image) -> DeviceStack:
    dev = require_cuda()
    img = check_image(image)
    if isinstance(img, torch.Tensor):
        if not img.is_cuda:
            return DeviceStack(img.contiguous().to(dev), True)
        return DeviceStack(img.contiguous(), False)
    arr = np.ascontiguousarray(img)
    return DeviceStack(torch.from_numpy(arr).to(dev), True)


def stream_ptr(device=None) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def workspace(nbytes: int, device=None) -> torch.Tensor:
    """Device scratch for one C-ABI call; its first 256 bytes (the device status
    word the kernels report bounded-wait timeouts into) start at zero."""
    device = device if device is not None else torch.device("cuda", torch.cuda.current_device())
    ws = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)
    ws[:256].zero_()
    return ws


class _Plan:
    __slots__ = ("handle", "key")

    def __init__(self, key):
        self.key = key
        h = C.c_void_p()
        _, H, W, m, R, s, iw = key
        N.check(N.lib().nx_esrrf_plan_create(C.byref(h), H, W, m, R, s, iw), "eSRRF plan")
        self.handle = h

    def __del__(self):
        try:
            if self.handle:
                N.lib().nx_esrrf_plan_destroy(self.handle)
        except Exception:
            pass


_plans: "collections.OrderedDict" = collections.OrderedDict()
_plans_lock = threading.Lock()
_PLAN_CACHE = 64


def get_plan(H: int, W: int, magnification: int, radius: float, sensitivity: float,
             intensity_weighting: bool) -> _Plan:
    """Cached per-device eSRRF plan (FP64-derived weight tables on the device)."""
    require_cuda()
    key = (torch.cuda.current_device(), int(H), int(W), int(magnification),
           float(np.float32(radius)), float(np.float32(sensitivity)), 1 if intensity_weighting else 0)
    with _plans_lock:
        p = _plans.get(key)
        if p is None:
            p = _Plan(key)
            _plans[key] = p
            while len(_plans) > _PLAN_CACHE:
                _plans.popitem(last=False)
        else:
            _plans.move_to_end(key)
        return p


class _FhtPlan:
    __slots__ = ("handle", "key")

    def __init__(self, key):
        self.key = key
        h = C.c_void_p()
        _, H, W, m, variant = key
        N.check(N.lib().nx_fht_plan_create_ex(C.byref(h), H, W, m, variant), "FHT plan")
        self.handle = h

    def __del__(self):
        try:
            if self.handle:
                N.lib().nx_fht_plan_destroy(self.handle)
        except Exception:
            pass


_fht_plans: "collections.OrderedDict" = collections.OrderedDict()


FHT_TILED, FHT_FULL_SPECTRUM = 0, 1


def get_fht_plan(H: int, W: int, magnification: int, variant: int = FHT_TILED) -> _FhtPlan:
    """Cached per-device Fourier-interpolation plan (tile layout, float64-derived
    operators and blending weights on the device).  ``variant``: FHT_TILED
    (interpolation.py, the use_fht path) or FHT_FULL_SPECTRUM
    (_interpolation.pyx, ErrorMap's reference interpolation)."""
    require_cuda()
    key = (torch.cuda.current_device(), int(H), int(W), int(magnification), int(variant))
    with _plans_lock:
        p = _fht_plans.get(key)
        if p is None:
            p = _FhtPlan(key)
            _fht_plans[key] = p
            while len(_fht_plans) > 16:
                _fht_plans.popitem(last=False)
        else:
            _fht_plans.move_to_end(key)
        return p
