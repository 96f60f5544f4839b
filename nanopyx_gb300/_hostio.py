"""Host-side staging for calls with NumPy buffers.

Pageable NumPy memory is copied into pinned buffers by a small pool of host
threads (NumPy releases the GIL for large copies), so the host->device and
device->host DMA run asynchronously on a copy stream at full link speed and
overlap the kernels.  Pinned buffers come from PyTorch's caching host
allocator, so repeated calls reuse them.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import threading

import numpy as np
import torch

_POOL = None
_WORKERS = 1
_LOCK = threading.Lock()
_MIN_PART = 1 << 21  # bytes per copy task


def _pool() -> cf.ThreadPoolExecutor:
    global _POOL, _WORKERS
    with _LOCK:
        if _POOL is None:
            _WORKERS = int(os.environ.get("NANOPYX_GB300_HOST_THREADS", "0")) or \
                max(1, min(8, (os.cpu_count() or 2) // 2))
            _POOL = cf.ThreadPoolExecutor(max_workers=_WORKERS, thread_name_prefix="nx-hostio")
        return _POOL


def _slices(shape, parts):
    """Index tuples that cover an array of `shape` in about `parts` pieces."""
    if len(shape) >= 2 and shape[0] < parts:
        per = -(-parts // shape[0])
        sub = np.linspace(0, shape[1], min(per, shape[1]) + 1).astype(int)
        return [(i, slice(a, b)) for i in range(shape[0])
                for a, b in zip(sub[:-1], sub[1:]) if b > a]
    cut = np.linspace(0, shape[0], min(parts, shape[0]) + 1).astype(int)
    return [(slice(a, b),) for a, b in zip(cut[:-1], cut[1:]) if b > a]


def par_copy(dst: np.ndarray, src: np.ndarray) -> None:
    """dst[...] = src with the work split over the host copy threads (any strides)."""
    if dst.shape != src.shape:
        raise ValueError(f"shape mismatch {dst.shape} vs {src.shape}")
    pool = _pool()
    parts = int(max(1, min(_WORKERS * 2, dst.nbytes // _MIN_PART)))
    if parts == 1 or dst.ndim == 0:
        np.copyto(dst, src)
        return
    futs = [pool.submit(np.copyto, dst[idx], src[idx]) for idx in _slices(dst.shape, parts)]
    for f in futs:
        f.result()


def pinned(shape, dtype=torch.float32) -> torch.Tensor:
    """A page-locked host tensor (from the caching host allocator)."""
    return torch.empty(shape, dtype=dtype, pin_memory=True)
