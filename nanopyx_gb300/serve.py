"""Serving: continuous-batching eSRRF reconstructions of streamed frame blocks.

A request is one reconstruction (H x W frames, magnification, radius,
sensitivity, correlations) whose frames arrive in blocks.  ``ESRRFServer``
runs a dispatcher thread that

* admits waiting requests in arrival order while their device memory -- the
  per-pixel temporal accumulator, one block of input, the push workspace and
  the output -- fits in an HBM budget (and a cap on concurrent requests);
* folds every block into its request's device-resident accumulator as soon as
  it arrives (``nx_esrrf_accum_push``), each request on its own CUDA stream, so
  the work of requests that are admitted together overlaps on the device and a
  request that arrives while others run starts as soon as memory frees up;
* finalises a request after its last block (temporal correlation + macro-pixel
  correction on the device) and copies the result back asynchronously.

Two latencies are kept per request: from the arrival of its last block to its
result being on the host (``latency``), and from the arrival of its first
block (``first_latency``).  ``serve_plain`` is the plain per-request path the server is
compared with: one request at a time, every call synchronous.

There is no reference counterpart: NanoPyx keeps a whole per-frame stack in
host RAM and reconstructs one stack per call (``eSRRF_workflow.py:76-112``).
"""
from __future__ import annotations

import collections
import threading
import time

import numpy as np
import torch

from . import _native as N
from ._device import get_plan, require_cuda, workspace

__all__ = ["ESRRFServer", "Request", "serve_plain"]


class Request:
    """One streamed reconstruction; ``result()`` blocks until it is done."""

    def __init__(self, rid, H, W, n_blocks, magnification, radius, sensitivity,
                 temporal_correlation, macro_pixel_correction, doIntensityWeighting):
        self.id = rid
        self.H, self.W, self.n_blocks = int(H), int(W), int(n_blocks)
        self.m = int(magnification)
        self.radius, self.sensitivity = float(radius), float(sensitivity)
        self.names = [temporal_correlation] if isinstance(temporal_correlation, str) \
            else list(temporal_correlation)
        if not self.names or any(n not in N.CORR_BITS for n in self.names):
            raise ValueError("Type of correlation must be AVG, VAR or TAC2")
        self.mask = 0
        for n in self.names:
            self.mask |= N.CORR_BITS[n]
        self.order = [b for b in ("AVG", "VAR", "TAC2") if self.mask & N.CORR_BITS[b]]
        self.mpc = bool(macro_pixel_correction)
        self.iw = bool(doIntensityWeighting)
        self.single = isinstance(temporal_correlation, str)
        self.t_submit = time.perf_counter()
        self.t_first_block = None
        self.t_last_block = None
        self.t_done = None
        self.host_blocks = collections.deque()
        self.blocks_received = 0
        self.blocks_pushed = 0
        self.frames = 0
        self.mpx_frames = 0.0
        self._done = threading.Event()
        self._result = None
        self.error = None
        # device state (dispatcher thread only)
        self.stream = None
        self.plan = None
        self.acc = None
        self.ws = None
        self.fin_ws = None
        self.out = None
        self.host_out = None
        self.event = None
        self.reserved = 0

    @property
    def latency(self):
        """Seconds from the arrival of the last block to the result on the host."""
        return None if self.t_done is None else self.t_done - self.t_last_block

    @property
    def first_latency(self):
        """Seconds from the arrival of the first block to the result on the host."""
        return None if self.t_done is None else self.t_done - self.t_first_block

    def result(self, timeout=None):
        if not self._done.wait(timeout):
            raise TimeoutError(f"request {self.id} not finished")
        if self.error is not None:
            raise self.error
        return self._result


def _bytes_needed(H, W, m, T_block, n_out):
    planeM = H * m * W * m
    return 4 * (5 * planeM * 2 + n_out * planeM + T_block * H * W) + (1 << 20)


class ESRRFServer:
    """Continuous-batching request loop (see module doc).

    ``hbm_budget``: bytes of device memory the server may hold for requests
    (default: half of the free memory at start); ``max_active``: cap on
    concurrently admitted requests; ``n_streams``: CUDA streams requests are
    spread over.
    """

    def __init__(self, hbm_budget: int | None = None, max_active: int = 32, n_streams: int = 8,
                 device=None):
        self.device = device if device is not None else require_cuda()
        if hbm_budget is None:
            free, _ = torch.cuda.mem_get_info(self.device)
            hbm_budget = free // 2
        self.budget = int(hbm_budget)
        self.used = 0
        self.max_active = int(max_active)
        self.streams = [torch.cuda.Stream(self.device) for _ in range(max(1, n_streams))]
        self._next_stream = 0
        self._lock = threading.Condition()
        self._waiting = collections.deque()
        self._active = []
        self._finishing = []
        self._closing = False
        self._ids = 0
        self.admitted_max = 0
        self._thread = threading.Thread(target=self._loop, name="esrrf-server", daemon=True)
        self._thread.start()

    # -- client side --------------------------------------------------------
    def submit(self, H, W, n_blocks, magnification=5, radius=1.5, sensitivity=1,
               temporal_correlation="AVG", macro_pixel_correction=True,
               doIntensityWeighting=True) -> Request:
        with self._lock:
            if self._closing:
                raise RuntimeError("server is closed")
            self._ids += 1
            r = Request(self._ids, H, W, n_blocks, magnification, radius, sensitivity,
                        temporal_correlation, macro_pixel_correction, doIntensityWeighting)
            self._waiting.append(r)
            self._lock.notify()
            return r

    def push(self, req: Request, block) -> None:
        """Deliver the next (T_block, H, W) block of ``req`` (NumPy, float32)."""
        a = np.ascontiguousarray(block, dtype=np.float32)
        if a.ndim == 2:
            a = a[None]
        if a.shape[1:] != (req.H, req.W):
            raise ValueError("block frame size does not match the request")
        with self._lock:
            if req.blocks_received >= req.n_blocks:
                raise ValueError("request already received all its blocks")
            req.host_blocks.append(a)
            if req.blocks_received == 0:
                req.t_first_block = time.perf_counter()
            req.blocks_received += 1
            req.mpx_frames += a.shape[0] * req.H * req.W / 1e6
            if req.blocks_received == req.n_blocks:
                req.t_last_block = time.perf_counter()
            self._lock.notify()

    def close(self, wait: bool = True):
        with self._lock:
            self._closing = True
            self._lock.notify()
        if wait:
            self._thread.join()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- dispatcher -----------------------------------------------------------
    def _admit(self):
        while self._waiting and len(self._active) < self.max_active:
            r = self._waiting[0]
            if not r.host_blocks:
                break  # admit when its first block is here (FIFO)
            T_block = r.host_blocks[0].shape[0]
            need = _bytes_needed(r.H, r.W, r.m, T_block, len(r.order))
            if (self._active or self._finishing) and self.used + need > self.budget:
                break  # a request alone may exceed the budget; others wait for memory
            self._waiting.popleft()
            r.reserved = need
            self.used += need
            r.stream = self.streams[self._next_stream % len(self.streams)]
            self._next_stream += 1
            try:
                with torch.cuda.stream(r.stream):
                    L = N.lib()
                    r.plan = get_plan(r.H, r.W, r.m, r.radius, r.sensitivity, r.iw)
                    r.acc = torch.empty(L.nx_esrrf_accum_bytes(r.plan.handle), dtype=torch.uint8,
                                        device=self.device)
                    r.ws = workspace(L.nx_esrrf_push_workspace_bytes(r.plan.handle, T_block),
                                     self.device)
                    r.fin_ws = workspace(256 + L.nx_macro_pixel_workspace_bytes(3, r.m),
                                         self.device)
                    r.out = torch.empty((len(r.order), r.H * r.m, r.W * r.m), dtype=torch.float32,
                                        device=self.device)
                    r.host_out = torch.empty(tuple(r.out.shape), dtype=torch.float32,
                                             pin_memory=True)
            except Exception as e:  # allocation failure: fail this request only
                self._fail(r, e)
                continue
            self._active.append(r)
            self.admitted_max = max(self.admitted_max, len(self._active))

    def _fail(self, r, e):
        r.error = e if isinstance(e, Exception) else RuntimeError(str(e))
        self.used -= r.reserved
        r.reserved = 0
        r.acc = r.ws = r.out = r.fin_ws = None
        r._done.set()

    def _dispatch(self, r):
        L = N.lib()
        while r.host_blocks:
            blk = r.host_blocks.popleft()
            with torch.cuda.stream(r.stream):
                x = torch.from_numpy(blk).to(self.device, non_blocking=True)
                if r.ws.numel() < L.nx_esrrf_push_workspace_bytes(r.plan.handle, blk.shape[0]):
                    r.ws = workspace(L.nx_esrrf_push_workspace_bytes(r.plan.handle, blk.shape[0]),
                                     self.device)
                N.check(L.nx_esrrf_accum_push(r.plan.handle, x.data_ptr(), blk.shape[0], r.frames,
                                              r.acc.data_ptr(), r.ws.data_ptr(), r.ws.numel(),
                                              r.stream.cuda_stream), "eSRRF push")
            # x was allocated on r.stream: the caching allocator reuses its memory
            # only for later work on that stream, after this push
            del x
            r.frames += blk.shape[0]
            r.blocks_pushed += 1
        if r.blocks_pushed == r.n_blocks:
            with torch.cuda.stream(r.stream):
                N.check(L.nx_esrrf_accum_finalize(r.plan.handle, r.acc.data_ptr(), r.frames,
                                                  r.mask, 1 if r.mpc else 0, r.out.data_ptr(),
                                                  r.fin_ws.data_ptr(), r.fin_ws.numel(),
                                                  r.stream.cuda_stream), "eSRRF finalize")
                r.host_out.copy_(r.out, non_blocking=True)
                r.event = r.stream.record_event()
            return True
        return False

    def _complete(self, r):
        st = N.lib().nx_workspace_status(r.ws.data_ptr(), r.stream.cuda_stream)
        r.t_done = time.perf_counter()
        res = r.host_out.numpy()
        res = res[[r.order.index(n) for n in r.names]].copy()
        r._result = res[0] if r.single else tuple(res)
        if st != N.NX_OK:
            try:
                N.check(st, f"request {r.id}")
            except Exception as e:
                r.error = e
        self.used -= r.reserved
        r.reserved = 0
        r.acc = r.ws = r.out = r.fin_ws = r.host_out = None
        r._done.set()

    def _loop(self):
        torch.cuda.set_device(self.device)
        while True:
            with self._lock:
                self._admit()
                work = [r for r in self._active if r.host_blocks]
                idle = not work and not self._finishing
                if idle and not self._waiting and not self._active and self._closing:
                    return
                if idle:
                    self._lock.wait(timeout=0.0005)
                    continue
            for r in work:
                try:
                    if self._dispatch(r):
                        with self._lock:
                            self._active.remove(r)
                            self._finishing.append(r)
                except Exception as e:
                    with self._lock:
                        if r in self._active:
                            self._active.remove(r)
                        self._fail(r, e)
            done = [r for r in self._finishing if r.event.query()]
            for r in done:
                self._finishing.remove(r)
                with self._lock:
                    self._complete(r)
            if not work and self._finishing and not done:
                time.sleep(0.0002)


def serve_plain(requests_blocks, params, device=None):
    """Plain per-request path: each request alone, every call synchronous.

    ``requests_blocks``: list of lists of (T_block, H, W) blocks; ``params``:
    list of keyword dicts (as ``ESRRFServer.submit``).  Returns the results.
    """
    dev = device if device is not None else require_cuda()
    L = N.lib()
    outs = []
    for blocks, kw in zip(requests_blocks, params):
        H, W = blocks[0].shape[1:]
        m = int(kw.get("magnification", 5))
        names = kw.get("temporal_correlation", "AVG")
        single = isinstance(names, str)
        names = [names] if single else list(names)
        mask = 0
        for n in names:
            mask |= N.CORR_BITS[n]
        order = [b for b in ("AVG", "VAR", "TAC2") if mask & N.CORR_BITS[b]]
        plan = get_plan(H, W, m, kw.get("radius", 1.5), kw.get("sensitivity", 1),
                        kw.get("doIntensityWeighting", True))
        acc = torch.empty(L.nx_esrrf_accum_bytes(plan.handle), dtype=torch.uint8, device=dev)
        frames = 0
        s = torch.cuda.current_stream(dev).cuda_stream
        for blk in blocks:
            x = torch.from_numpy(np.ascontiguousarray(blk, dtype=np.float32)).to(dev)
            ws = workspace(L.nx_esrrf_push_workspace_bytes(plan.handle, x.shape[0]), dev)
            N.check(L.nx_esrrf_accum_push(plan.handle, x.data_ptr(), x.shape[0], frames,
                                          acc.data_ptr(), ws.data_ptr(), ws.numel(), s))
            torch.cuda.synchronize(dev)
            frames += x.shape[0]
        out = torch.empty((len(order), H * m, W * m), dtype=torch.float32, device=dev)
        fws = workspace(256 + L.nx_macro_pixel_workspace_bytes(3, m), dev)
        N.check(L.nx_esrrf_accum_finalize(plan.handle, acc.data_ptr(), frames, mask,
                                          1 if kw.get("macro_pixel_correction", True) else 0,
                                          out.data_ptr(), fws.data_ptr(), fws.numel(), s))
        res = out.cpu().numpy()[[order.index(n) for n in names]]
        outs.append(res[0] if single else tuple(res))
    return outs
