"""Liquid-Engine-shaped base class of the ops.

Mirrors the protocol the reference's op classes follow (third-party
``liquid_engine.LiquidEngine``, used at e.g.
``src/nanopyx/core/transform/_le_esrrf.pyx:21-37``): a class sets
``_designation``, exposes ``run(...)`` and ``benchmark(...)``, and records
``_last_runtype`` / ``_last_time``.  Here there is exactly one implementation of
every op -- the sm_103a CUDA path -- so ``run_type`` is accepted for call
compatibility and always resolves to ``"CUDA"``; no other backend exists to
dispatch to.
"""
from __future__ import annotations

import time

import torch

RUN_TYPE = "CUDA"


class LiquidEngine:
    _designation = "LiquidEngine"

    def __init__(self, clear_benchmarks: bool = False, testing: bool = False,
                 verbose: bool = True, **kwargs):
        self.testing = testing
        self.verbose = verbose
        self._last_runtype = None
        self._last_time = None
        self._run_types = {RUN_TYPE: self._run_cuda}

    def _run_cuda(self, *args, **kwargs):  # pragma: no cover - abstract
        raise NotImplementedError

    def _run(self, *args, run_type=None, **kwargs):
        t0 = time.perf_counter()
        out = self._run_cuda(*args, **kwargs)
        self._last_time = time.perf_counter() - t0
        self._last_runtype = RUN_TYPE
        return out

    def benchmark(self, *args, **kwargs):
        """``[[seconds, run_type_name, output], ...]`` (one run type: CUDA)."""
        self._run(*args, **kwargs)  # warm-up (plans, first-touch)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = self._run(*args, **kwargs)
        torch.cuda.synchronize()
        return [[time.perf_counter() - t0, RUN_TYPE, out]]
