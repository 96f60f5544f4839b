"""Parity at the benchmarked configurations against the compiled reference.

* Large single eSRRF (the benchmark's workload, shortened in time): 108 frames
  x 512 x 512 from the 400-emitter blinking generator, magnification 5,
  radius 1.5, sensitivity 2, VAR and TAC2, 100 frames per timepoint (one full
  timepoint and a short 8-frame tail), macro-pixel correction on.
* Parameter sweep: 16 frames x 256 x 256 at 150 emitters, magnification 4,
  radius {1, 1.5, 2, 2.5} x sensitivity {1, 2, 3, 4}, AVG -- the reference runs
  one full eSRRF_ST per pair (core/analysis/parameter_sweep.py:33-40).

Bar: max |got - ref| / (max(ref) - min(ref)) <= 1e-4 against the reference.
Beside it each test prints the error of both sides against the FP64 oracle's
temporal step and macro-pixel correction applied to the reference's own
per-frame maps (the per-frame maps themselves are pinned to the FP64 oracle by
the golden and odd-size tests).
"""
import numpy as np
import pytest
import torch

import nanopyx_gb300 as nx
import reference_runs as RR
from conftest import rel_err
from nanopyx_gb300 import _native
from nanopyx_gb300.synthetic import blinking_stack

pytestmark = pytest.mark.gpu
TOL = 1e-4


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    _native.lib()
    yield
    torch.cuda.synchronize()


def test_large_single_esrrf_against_reference():
    T, H, W, m, r, s, fpt = 108, 512, 512, 5, 1.5, 2.0, 100
    x = blinking_stack(T, H, W, 400, seed=1)
    var, tac = nx.eSRRF(x, magnification=m, radius=r, sensitivity=s, frames_per_timepoint=fpt,
                        temporal_correlation=("VAR", "TAC2"), macro_pixel_correction=True)
    assert var.shape == tac.shape == (2, H * m, W * m)
    R = RR.load()
    st = RR.esrrf_st(R, x, m, r, s)
    for name, got in (("VAR", var), ("TAC2", tac)):
        ref = RR.esrrf_from_maps(R, st, m, fpt, name, True)
        f64 = RR.fp64_from_maps(st, m, fpt, name, True)
        for tp in range(2):
            e_ref = rel_err(got[tp], ref[tp])
            print(f"\n{name} timepoint {tp}: gpu vs reference {e_ref:.2e}; "
                  f"gpu vs FP64 {rel_err(got[tp], f64[tp]):.2e}; "
                  f"reference vs FP64 {rel_err(ref[tp], f64[tp]):.2e}")
            assert e_ref <= TOL, (name, tp, e_ref)


def test_parameter_sweep_grid_against_reference():
    x = blinking_stack(16, 256, 256, 150, seed=2)
    sens, radii, m = [1, 2, 3, 4], [1.0, 1.5, 2.0, 2.5], 4
    grid = nx.esrrf_parameter_sweep(x, magnification=m, sensitivities=sens, radii=radii)
    assert grid.shape == (4, 4, 1024, 1024)
    R = RR.load()
    worst = 0.0
    for i, s in enumerate(sens):
        for j, r in enumerate(radii):
            st = RR.esrrf_st(R, x, m, r, s, block=16)
            ref = RR.esrrf_from_maps(R, st, m, 0, "AVG", False)[0]
            f64 = RR.fp64_from_maps(st, m, 0, "AVG", False)[0]
            e = rel_err(grid[i, j], ref)
            worst = max(worst, e)
            print(f"\ns={s} R={r}: gpu vs reference {e:.2e}; gpu vs FP64 "
                  f"{rel_err(grid[i, j], f64):.2e}; reference vs FP64 {rel_err(ref, f64):.2e}")
            assert e <= TOL, (s, r, e)
