"""Failure detection without a GPU fault.

A device wait that can never be satisfied (an mbarrier nothing arrives on)
must end by itself after its bound, record the time-out in the workspace
status word, and leave the context usable: the host sees DeviceTimeoutError
and the next computation still runs and is correct.
"""
import numpy as np
import pytest
import torch

import nanopyx_gb300 as nx
from nanopyx_gb300 import _native
from nanopyx_gb300._device import workspace

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_reports_status():
    L = _native.lib()
    s = torch.cuda.current_stream().cuda_stream
    ws = workspace(256)
    assert L.nx_selftest_wait_timeout(ws.data_ptr(), ws.numel(), 20_000_000, s) == _native.NX_OK
    rc = L.nx_workspace_status(ws.data_ptr(), s)
    assert rc == _native.NX_ERR_DEVICE_TIMEOUT
    with pytest.raises(_native.DeviceTimeoutError):
        _native.check(rc, "self-test")
    # the context is still usable and results are still right
    x = np.random.default_rng(0).random((3, 16, 16)).astype(np.float32)
    out = nx.calculate_eSRRF_temporal_correlations(x, "AVG")
    assert np.allclose(out, x.mean(axis=0), rtol=1e-6)
    # a clean status word reads OK again
    ws.zero_()
    assert L.nx_workspace_status(ws.data_ptr(), s) == _native.NX_OK


def test_selftest_refuses_long_waits_and_missing_workspace():
    L = _native.lib()
    s = torch.cuda.current_stream().cuda_stream
    ws = workspace(256)
    assert L.nx_selftest_wait_timeout(ws.data_ptr(), ws.numel(), 5_000_000_000, s) == \
        _native.NX_ERR_INVALID_ARG
    assert L.nx_selftest_wait_timeout(None, 0, 1000, s) == _native.NX_ERR_WORKSPACE


def test_fused_kernel_abort_path_reports_timeout_and_context_stays_usable():
    """The fused eSRRF kernel's own bounded waits: with its producers withholding
    one `full` arrival, the consumers' 20 ms wait runs out, the CTA's abort flag
    ends every other wait, in-flight TMA copies are drained and the kernel
    returns; the host reads NX_ERR_DEVICE_TIMEOUT and the next call is correct."""
    from nanopyx_gb300 import _device
    from nanopyx_gb300.synthetic import blinking_stack

    L = _native.lib()
    stream = torch.cuda.current_stream()
    s = stream.cuda_stream
    x = torch.from_numpy(blinking_stack(6, 64, 96, 12, seed=3)).cuda()
    plan = _device.get_plan(64, 96, 5, 1.5, 1.0, True)
    ws = workspace(L.nx_esrrf_st_workspace_bytes(plan.handle, 6))
    good = torch.empty((6, 320, 480), device="cuda")
    _native.check(L.nx_esrrf_st(plan.handle, x.data_ptr(), 6, good.data_ptr(), ws.data_ptr(),
                                ws.numel(), s))
    assert L.nx_workspace_status(ws.data_ptr(), s) == _native.NX_OK
    out = torch.zeros_like(good)
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    assert L.nx_selftest_fused_abort(plan.handle, x.data_ptr(), 6, out.data_ptr(), ws.data_ptr(),
                                     ws.numel(), 20_000_000, s) == _native.NX_OK
    t1.record(stream)
    assert L.nx_workspace_status(ws.data_ptr(), s) == _native.NX_ERR_DEVICE_TIMEOUT
    # every CTA gave up after about one 20 ms bound, not the 2 s default
    assert t0.elapsed_time(t1) < 1000.0
    # the aborted CTAs returned before their first store
    assert not out.any()
    # the same context computes the same result as before
    again = torch.empty_like(good)
    _native.check(L.nx_esrrf_st(plan.handle, x.data_ptr(), 6, again.data_ptr(), ws.data_ptr(),
                                ws.numel(), s))
    assert L.nx_workspace_status(ws.data_ptr(), s) == _native.NX_OK
    assert torch.equal(again, good)
