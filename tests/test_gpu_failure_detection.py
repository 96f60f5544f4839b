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
