"""The allocation-free macro-pixel correction entry point.

Callers such as real-time acquisition loops (all memory reserved at start-up)
or hosts whose own allocator owns the GPU cannot let a library allocate device
memory mid-run; nx_macro_pixel_correct_static serves them with a library-owned
256 KiB device scratch array.  This file is collected last so that a failure
here never hides another test.  Calls go through the C ABI (ctypes).
"""
import numpy as np
import pytest
import torch

from conftest import rel_err
from nanopyx_gb300 import _native

pytestmark = pytest.mark.gpu


def _stream():
    return torch.cuda.current_stream().cuda_stream


def test_static_scratch_matches_workspace_variant_on_two_calls():
    L = _native.lib()
    rng = np.random.default_rng(2024)
    # two calls in a row, different shapes: the second must not see the first's map
    for S, rows, cols, m in ((3, 40, 45, 5), (2, 24, 36, 4)):
        x = (rng.random((S, rows, cols)) + 0.1).astype(np.float32)
        x[0, :, :2] = 0.0
        ref = torch.from_numpy(x).cuda()
        got = ref.clone()
        ws = torch.empty(L.nx_macro_pixel_workspace_bytes(S, m), dtype=torch.uint8,
                         device="cuda")
        assert L.nx_macro_pixel_correct(ref.data_ptr(), S, rows, cols, m, ws.data_ptr(),
                                        ws.numel(), _stream()) == _native.NX_OK
        assert L.nx_macro_pixel_correct_static(got.data_ptr(), S, rows, cols, m,
                                               _stream()) == _native.NX_OK
        torch.cuda.synchronize()
        assert rel_err(got.cpu().numpy(), ref.cpu().numpy()) <= 1e-6


def test_static_scratch_rejects_calls_beyond_its_size():
    L = _native.lib()
    img = torch.ones((1, 8, 8), device="cuda")
    # 300 slices at m = 16 need more than the 256 KiB static scratch
    rc = L.nx_macro_pixel_correct_static(img.data_ptr(), 300, 8, 8, 16, _stream())
    assert rc == _native.NX_ERR_INVALID_ARG
    assert "static scratch" in L.nx_last_error().decode()
    torch.cuda.synchronize()
    assert torch.equal(img, torch.ones_like(img))
