"""The allocation-free macro-pixel correction entry point.

Callers such as real-time acquisition loops (all memory reserved at start-up)
or hosts whose own allocator owns the GPU cannot let a library allocate device
memory mid-run; nx_macro_pixel_correct_static serves them with a library-owned
256 KiB device scratch array.  The tests cover two calls in a row against the
workspace variant, the exact size limit for several magnifications, and a
fresh process under lazy module loading with a start-up call first.  This file
is collected last so that a failure here never hides another test.  Calls go
through the C ABI (ctypes).
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


def _limit(m, rows):
    """Largest slice count whose map scratch fits the 256 KiB array:
    S * m^2 * min(64, max(1, rows)) floats <= 65536."""
    return 65536 // (m * m * min(64, max(1, rows)))


@pytest.mark.parametrize("m,rows,cols", [(2, 64, 40), (5, 64, 12), (16, 64, 6), (33, 3, 4)])
def test_static_scratch_limit_boundary(m, rows, cols):
    """The largest accepted call matches the workspace variant; one slice more
    is rejected before anything runs and leaves the images untouched."""
    L = _native.lib()
    S = _limit(m, rows)
    assert S >= 1
    rng = np.random.default_rng(m)
    x = (rng.random((S + 1, rows * m, cols * m)) + 0.1).astype(np.float32)
    ref = torch.from_numpy(x[:S]).cuda()
    got = ref.clone()
    ws = torch.empty(L.nx_macro_pixel_workspace_bytes(S, m), dtype=torch.uint8, device="cuda")
    assert L.nx_macro_pixel_correct(ref.data_ptr(), S, rows * m, cols * m, m, ws.data_ptr(),
                                    ws.numel(), _stream()) == _native.NX_OK
    assert L.nx_macro_pixel_correct_static(got.data_ptr(), S, rows * m, cols * m, m,
                                           _stream()) == _native.NX_OK
    torch.cuda.synchronize()
    assert rel_err(got.cpu().numpy(), ref.cpu().numpy()) <= 1e-6
    over = torch.from_numpy(x).cuda()
    rc = L.nx_macro_pixel_correct_static(over.data_ptr(), S + 1, rows * m, cols * m, m,
                                         _stream())
    assert rc == _native.NX_ERR_INVALID_ARG
    assert "static scratch" in L.nx_last_error().decode()
    torch.cuda.synchronize()
    assert np.array_equal(over.cpu().numpy(), x)


_LAZY_CHILD = """
import numpy as np, torch
from nanopyx_gb300 import _native
L = _native.lib()
s = torch.cuda.current_stream().cuda_stream
# start-up call: under lazy loading it loads the kernels and reserves the array
warm = torch.ones((1, 10, 10), device="cuda")
assert L.nx_macro_pixel_correct_static(warm.data_ptr(), 1, 10, 10, 5, s) == 0, \
    L.nx_last_error()
rng = np.random.default_rng(7)
for S, rows, cols, m in ((3, 40, 45, 5), (2, 24, 36, 4)):
    x = torch.from_numpy((rng.random((S, rows, cols)) + 0.1).astype(np.float32)).cuda()
    got = x.clone()
    ws = torch.empty(L.nx_macro_pixel_workspace_bytes(S, m), dtype=torch.uint8, device="cuda")
    assert L.nx_macro_pixel_correct(x.data_ptr(), S, rows, cols, m, ws.data_ptr(), ws.numel(),
                                    s) == 0
    assert L.nx_macro_pixel_correct_static(got.data_ptr(), S, rows, cols, m, s) == 0
    torch.cuda.synchronize()
    d = (got - x).abs().max().item() / (x.max() - x.min()).item()
    assert d <= 1e-6, d
print("lazy ok")
"""


def test_static_scratch_under_lazy_module_loading():
    """In a fresh process with CUDA_MODULE_LOADING=LAZY, a start-up call makes
    the array resident and later calls still match the workspace variant."""
    import os
    import subprocess
    import sys

    from conftest import ROOT

    env = dict(os.environ, CUDA_MODULE_LOADING="LAZY", PYTHONPATH=ROOT)
    r = subprocess.run([sys.executable, "-c", _LAZY_CHILD], env=env, cwd=ROOT,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "lazy ok" in r.stdout


def test_static_scratch_rejects_calls_beyond_its_size():
    L = _native.lib()
    img = torch.ones((1, 8, 8), device="cuda")
    # 300 slices at m = 16 need more than the 256 KiB static scratch
    rc = L.nx_macro_pixel_correct_static(img.data_ptr(), 300, 8, 8, 16, _stream())
    assert rc == _native.NX_ERR_INVALID_ARG
    assert "static scratch" in L.nx_last_error().decode()
    torch.cuda.synchronize()
    assert torch.equal(img, torch.ones_like(img))
