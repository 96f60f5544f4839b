"""The use_fht=True path: Fourier interpolation as batched FP32 GEMMs.

Against the compiled reference's golden vectors (interpolation.py's
fht_space_interpolation and eSRRF_ST(use_fht=True) from _le_esrrf.pyx:183-188)
and against the FP64 oracle on a frame large enough for the reference's
256-pixel tiles.  Bar: max |d| / range <= 1e-4.
"""
import numpy as np
import pytest
import torch

import nanopyx_gb300 as nx
from conftest import rel_err
from nanopyx_gb300 import _native
from nanopyx_gb300.synthetic import blinking_stack
from oracle import esrrf_np as O

pytestmark = pytest.mark.gpu
TOL = 1e-4


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    _native.lib()
    yield
    torch.cuda.synchronize()


@pytest.mark.parametrize("mag", [2, 5, 10])
def test_fht_interpolation_matches_reference(golden, mag):
    got = nx.fht_space_interpolation(golden["fht/input"], mag)
    e = rel_err(got, golden[f"fht/{mag}"])
    print(f"\nFHT x{mag}: gpu vs reference {e:.2e}")
    assert e <= TOL


def test_fht_tiled_interpolation_matches_reference(golden):
    got = nx.fht_space_interpolation(golden["fht/tiled_input"], 2)
    assert got.shape == golden["fht/tiled_2"].shape
    assert rel_err(got, golden["fht/tiled_2"]) <= TOL


@pytest.mark.parametrize("k,m,pad", [(0, 2, False), (1, 3, True), (2, 2, True)])
def test_esrrf_st_fht_matches_reference(golden, k, m, pad):
    got = nx.eSRRF_ST(verbose=False).run(golden["fht/input"], magnification=m, radius=1.5,
                                         sensitivity=1, use_fht=True, pad_edges=pad)
    e = rel_err(got, golden[f"fht/esrrf_st/{k}"])
    print(f"\neSRRF_ST fht m={m} pad={pad}: gpu vs reference {e:.2e}")
    assert e <= TOL


def test_fht_several_tiles_against_oracle():
    """300 x 300 frames: 2 x 2 tiles of the reference's layout, edge tiles of
    76 pixels padded to their own power-of-two square."""
    x = blinking_stack(2, 300, 300, 60, seed=81)
    got = nx.fht_space_interpolation(x, 2)
    assert rel_err(got, O.fht_space_interpolation(x, 2)) <= TOL
    d = torch.from_numpy(x).cuda()
    on_dev = nx.fht_space_interpolation(d, 2)
    assert on_dev.is_cuda and np.array_equal(on_dev.cpu().numpy(), got)


def test_esrrf_fht_workflow_against_oracle():
    x = blinking_stack(6, 24, 28, 6, seed=82)
    got = nx.eSRRF(x, magnification=2, radius=1.5, sensitivity=2, frames_per_timepoint=4,
                   temporal_correlation=("AVG", "VAR"), use_fht=True, pad_edges=True)
    for name, g in zip(("AVG", "VAR"), got):
        ref = []
        for a in (0, 4):
            st = O.esrrf_st_fht(x[a:a + 4], 2, 1.5, 2, True, True)
            ref.append(O.macro_pixel_correct(O.temporal_correlation(st, name), 2)[0])
        assert rel_err(g, np.stack(ref)) <= TOL, name
