"""eSRRF-3D on the GPU against the compiled reference's golden vectors
(_le_esrrf3d.pyx, the eSRRF3D workflow) and the FP64 oracle.  Bar: max |d| /
range <= 1e-4."""
import numpy as np
import pytest
import torch

import nanopyx_gb300 as nx
from conftest import rel_err
from nanopyx_gb300 import _native
from oracle import esrrf_np as O

pytestmark = pytest.mark.gpu
TOL = 1e-4
ESRRF3D_CASES = [(2, 2, 1.5, 1, "average", 1), (3, 1, 1.0, 2, "std", 1), (2, 3, 2.0, 1, "average", 0),
                 (1, 2, 1.5, 1, "average", 1)]


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    _native.lib()
    yield
    torch.cuda.synchronize()


@pytest.mark.parametrize("k", range(len(ESRRF3D_CASES)))
def test_esrrf3d_st_matches_reference(golden, k):
    mxy, mz, r, s, mode, iw = ESRRF3D_CASES[k]
    got = nx.eSRRF3D_ST(verbose=False).run(golden["esrrf3d/input"][:3], magnification_xy=mxy,
                                           magnification_z=mz, radius=r, sensitivity=s,
                                           mode=mode, doIntensityWeighting=bool(iw))
    e = rel_err(got, golden[f"esrrf3d/{k}"])
    print(f"\neSRRF3D case {k}: gpu vs reference {e:.2e}")
    assert e <= TOL


def test_esrrf3d_workflow_matches_reference(golden):
    got = nx.eSRRF3D(golden["esrrf3d/input"], 2, 2, 1.5, frames_per_timepoint=2)
    assert got.shape == golden["esrrf3d/workflow"].shape
    assert rel_err(got, golden["esrrf3d/workflow"]) <= TOL


@pytest.mark.parametrize("mode", ["average", "std"])
def test_esrrf3d_larger_volume_against_oracle(mode):
    rng = np.random.default_rng(7)
    x = (rng.random((4, 10, 40, 36)) * 200 + 20).astype(np.float32)
    got = nx.eSRRF3D_ST(verbose=False).run(x, magnification_xy=3, magnification_z=2, radius=1.5,
                                           sensitivity=2, mode=mode)
    ref = O.esrrf3d_st(x, 3, 2, 1.5, 2.8, 4.0, 2, mode, True)
    assert rel_err(got, ref) <= TOL


def test_esrrf3d_device_tensors_and_radius_check(golden):
    x = torch.from_numpy(golden["esrrf3d/input"][:3]).cuda()
    got = nx.eSRRF3D_ST(verbose=False).run(x, magnification_xy=2, magnification_z=2)
    assert got.is_cuda
    assert rel_err(got.cpu().numpy(), golden["esrrf3d/0"]) <= TOL
    assert nx.eSRRF3D_ST(verbose=False).run(x, radius=8.0) is None  # > H / 2: warning, None


def test_cli_esrrf_end_to_end(tmp_path):
    """The command-line front door: TIFF in, the same reconstruction as the
    Python call, TIFF out."""
    from nanopyx_gb300 import cli, tiff
    from nanopyx_gb300.synthetic import blinking_stack

    x = blinking_stack(12, 32, 40, 8, seed=5)
    src, dst = tmp_path / "in.tif", tmp_path / "out.tif"
    tiff.imwrite(str(src), x)
    assert cli.main(["linkinpy-SuperResolution-eSRRF", str(src), str(dst), "--magnification",
                     "4", "--temporal-correlation", "VAR"]) == 0
    ref = nx.eSRRF(x, magnification=4, temporal_correlation="VAR")
    got = tiff.imread(str(dst))
    assert got.shape == ref.shape and np.array_equal(got, ref)


def test_esrrf3d_single_frame_and_margins_covering_the_volume():
    """One frame; and a volume whose margins leave no inner voxel (all zero)."""
    rng = np.random.default_rng(8)
    x = (rng.random((1, 6, 20, 20)) * 100 + 10).astype(np.float32)
    got = nx.eSRRF3D_ST(verbose=False).run(x, magnification_xy=2, magnification_z=2)
    assert rel_err(got, O.esrrf3d_st(x, 2, 2)) <= TOL
    # radius_z = 1.0 * 2.0 / 2.0 = S / 2: accepted, and the z margin int(radius_z)
    # = 1 leaves no inner slice, so every voxel stays 0
    y = (rng.random((2, 2, 8, 8)) * 100 + 10).astype(np.float32)
    got = nx.eSRRF3D_ST(verbose=False).run(y, magnification_xy=1, magnification_z=1,
                                           radius=1.0, PSF_ratio=2.0, voxel_ratio=2.0)
    assert got.shape == (2, 8, 8)
    ref = O.esrrf3d_st(y, 1, 1, 1.0, 2.0, 2.0)
    assert not np.any(ref) and np.array_equal(got, ref.astype(np.float32))
    # one slice past that radius the reference declines (warning, None)
    assert nx.eSRRF3D_ST(verbose=False).run(y, magnification_xy=1, magnification_z=1,
                                            radius=1.5, PSF_ratio=2.8, voxel_ratio=4.0) is None
