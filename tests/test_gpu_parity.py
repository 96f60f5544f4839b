"""GPU parity of the CUDA path against the reference's golden vectors and the oracle.

Bar (floating point): max |got - ref| / (max(ref) - min(ref)) <= 1e-4, the
tolerance the eSRRF/SRRF path is held to; integer-exact steps (Roberts-Cross)
are compared bit for bit.  Every call goes through the package, which calls the
C ABI of libnanopyx_gb300.so.
"""
import warnings

import numpy as np
import pytest
import torch

import nanopyx_gb300 as nx
from conftest import rel_err
from nanopyx_gb300 import _native
from nanopyx_gb300.synthetic import blinking_stack
from oracle import esrrf_np as O
from oracle import ref_build

pytestmark = pytest.mark.gpu
TOL = 1e-4


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    _native.lib()
    yield
    torch.cuda.synchronize()


def test_esrrf_st_matches_reference(golden):
    x = golden["esrrf_st/input"]
    for k, (m, r, s, iw) in enumerate(golden["esrrf_st/cases"]):
        got = nx.eSRRF_ST(verbose=False).run(x, magnification=int(m), radius=float(r),
                                             sensitivity=float(s), doIntensityWeighting=bool(iw))
        assert isinstance(got, np.ndarray) and got.dtype == np.float32
        e = rel_err(got, golden[f"esrrf_st/{k}"])
        assert e <= TOL, (k, m, r, s, iw, e)


@pytest.mark.parametrize("corr", ["AVG", "VAR", "TAC2"])
@pytest.mark.parametrize("mpc", [0, 1])
def test_esrrf_matches_reference(golden, corr, mpc):
    x = golden["esrrf/input"]
    got = nx.eSRRF(x, magnification=5, radius=1.5, sensitivity=2, frames_per_timepoint=5,
                   temporal_correlation=corr, macro_pixel_correction=bool(mpc))
    ref = golden[f"esrrf/{corr}/{mpc}"]
    assert got.shape == ref.shape
    assert rel_err(got, ref) <= TOL


def test_multi_correlation_single_pass_equals_separate_calls(golden):
    x = golden["esrrf/input"]
    v, t, a = nx.eSRRF(x, 5, 1.5, 2, frames_per_timepoint=5,
                       temporal_correlation=("VAR", "TAC2", "AVG"))
    for name, arr in (("VAR", v), ("TAC2", t), ("AVG", a)):
        one = nx.eSRRF(x, 5, 1.5, 2, frames_per_timepoint=5, temporal_correlation=name)
        assert np.array_equal(arr, one), name


def test_shift_magnify_matches_reference(golden):
    x = golden["cr/input"]
    op = nx.CRShiftAndMagnify(verbose=False)
    assert rel_err(op.run(x, 0, 0, 5, 5), golden["cr/0"]) <= 1e-6
    assert rel_err(op.run(x, 0.3, -1.2, 2.5, 3.0), golden["cr/1"]) <= 1e-6
    assert rel_err(op.run(x, 0, 0, 10, 10), golden["cr/2"]) <= 1e-6


@pytest.mark.parametrize("mag_r,mag_c,sr,sc", [(0.5, 0.75, 0.0, 0.0), (2.5, 3.0, 0.3, -1.2),
                                               (1.0, 7.0, -2.0, 0.5), (5.0, 5.0, 0.0, 0.0)])
def test_shift_magnify_tiles_and_small_magnifications_against_oracle(mag_r, mag_c, sr, sc):
    """Magnifications >= 1 run the tiled kernel (partial tiles at these sizes),
    smaller ones the per-pixel kernel; both against the FP64 oracle."""
    x = blinking_stack(3, 37, 70, 12, seed=61)
    got = nx.CRShiftAndMagnify(verbose=False).run(x, sr, sc, mag_r, mag_c)
    ref = O.cr_shift_magnify(x, sr, sc, mag_r, mag_c)
    assert got.shape == ref.shape
    # the oracle's sampling coordinates are float64, the reference's (and these)
    # float32 i / mag - shift
    assert rel_err(got, ref) <= 1e-5


def test_temporal_correlations_long_stacks_against_oracle():
    """T <= 400 stages each pixel block in shared memory, longer stacks use the
    two-pass per-pixel kernel; both against float64."""
    rng = np.random.default_rng(62)
    for T in (3, 400, 401):
        x = (rng.random((T, 9, 13)) * 3 + 0.5).astype(np.float32)
        for corr in ("AVG", "VAR", "TAC2"):
            got = nx.calculate_eSRRF_temporal_correlations(x, corr)
            assert rel_err(got, O.temporal_correlation(x, corr)) <= 1e-5, (T, corr)


def test_roberts_cross_bit_exact(golden):
    gc, gr = nx.GradientRobertsCross(verbose=False).run(golden["cr/input"])
    assert np.array_equal(gc, golden["robx/gc"])
    assert np.array_equal(gr, golden["robx/gr"])


def test_rgc_standalone_matches_reference(golden):
    gci, gri, mag = golden["rgc/gci"], golden["rgc/gri"], golden["rgc/mag"]
    op = nx.RadialGradientConvergence(verbose=False)
    assert rel_err(op.run(gci, gri, mag, 4, 1.5, 1), golden["rgc/0"]) <= TOL
    assert rel_err(op.run(gci, gri, mag, 4, 1.5, 2, pad_edges=True), golden["rgc/1"]) <= TOL
    assert rel_err(op.run(gci, gri, mag, 4, 2.0, 1, doIntensityWeighting=False),
                   golden["rgc/2"]) <= TOL


def test_radiality_and_srrf_match_reference(golden):
    x = golden["srrf/input"]
    for k, (m, ring, border, pos) in enumerate([(5, 0.5, 0, True), (4, 1.0, 1, False),
                                                 (2, 0.5, 0, True)]):
        mag = nx.CRShiftAndMagnify(verbose=False).run(x, 0, 0, m, m)
        got = nx.Radiality(verbose=False).run(x, mag, magnification=m, ringRadius=ring,
                                              border=border, radialityPositivityConstraint=pos)
        assert rel_err(got, golden[f"srrf/{k}"]) <= TOL, k
        full = nx.SRRF(x, magnification=m, ringRadius=ring, border=border,
                       radialityPositivityConstraint=pos)
        assert rel_err(full, golden[f"srrf/{k}/mpc"]) <= TOL, k


def test_temporal_correlations_match_numpy_reference(golden):
    x = golden["temporal/input"]
    for corr in ("AVG", "VAR", "TAC2"):
        got = nx.calculate_eSRRF_temporal_correlations(x, corr)
        assert rel_err(got, golden[f"temporal/{corr}"]) <= 1e-6, corr
    with pytest.raises(ValueError):
        nx.calculate_eSRRF_temporal_correlations(x, "ACF")
    xs = golden["srrf_temporal/input"]
    for order in (0, 1, -1, 2, 3, 4):
        got = nx.calculate_SRRF_temporal_correlations(xs, order)
        assert rel_err(got, golden[f"srrf_temporal/{order}"]) <= 1e-5, order


@pytest.mark.parametrize("T,order", [(12, 2), (12, 3), (12, 4), (39, 3), (40, 2), (40, 4)])
def test_acrf_lag_integration_matches_reference(golden, T, order):
    x = golden[f"srrf_lag/{T}/input"]
    got = nx.calculate_SRRF_temporal_correlations(x, order, True)
    assert rel_err(got, golden[f"srrf_lag/{T}/{order}"]) <= 1e-6
    # the input is not modified (the re-binning works on a copy)
    assert np.array_equal(x, golden[f"srrf_lag/{T}/input"])


def test_acrf_lag_integration_larger_stack_and_index_errors():
    x = blinking_stack(100, 40, 48, 10, seed=51)
    for order in (2, 4):
        got = nx.calculate_SRRF_temporal_correlations(x, order, True)
        assert rel_err(got, O.srrf_acrf_integrated(x, order)) <= 1e-5, order
    for T, order in ((7, 3), (9, 4)):
        with pytest.raises(IndexError):
            nx.calculate_SRRF_temporal_correlations(x[:T], order, True)
    # the flag does not apply to orders 0, 1, -1 (as in the reference)
    assert np.array_equal(nx.calculate_SRRF_temporal_correlations(x, 1, True),
                          nx.calculate_SRRF_temporal_correlations(x, 1))


def test_macro_pixel_corrector_matches_reference(golden):
    got = nx.macro_pixel_corrector(golden["mpc/input"], 5)
    assert rel_err(got, golden["mpc/5"]) <= 1e-6


@pytest.mark.parametrize("T,H,W,m,r", [
    (1, 3, 5, 2, 1.5), (2, 17, 31, 5, 1.5), (3, 2, 9, 2, 1.0), (2, 31, 17, 4, 2.0),
    (1, 1, 7, 3, 1.5), (3, 20, 21, 5, 1.5), (2, 33, 65, 2, 2.5), (1, 9, 40, 6, 1.0),
])
def test_odd_sizes_against_oracle(T, H, W, m, r):
    x = blinking_stack(T, H, W, max(1, H * W // 40), seed=H * 100 + W)
    got = nx.eSRRF_ST(verbose=False).run(x, magnification=m, radius=r, sensitivity=1)
    ref = O.esrrf_st(x, m, r, 1)
    if np.ptp(ref) == 0:
        assert np.array_equal(got, ref.astype(np.float32))
    else:
        assert rel_err(got, ref) <= TOL


def test_results_are_deterministic():
    x = blinking_stack(8, 64, 64, 20, seed=21)
    a = nx.eSRRF(x, 5, 1.5, 2, temporal_correlation=("VAR", "TAC2"))
    b = nx.eSRRF(x, 5, 1.5, 2, temporal_correlation=("VAR", "TAC2"))
    for u, v in zip(a, b):
        assert np.array_equal(u, v)


def test_tensor_in_tensor_out_stays_on_device():
    x = torch.from_numpy(blinking_stack(4, 32, 32, 8, seed=22)).cuda()
    out = nx.eSRRF(x, 4, 1.5, 1)
    assert isinstance(out, torch.Tensor) and out.is_cuda and tuple(out.shape) == (128, 128)
    ref = nx.eSRRF(x.cpu().numpy(), 4, 1.5, 1)
    assert np.array_equal(out.cpu().numpy(), ref)


def test_streamed_blocks_equal_one_shot():
    x = blinking_stack(23, 40, 48, 10, seed=23)
    one = nx.eSRRF(x, 5, 1.5, 1, temporal_correlation=("AVG", "VAR", "TAC2"))
    acc = nx.ESRRFAccumulator(40, 48, 5, 1.5, 1)
    for a, b in ((0, 7), (7, 8), (8, 20), (20, 23)):
        acc.push(x[a:b])
    got = acc.finalize(("AVG", "VAR", "TAC2"))
    for u, v in zip(got, one):
        assert rel_err(u, v) <= 1e-5


def test_timepoints_equal_separate_calls():
    x = blinking_stack(30, 48, 40, 12, seed=24)
    full = nx.eSRRF(x, 4, 2.0, 2, frames_per_timepoint=12, temporal_correlation="TAC2")
    assert full.shape == (3, 192, 160)
    for i, (a, b) in enumerate(((0, 12), (12, 24), (24, 30))):
        one = nx.eSRRF(x[a:b], 4, 2.0, 2, temporal_correlation="TAC2")
        assert rel_err(full[i], one) <= 1e-5


def test_one_frame_tail_timepoint_like_the_reference():
    """A last timepoint of one frame: the reference's VAR is 0 there and its TAC2
    the mean of an empty lag product, NaN at every pixel (NaN through the
    macro-pixel correction too); the full timepoint matches the oracle."""
    x = blinking_stack(11, 20, 24, 6, seed=9)
    var, tac2 = nx.eSRRF(x, 2, 1.5, 1, frames_per_timepoint=10,
                         temporal_correlation=("VAR", "TAC2"))
    assert var.shape == tac2.shape == (2, 40, 48)
    assert np.all(var[1] == 0) and np.all(np.isnan(tac2[1]))
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", RuntimeWarning)  # the oracle's empty-slice mean
        for got, name in ((var, "VAR"), (tac2, "TAC2")):
            ref = O.esrrf(x, 2, 1.5, 1, 10, name)
            assert np.isnan(ref[1]).all() == (name == "TAC2")
            assert rel_err(got[0], ref[0]) <= TOL, name


def test_cfg0_against_reference():
    """100 frames x 100 x 100, 40 emitters, m=5, R=1.5, s=1, AVG + MPC."""
    x = blinking_stack(100, 100, 100, 40, seed=0)
    got = nx.eSRRF(x, magnification=5, radius=1.5, sensitivity=1, temporal_correlation="AVG")
    if ref_build.available():
        R = ref_build.load()
        st = R["eSRRF_ST"](verbose=False).run(x, magnification=5, radius=1.5, sensitivity=1,
                                              run_type="Threaded")
        tc = R["calculate_eSRRF_temporal_correlations"](st, "AVG")
        ref = R["macro_pixel_corrector"](np.expand_dims(np.asarray(tc), 0), magnification=5)[0]
    else:
        ref = O.esrrf(x[:10], 5, 1.5, 1, 0, "AVG")
        got = nx.eSRRF(x[:10], magnification=5, radius=1.5, sensitivity=1)
    assert rel_err(got, ref) <= TOL


def test_large_frame_properties():
    """512 x 512 frames at m=5, s=2: VAR >= 0, margins 0, finite, block split invariant."""
    x = blinking_stack(12, 512, 512, 400, seed=1)
    var, tac = nx.eSRRF(x, 5, 1.5, 2, frames_per_timepoint=6,
                        temporal_correlation=("VAR", "TAC2"), macro_pixel_correction=False)
    assert var.shape == (2, 2560, 2560)
    assert np.isfinite(var).all() and np.isfinite(tac).all()
    assert (var >= 0).all()
    mg = int(1.5 * 5)
    assert not var[:, :mg].any() and not var[:, -mg:].any()
    assert not var[:, :, :mg].any() and not var[:, :, -mg:].any()
    second = nx.eSRRF(x[6:], 5, 1.5, 2, temporal_correlation="VAR", macro_pixel_correction=False)
    assert rel_err(var[1], second) <= 1e-5
    # the FP64 oracle on a crop of frames reproduces the per-frame maps
    st = nx.eSRRF_ST(verbose=False).run(x[:1], 5, 1.5, 2)
    ref = O.esrrf_st(x[:1, :96, :96], 5, 1.5, 2)
    # interior of the crop only (the crop's own border differs from the full frame's)
    assert rel_err(st[0, 40:400, 40:400], ref[0, 40:400, 40:400]) <= TOL


@pytest.mark.parametrize("m,ring,border", [(5, 0.5, 0), (3, 1.5, 1), (7, 0.5, 0), (4, 2.5, 0)])
def test_srrf_fused_and_general_paths_against_oracle(m, ring, border):
    """m in {2,3,4,5,6,8} with ring <= 2 px run the fused kernel, the rest the general one."""
    x = blinking_stack(2, 21, 26, 4, seed=m * 10 + border)
    got = nx.SRRF(x, magnification=m, ringRadius=ring, border=border)
    mag = O.cr_shift_magnify(x, 0, 0, m, m)
    ref = O.macro_pixel_correct(O.radiality(x, mag, m, ring, border), m)
    assert rel_err(got, ref) <= TOL


@pytest.mark.parametrize("m,r,corr", [(8, 2.0, "VAR"), (5, 3.0, "TAC2"), (6, 2.5, "AVG"), (8, 1.5, "AVG")])
def test_one_frame_per_pass_instantiations_against_oracle(m, r, corr):
    """Large windows / magnifications whose frame-pair layout does not fit shared memory run
    one frame per pass; odd frame counts exercise the single-frame tail of a pass too."""
    x = blinking_stack(5, 22, 34, 6, seed=m * 7 + int(r * 2))
    got = nx.eSRRF(x, magnification=m, radius=r, sensitivity=2, temporal_correlation=corr,
                   macro_pixel_correction=False)
    ref = O.esrrf(x, m, r, 2, 0, corr, True, False)
    assert rel_err(got, np.squeeze(ref)) <= TOL
