"""Parameter-sweep scoring on the GPU: ErrorMap (RSP/RSE), FRC, QnR.

Against the compiled reference's golden vectors (error_map.pyx, frc.pyx,
parameter_sweep.py), against the FP64 oracle (oracle/scoring_np.py) for the
building blocks -- full-spectrum Fourier interpolation, Gaussian blur, moment
sums, FFT ring sums -- and, where the compiled reference is built, against a
live ParameterSweep run.  Bars: images 1e-5 of the range; RSP 1e-5 absolute;
RSE 1e-5 relative; FRC resolution 1e-4 relative; QnR 1e-4 absolute; the Brent
minimum of the flat RMSE curve to 5e-3 relative.
"""
import numpy as np
import pytest
import torch

import nanopyx_gb300 as nx
from conftest import rel_err
from nanopyx_gb300 import _native, scoring
from nanopyx_gb300.synthetic import blinking_stack
from oracle import ref_build
from oracle import scoring_np as S

pytestmark = pytest.mark.gpu
SCORE_CASES = [(2, 1.5, 1, 0), (4, 1.0, 2, 0), (2, 2.0, 1, 1)]


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    _native.lib()
    yield
    torch.cuda.synchronize()


@pytest.mark.parametrize("mag", [2, 4])
def test_full_spectrum_interpolation_matches_reference(golden, mag):
    from nanopyx_gb300.transform import _fht_device

    x = torch.from_numpy(golden["score/dht/input"]).cuda()
    got = _fht_device(x[None], mag, 1)[0].cpu().numpy()
    e = rel_err(got, golden[f"score/dht/{mag}"])
    print(f"\nfull-spectrum FHT x{mag}: gpu vs reference {e:.2e}")
    assert e <= 1e-5


@pytest.mark.parametrize("shape", [(64, 48), (37, 101), (5, 7)])
@pytest.mark.parametrize("sigma", [-3.0, 0.0, 0.3, 1.7, 6.79, 40.0])
def test_gaussian_blur_matches_scipy(shape, sigma):
    from scipy.ndimage import gaussian_filter

    rng = np.random.default_rng(int(abs(sigma) * 10) + shape[0])
    x = (rng.random(shape) * 100 + 50).astype(np.float32)
    got = scoring.gaussian_blur(torch.from_numpy(x).cuda(), sigma).cpu().numpy()
    ref = gaussian_filter(x.astype(np.float64), sigma)
    assert np.abs(got - ref).max() <= 2e-5 * np.abs(ref).max()
    got = scoring.gaussian_blur(torch.from_numpy(x).cuda(), sigma, 0.25, -3.0).cpu().numpy()
    ref = gaussian_filter((np.float32(0.25) * x + np.float32(-3.0)).astype(np.float64), sigma)
    assert np.abs(got - ref).max() <= 2e-5 * np.abs(ref).max()


def test_moment_sums_match_float64():
    rng = np.random.default_rng(5)
    x = rng.random((3, 1000, 37)).astype(np.float32) * 10
    y = rng.random((1000, 37)).astype(np.float32) * 10
    got = scoring.moment_sums(torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda().reshape(-1))
    for b in range(3):
        a, c = x[b].ravel().astype(np.float64), y.ravel().astype(np.float64)
        d = (x[b] - y).ravel().astype(np.float64)
        da, dc = a - a.mean(), c - c.mean()
        ref = [a.sum(), c.sum(), (da * da).sum(), (da * dc).sum(), (dc * dc).sum(), (d * d).sum()]
        assert np.allclose(got[b][:2], ref[:2], rtol=1e-7, atol=0)
        assert np.allclose(got[b][2:], ref[2:], rtol=1e-6, atol=0)
    # a large offset and a small spread: the centred moments do not cancel
    z = (1000.0 + rng.standard_normal(1 << 20) * 0.01).astype(np.float32)
    w = (z + rng.standard_normal(1 << 20).astype(np.float32) * 0.01).astype(np.float32)
    got = scoring.moment_sums(torch.from_numpy(z).cuda(), torch.from_numpy(w).cuda())[0]
    a, c = z.astype(np.float64), w.astype(np.float64)
    da, dc = a - a.mean(), c - c.mean()
    assert np.allclose(got[2:5], [(da * da).sum(), (da * dc).sum(), (dc * dc).sum()], rtol=1e-5)


@pytest.mark.parametrize("n", [26, 36, 200, 256, 1280])
def test_frc_curve_matches_oracle(n):
    """Unsmoothed FRC curves through the mixed-radix FFT (26 = 2 x 13 takes the
    generic radix path; 1280 = 4^4 x 5 the m = 5 sizes)."""
    a = blinking_stack(2, n, n + 3, max(4, n // 8), seed=n)
    fc = scoring.FIRECalculator()
    got = fc._frc_curve(torch.from_numpy(a[0]).cuda(), torch.from_numpy(a[1]).cuda())
    ref = S.frc_curve(a[0], a[1])
    assert got.shape == ref.shape
    assert np.array_equal(got[:, 2], ref[:, 2])  # samples per ring
    assert np.abs(got[:, 0] - ref[:, 0]).max() <= 1e-7
    assert np.abs(got[:, 1] - ref[:, 1]).max() <= 1e-4


@pytest.mark.parametrize("k", range(len(SCORE_CASES)))
def test_error_map_matches_reference(golden, k):
    xs = golden["score/stack"]
    em = nx.ErrorMap()
    em.optimise(np.mean(xs, axis=0), golden[f"score/em/{k}/sr"], SCORE_CASES[k][3])
    sigma, alpha, beta, rse, rsp = golden[f"score/em/{k}/vals"]
    print(f"\nErrorMap {k}: RSP gpu {em.getRSP():.7f} reference {rsp:.7f}; sigma gpu "
          f"{em.get_sigma():.5f} reference {sigma:.5f} ({em.n_evaluations} evaluations)")
    assert abs(em.get_sigma() - sigma) <= 5e-3 * sigma
    assert abs(em._alpha - alpha) <= 2e-3 * abs(alpha)
    assert abs(em._beta - beta) <= 1e-4 * abs(beta)
    assert abs(em.getRSE() - rse) <= 1e-5 * rse
    assert abs(em.getRSP() - rsp) <= 1e-5
    assert rel_err(em.imRSE, golden[f"score/em/{k}/imRSE"]) <= 1e-3
    assert isinstance(em.imRSE, np.ndarray)


def test_error_map_device_inputs_give_device_maps(golden):
    xs = torch.from_numpy(golden["score/stack"]).cuda()
    em = nx.ErrorMap()
    em.optimise(xs.mean(dim=0), torch.from_numpy(golden["score/em/0/sr"]).cuda())
    assert em.imRSE.is_cuda
    assert abs(em.getRSP() - golden["score/em/0/vals"][4]) <= 1e-5


@pytest.mark.parametrize("k", range(len(SCORE_CASES)))
def test_fire_number_matches_reference(golden, k):
    f = nx.FIRECalculator().calculate_fire_number(golden[f"score/frc/{k}/odd"],
                                                  golden[f"score/frc/{k}/even"])
    ref = golden[f"score/frc/{k}/fire"][0]
    print(f"\nFRC {k}: gpu {f:.6f} reference {ref:.6f}")
    assert abs(f - ref) <= 1e-4 * ref


def test_fire_number_even_square_crop(golden):
    a = golden["score/frc/crop/images"]
    fc = nx.FIRECalculator()
    f = fc.calculate_fire_number(a[0], a[1])
    assert fc.field_of_view == 36
    assert abs(f - golden["score/frc/crop/fire"][0]) <= 1e-4 * f


def test_sweep_qnr_matches_reference(golden):
    q = nx.ParameterSweep().run(golden["score/sweep/input"], 2, [1, 2], [1.0, 1.5])
    ref = golden["score/sweep/qnr"]
    print(f"\nQnR gpu {np.round(q.ravel(), 6)} reference {np.round(ref.ravel(), 6)}")
    assert np.abs(q - ref).max() <= 1e-4


def test_sweep_qnr_with_frame_slices_matches_reference(golden):
    q = nx.ParameterSweep().run(golden["score/sweep/input"], 2, [1, 2], [1.0, 1.5], n_frames=4)
    assert np.abs(q - golden["score/sweep/qnr_nframes4"]).max() <= 1e-4


def test_run_esrrf_parameter_sweep_front_door(golden):
    x = golden["score/sweep/input"]
    q = nx.run_esrrf_parameter_sweep(x, 2, [1, 2], [1.0, 1.5], return_qnr=True)
    assert np.abs(q - golden["score/sweep/qnr"]).max() <= 1e-4
    best = nx.run_esrrf_parameter_sweep(x, 2, [1, 2], [1.0, 1.5])
    si, ri = np.unravel_index(np.argmax(golden["score/sweep/qnr"]), (2, 2))
    assert best == ([1, 2][si], [1.0, 1.5][ri])


@pytest.mark.parametrize("corr", ["VAR", "TAC2"])
def test_sweep_with_other_correlations_against_oracle(corr):
    """VAR / TAC2 reconstructions (all, odd and even frames as separate batch
    items) scored like AVG."""
    from oracle import esrrf_np as O

    x = blinking_stack(8, 32, 32, 10, seed=31)
    ps = nx.ParameterSweep()
    q = ps.run(x, 2, [1, 2], [1.5], temporal_correlation=corr)
    rsp = np.zeros((2, 1))
    frc = np.zeros((2, 1))
    for si, s in enumerate([1, 2]):
        rgc = O.esrrf_st(x, 2, 1.5, s)
        rec = O.temporal_correlation(rgc, corr)
        rsp[si, 0] = S.error_map(np.mean(x, 0), rec)["rsp"]
        frc[si, 0] = S.fire_number(O.temporal_correlation(rgc[1::2], corr),
                                   O.temporal_correlation(rgc[::2], corr))[0]
    assert np.abs(ps.RSP_map - rsp).max() <= 1e-4
    assert np.abs(ps.FRC_map - frc).max() <= 1e-3 * np.abs(frc).max()


def test_sweep_against_live_reference():
    """A 3 x 3 grid at m = 4 against the compiled reference's ParameterSweep."""
    if not ref_build.available():
        pytest.skip("compiled reference not built here")
    R = ref_build.load()
    x = blinking_stack(16, 48, 48, 20, seed=32)
    sens, radii = [1, 2, 4], [1.0, 1.5, 2.0]
    ref = np.asarray(R["ParameterSweep"]().run(x, 4, sens, radii))
    got = nx.ParameterSweep().run(x, 4, sens, radii)
    print(f"\nQnR 3x3 m=4: max |gpu - reference| {np.abs(got - ref).max():.2e}")
    assert np.abs(got - ref).max() <= 1e-4


@pytest.mark.parametrize("sigma", [0.14, 0.33, 2.2, 9.0])
def test_blur_float64_sums_reproduce_scipy_float32(sigma):
    """With float64 sums each pass rounds like scipy's float32 output: the
    near-identity blurs whose difference from the image is the signal."""
    from scipy.ndimage import gaussian_filter

    rng = np.random.default_rng(3)
    x = (rng.random((96, 80)) * 100 + 50).astype(np.float32)
    got = scoring.gaussian_blur_batch(torch.from_numpy(x).cuda()[None], [sigma], [0],
                                      float64_sums=True)[0].cpu().numpy()
    ref = gaussian_filter(x, sigma)
    assert ref.dtype == np.float32
    ulp = np.spacing(np.abs(ref).astype(np.float32))
    assert np.all(np.abs(got - ref) <= ulp)
    hp_got, hp_ref = x - got, x - ref
    assert np.abs(hp_got - hp_ref).max() <= np.spacing(np.float32(150))


def test_decorr_prepare_matches_oracle():
    from oracle import scoring_np as S

    rng = np.random.default_rng(4)
    x = (rng.random((57, 93)) * 100 + 50).astype(np.float32)
    L = _native.lib()
    t = torch.from_numpy(x).cuda()
    out = torch.empty((128, 128), dtype=torch.float32, device="cuda")
    from nanopyx_gb300._device import workspace
    ws = workspace(L.nx_decorr_prepare_workspace_bytes(57, 93))
    assert L.nx_decorr_prepare(t.data_ptr(), 57, 93, out.data_ptr(), 128, ws.data_ptr(),
                               ws.numel(), torch.cuda.current_stream().cuda_stream) == 0
    ref = S.decorr_pad(S.apodize_edges(x))
    assert np.abs(out.cpu().numpy() - ref).max() <= 1e-4


@pytest.mark.parametrize("k", range(5))
def test_decorrelation_resolution_matches_reference(golden, k):
    got = nx.DecorrAnalysis().run_analysis(golden[f"score/decorr/{k}/image"])
    ref = golden["score/decorr/resolution"][k]
    print(f"\ndecorrelation {k}: gpu {got:.6f} reference {ref:.6f}")
    assert abs(got - ref) <= 1e-5 * ref


def test_sweep_qnr_with_decorrelation_matches_reference(golden):
    q = nx.ParameterSweep().run(golden["score/sweep/input"], 2, [1, 2], [1.0, 1.5],
                                use_decorr=True)
    assert np.abs(q - golden["score/sweep/qnr_decorr"]).max() <= 1e-4


def test_cli_decorrelation_command(golden, tmp_path):
    from nanopyx_gb300 import cli, tiff

    src, dst = tmp_path / "sr.tif", tmp_path / "dec.csv"
    tiff.imwrite(str(src), golden["score/decorr/0/image"])
    assert cli.main(["linkinpy-Metrics-ImageDecorrelationAnalysis", str(src), str(dst)]) == 0
    val = float(dst.read_text().splitlines()[1].split(",")[1])
    assert abs(val - golden["score/decorr/resolution"][0]) <= 1e-5 * val


def test_sweep_with_more_than_four_sensitivities_against_oracle():
    """Five sensitivities: two sensitivity groups per radius in the batch."""
    from oracle import esrrf_np as O

    x = blinking_stack(6, 24, 24, 6, seed=41)
    sens = [1, 1.5, 2, 3, 4]
    ps = nx.ParameterSweep()
    ps.run(x, 2, sens, [1.5])
    for si, s in enumerate(sens):
        rgc = O.esrrf_st(x, 2, 1.5, s)
        rsp = S.error_map(np.mean(x, 0), rgc.mean(0))["rsp"]
        frc = S.fire_number(rgc[1::2].mean(0), rgc[::2].mean(0))[0]
        assert abs(ps.RSP_map[si, 0] - rsp) <= 1e-4
        assert abs(ps.FRC_map[si, 0] - frc) <= 1e-3 * max(abs(frc), 1.0)


def test_error_map_without_magnification_against_oracle():
    """Reference and SR image of one size: no interpolation (error_map.pyx:54-57)."""
    rng = np.random.default_rng(9)
    ref = (rng.random((40, 36)) * 50 + 100).astype(np.float32)
    sr = (ref + rng.standard_normal((40, 36)).astype(np.float32) * 3).astype(np.float32)
    em = nx.ErrorMap()
    em.optimise(ref, sr)
    o = S.error_map(ref, sr)
    assert abs(em.getRSP() - o["rsp"]) <= 1e-5
    assert abs(em.getRSE() - o["rse"]) <= 1e-4 * o["rse"]
