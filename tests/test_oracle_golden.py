"""Pin the FP64 oracle (oracle/esrrf_np.py) against the reference's own outputs.

The golden vectors were produced by the reference's compiled Cython path
(tests/golden/make_golden.py); the oracle is accepted only if it reproduces
every one of them within the parity bar of this path (1e-4 of the output range;
observed ~1e-6 at these sizes -- the difference is the reference's float32
rounding of its sampling coordinates).
"""
import numpy as np
import pytest

from conftest import rel_err
from oracle import esrrf_np as O
from oracle import ref_build

TOL = 1e-4


def test_oracle_esrrf_st(golden):
    x = golden["esrrf_st/input"]
    for k, (m, r, s, iw) in enumerate(golden["esrrf_st/cases"]):
        got = O.esrrf_st(x, int(m), float(r), float(s), bool(iw))
        assert rel_err(got, golden[f"esrrf_st/{k}"]) <= TOL, (k, m, r, s, iw)


@pytest.mark.parametrize("corr", ["AVG", "VAR", "TAC2"])
@pytest.mark.parametrize("mpc", [0, 1])
def test_oracle_esrrf_full(golden, corr, mpc):
    x = golden["esrrf/input"]
    got = O.esrrf(x, 5, 1.5, 2, 5, corr, True, bool(mpc))
    assert rel_err(got, golden[f"esrrf/{corr}/{mpc}"]) <= TOL


def test_oracle_cr_and_robx(golden):
    x = golden["cr/input"]
    assert rel_err(O.cr_shift_magnify(x, 0, 0, 5, 5), golden["cr/0"]) <= 1e-6
    assert rel_err(O.cr_shift_magnify(x, 0.3, -1.2, 2.5, 3.0), golden["cr/1"]) <= 1e-6
    assert rel_err(O.cr_shift_magnify(x, 0, 0, 10, 10), golden["cr/2"]) <= 1e-6
    gc, gr = O.roberts_cross(x)
    # float64 restatement vs the reference's float32 sums: equal to float32 rounding
    assert rel_err(gc, golden["robx/gc"]) <= 1e-6
    assert rel_err(gr, golden["robx/gr"]) <= 1e-6


def test_oracle_rgc_standalone(golden):
    gci, gri, mag = golden["rgc/gci"], golden["rgc/gri"], golden["rgc/mag"]
    assert rel_err(O.radial_gradient_convergence(gci, gri, mag, 4, 1.5, 1), golden["rgc/0"]) <= TOL
    assert rel_err(O.radial_gradient_convergence(gci, gri, mag, 4, 1.5, 2, True, True),
                   golden["rgc/1"]) <= TOL
    assert rel_err(O.radial_gradient_convergence(gci, gri, mag, 4, 2.0, 1, False),
                   golden["rgc/2"]) <= TOL


def test_oracle_radiality(golden):
    x = golden["srrf/input"]
    for k, (m, ring, border, pos) in enumerate([(5, 0.5, 0, True), (4, 1.0, 1, False),
                                                 (2, 0.5, 0, True)]):
        mag = O.cr_shift_magnify(x, 0, 0, m, m)
        got = O.radiality(x, mag, m, ring, border, pos)
        assert rel_err(got, golden[f"srrf/{k}"]) <= TOL, k
        assert rel_err(O.macro_pixel_correct(got, m), golden[f"srrf/{k}/mpc"]) <= TOL, k


def test_oracle_temporal_and_mpc(golden):
    x = golden["temporal/input"]
    for corr in ("AVG", "VAR", "TAC2"):
        assert rel_err(O.temporal_correlation(x, corr), golden[f"temporal/{corr}"]) <= 1e-5
    x = golden["mpc/input"]
    assert rel_err(O.macro_pixel_correct(x, 5), golden["mpc/5"]) <= 1e-5


LAG_CASES = [(12, 2), (12, 3), (12, 4), (39, 3), (40, 2), (40, 4)]


@pytest.mark.parametrize("T,order", LAG_CASES)
def test_oracle_acrf_lag_integration(golden, T, order):
    got = O.srrf_acrf_integrated(golden[f"srrf_lag/{T}/input"], order)
    assert rel_err(got, golden[f"srrf_lag/{T}/{order}"]) <= 1e-5


def test_oracle_lag_schedule_reproduces_the_reference_index_errors():
    """Orders 3 and 4 raise IndexError at these frame counts in the reference
    (its binning reads frame t*order + order - 2 past the end); order 2 never."""
    fails = {3: [7, 10, 13, 16, 19, 22, 25, 28, 31, 34, 37, 40],
             4: [6, 9, 10, 13, 14, 17, 18, 21, 22, 25, 26, 29, 30, 33, 34, 37, 38]}
    for order in (2, 3, 4):
        got = []
        for T in range(1, 41):
            try:
                O.acrf_lag_levels(T, order)
            except IndexError:
                got.append(T)
        assert got == fails.get(order, []), order


@pytest.mark.parametrize("mag", [2, 5, 10])
def test_oracle_fht_interpolation(golden, mag):
    got = O.fht_space_interpolation(golden["fht/input"], mag)
    assert rel_err(got, golden[f"fht/{mag}"]) <= 1e-5


def test_oracle_fht_interpolation_tiled(golden):
    """Frames over 256 px a side are interpolated in Hann-blended tiles."""
    got = O.fht_space_interpolation(golden["fht/tiled_input"], 2)
    assert rel_err(got, golden["fht/tiled_2"]) <= 1e-5


@pytest.mark.parametrize("k,m,pad", [(0, 2, False), (1, 3, True), (2, 2, True)])
def test_oracle_esrrf_st_fht(golden, k, m, pad):
    got = O.esrrf_st_fht(golden["fht/input"], m, 1.5, 1, True, pad)
    assert rel_err(got, golden[f"fht/esrrf_st/{k}"]) <= TOL


def test_oracle_rejects_bad_correlation():
    with pytest.raises(ValueError):
        O.temporal_correlation(np.zeros((2, 3, 3)), "MAX")


def test_compiled_reference_reproduces_golden(golden):
    if not ref_build.available():
        pytest.skip("oracle/_ref not built on this machine")
    R = ref_build.load()
    x = golden["esrrf_st/input"]
    for k, (m, r, s, iw) in enumerate(golden["esrrf_st/cases"][:4]):
        out = R["eSRRF_ST"](verbose=False).run(x, magnification=int(m), radius=float(r),
                                               sensitivity=float(s), doIntensityWeighting=bool(iw),
                                               run_type="Threaded")
        assert rel_err(out, golden[f"esrrf_st/{k}"]) <= 1e-5


# --- parameter-sweep scoring (oracle/scoring_np.py) ---------------------------
SCORE_CASES = [(2, 1.5, 1, 0), (4, 1.0, 2, 0), (2, 2.0, 1, 1)]


@pytest.mark.parametrize("mag", [2, 4])
def test_oracle_dht_interpolation(golden, mag):
    from oracle import scoring_np as S

    got = S.dht_interpolate(golden["score/dht/input"], mag)
    assert rel_err(got, golden[f"score/dht/{mag}"]) <= 1e-5


@pytest.mark.parametrize("k", range(len(SCORE_CASES)))
def test_oracle_error_map(golden, k):
    """RSP, RSE and the fit agree with the reference's ErrorMap; the Brent
    minimum of the (flat) RMSE curve agrees to a few 1e-3."""
    from oracle import scoring_np as S

    xs = golden["score/stack"]
    e = S.error_map(np.mean(xs, axis=0), golden[f"score/em/{k}/sr"], SCORE_CASES[k][3])
    sigma, alpha, beta, rse, rsp = golden[f"score/em/{k}/vals"]
    assert abs(e["sigma"] - sigma) <= 5e-3 * sigma
    assert abs(e["alpha"] - alpha) <= 2e-3 * abs(alpha)
    assert abs(e["beta"] - beta) <= 1e-4 * abs(beta)
    assert abs(e["rse"] - rse) <= 1e-5 * rse
    assert abs(e["rsp"] - rsp) <= 1e-5
    assert rel_err(e["imRSE"], golden[f"score/em/{k}/imRSE"]) <= 1e-3


@pytest.mark.parametrize("k", range(len(SCORE_CASES)))
def test_oracle_fire_number(golden, k):
    from oracle import scoring_np as S

    f, _ = S.fire_number(golden[f"score/frc/{k}/odd"], golden[f"score/frc/{k}/even"])
    assert abs(f - golden[f"score/frc/{k}/fire"][0]) <= 1e-5 * f


def test_oracle_fire_number_even_square_crop(golden):
    from oracle import scoring_np as S

    a = golden["score/frc/crop/images"]
    f, curve = S.fire_number(a[0], a[1])
    assert curve.shape == (36 // 2 - 1, 3)
    assert abs(f - golden["score/frc/crop/fire"][0]) <= 1e-5 * f


def test_oracle_qnr_of_the_sweep(golden):
    """The oracle's eSRRF_ST + ErrorMap + FRC + QnR reproduces the reference's
    ParameterSweep.run on a 2 x 2 grid."""
    from oracle import scoring_np as S

    xq = golden["score/sweep/input"]
    rsp = np.zeros((2, 2))
    frc = np.zeros((2, 2))
    for si, s in enumerate([1, 2]):
        for ri, r in enumerate([1.0, 1.5]):
            rgc = O.esrrf_st(xq, 2, r, s)
            rsp[si, ri] = S.error_map(np.mean(xq, 0), rgc.mean(0))["rsp"]
            frc[si, ri] = S.fire_number(rgc[1::2].mean(0), rgc[::2].mean(0))[0]
    assert np.abs(S.qnr(rsp, frc) - golden["score/sweep/qnr"]).max() <= 1e-5


# --- eSRRF-3D -------------------------------------------------------------------
ESRRF3D_CASES = [(2, 2, 1.5, 1, "average", 1), (3, 1, 1.0, 2, "std", 1), (2, 3, 2.0, 1, "average", 0),
                 (1, 2, 1.5, 1, "average", 1)]


@pytest.mark.parametrize("k", range(len(ESRRF3D_CASES)))
def test_oracle_esrrf3d_st(golden, k):
    mxy, mz, r, s, mode, iw = ESRRF3D_CASES[k]
    got = O.esrrf3d_st(golden["esrrf3d/input"][:3], mxy, mz, r, 2.8, 4.0, s, mode, bool(iw))
    assert rel_err(got, golden[f"esrrf3d/{k}"]) <= 1e-5


def test_oracle_esrrf3d_workflow(golden):
    got = O.esrrf3d(golden["esrrf3d/input"], 2, 2, 1.5, frames_per_timepoint=2)
    assert rel_err(got, golden["esrrf3d/workflow"]) <= 1e-5


@pytest.mark.parametrize("k", range(5))
def test_oracle_decorrelation_resolution(golden, k):
    from oracle import scoring_np as S

    got = S.decorr_resolution(golden[f"score/decorr/{k}/image"])
    assert abs(got - golden["score/decorr/resolution"][k]) <= 1e-6 * got


def test_oracle_qnr_of_the_sweep_with_decorrelation(golden):
    from oracle import scoring_np as S

    xq = golden["score/sweep/input"]
    rsp = np.zeros((2, 2))
    res = np.zeros((2, 2))
    for si, s in enumerate([1, 2]):
        for ri, r in enumerate([1.0, 1.5]):
            rec = O.esrrf_st(xq, 2, r, s).mean(0)
            rsp[si, ri] = S.error_map(np.mean(xq, 0), rec)["rsp"]
            res[si, ri] = S.decorr_resolution(rec.astype(np.float32))
    assert np.abs(S.qnr(rsp, res) - golden["score/sweep/qnr_decorr"]).max() <= 1e-5
