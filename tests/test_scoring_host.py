"""Host-side logic of the sweep scoring (no GPU): the FRC curve's smoothing and
threshold crossing, the QnR map, the decorrelation peak search and the
regression / Pearson statistics formed from moment sums -- each against the
oracle (oracle/scoring_np.py) and, where the compiled reference is built in
this container, against the reference itself."""
import contextlib
import io

import numpy as np
import pytest
from scipy import ndimage, stats

from nanopyx_gb300 import scoring
from oracle import ref_build
from oracle import scoring_np as S


def _pair(n, seed):
    rng = np.random.default_rng(seed)
    base = ndimage.gaussian_filter(rng.random((n, n)), 2.0) * 400
    a = (base + rng.normal(0, 3, (n, n))).astype(np.float32)
    b = (base + rng.normal(0, 3, (n, n))).astype(np.float32)
    return a, b


@pytest.mark.parametrize("n,seed", [(64, 1), (96, 2), (128, 3)])
def test_fire_number_from_a_curve_matches_the_oracle(n, seed):
    """Savitzky-Golay smoothing, the 1/7 crossing in the reference's float32
    segment arithmetic, and 1 / frequency."""
    a, b = _pair(n, seed)
    curve = S.frc_curve(a, b)
    fc = scoring.FIRECalculator()
    got = fc._from_curve(curve.copy(), n)
    ref, smoothed = S.fire_number(a, b)
    assert ref > 0 and fc.intersections.shape[0] >= 1
    assert np.allclose(fc.frc_curve[:, 1], smoothed[:, 1], rtol=0, atol=1e-12)
    assert abs(got - ref) <= 1e-5 * ref


def test_fire_number_without_a_crossing_is_zero():
    curve = np.zeros((40, 3))
    curve[:, 0] = np.linspace(0, 0.5, 40)
    curve[:, 1] = 0.9  # never reaches 1/7
    assert scoring.FIRECalculator()._from_curve(curve, 82) == 0.0


def test_qnr_map_matches_the_oracle_and_the_reference():
    rng = np.random.default_rng(5)
    rsp = rng.random((4, 4))
    frc = rng.random((4, 4)) * 20 + 2
    got = scoring.calculate_qnr_score(rsp, frc)
    assert np.allclose(got, S.qnr(rsp, frc), rtol=1e-12, atol=0)
    with pytest.raises(AssertionError):
        scoring.calculate_qnr_score(rsp, frc[:3])
    if not ref_build.available():
        pytest.skip("compiled reference not built in this container")
    R = ref_build.load()
    with contextlib.redirect_stdout(io.StringIO()):  # the reference prints its inputs
        ref = R["ParameterSweep"]().calculate_qnr_score(rsp, frc)
    assert np.array_equal(got, ref)


def test_decorrelation_peak_search_matches_the_oracle():
    """The walk back from a maximum at the curve's last point, on curves with
    interior peaks, rising ends and plateaus."""
    rng = np.random.default_rng(6)
    n_r = 50
    curves = [np.sin(np.linspace(0, np.pi, n_r)) * 0.8,          # interior peak
              np.linspace(0, 1, n_r),                             # rising to the end
              np.concatenate([np.linspace(0, 0.6, 40), np.full(10, 0.6)]),  # plateau at the end
              np.concatenate([np.linspace(0, 0.5, 30), np.linspace(0.5, 0.7, 20)]),
              rng.random(n_r) * 0.5]
    for d in curves:
        d = d.astype(np.float32)
        f, a = scoring._d_corr_max(d, 0.0, 1.0, n_r)
        fr, ar = S._d_corr_max(d.astype(np.float64), 0.0, 1.0, n_r)
        assert abs(float(f) - fr) <= 1e-6 and abs(float(a) - ar) <= 1e-6


def test_decorrelation_best_and_max_match_the_oracle():
    rng = np.random.default_rng(7)
    for _ in range(20):
        kc = rng.random(12).astype(np.float32)
        a = rng.random(12).astype(np.float32)
        got = scoring._best_and_max(kc, a)
        ref = S._scores(kc, a)
        for g, r in zip(got, ref):
            assert g[2] == r[2] and g[0] == r[0] and g[1] == r[1]


def test_regression_and_pearson_from_centred_moment_sums():
    rng = np.random.default_rng(8)
    x = rng.random(5000) * 10
    y = 3.2 * x - 1.5 + rng.normal(0, 0.4, x.size)
    mx, my = x.mean(), y.mean()
    s = np.array([x.sum(), y.sum(), ((x - mx) ** 2).sum(), ((x - mx) * (y - my)).sum(),
                  ((y - my) ** 2).sum(), ((x - y) ** 2).sum()])
    slope, intercept, rmse = scoring._regression(s, x.size)
    lr = stats.linregress(x, y)
    assert abs(slope - lr.slope) <= 1e-12 * abs(lr.slope)
    assert abs(intercept - lr.intercept) <= 1e-10
    assert abs(rmse - np.sqrt(np.mean((slope * x + intercept - y) ** 2))) <= 1e-10
    assert abs(scoring._pearson(s, x.size) - np.corrcoef(x, y)[0, 1]) <= 1e-6
    # a constant image has no correlation (the reference's 0)
    z = np.array([x.sum(), 5.0 * x.size, s[2], 0.0, 0.0, 0.0])
    assert scoring._pearson(z, x.size) == 0.0
