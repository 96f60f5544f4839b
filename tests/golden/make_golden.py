"""Generate the golden vectors in ``tests/golden/golden.npz``.

Runs the reference's OWN compiled CPU path (``oracle/_ref``, built from the
reference sources by ``oracle/ref_build.py``) on small seeded inputs and stores
inputs + outputs.  The reference's test-suite has no numeric fixtures for this
path (its eSRRF/SRRF tests are smoke tests on a network dataset), so these
vectors are what pins both the FP64 oracle and the CUDA path.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from nanopyx_gb300.synthetic import blinking_stack  # noqa: E402
from oracle import ref_build  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.npz")

# (magnification, radius, sensitivity, intensity weighting)
ESRRF_ST_CASES = [
    (5, 1.5, 1, True), (5, 1.5, 2, True), (2, 1.5, 1, True), (4, 2.5, 2, True),
    (3, 1.0, 1, False), (5, 2.0, 4, True), (1, 1.5, 1, True), (6, 1.5, 1, True),
    (8, 1.0, 1, True), (7, 1.5, 1, True), (5, 3.5, 1, True), (2, 0.4, 1, True),
    (4, 1.25, 1.5, True),
]
# eSRRF-3D: (magnification_xy, magnification_z, radius, sensitivity, mode, intensity weighting)
ESRRF3D_CASES = [(2, 2, 1.5, 1, "average", 1), (3, 1, 1.0, 2, "std", 1), (2, 3, 2.0, 1, "average", 0),
                 (1, 2, 1.5, 1, "average", 1)]
# decorrelation analysis of eSRRF reconstructions: (T, H, W, magnification, seed)
DECORR_CASES = [(10, 32, 32, 2, 1), (10, 40, 50, 2, 2), (20, 64, 64, 2, 3), (8, 48, 48, 3, 4),
                (6, 60, 45, 3, 5)]
# scoring: (magnification, radius, sensitivity, ErrorMap fixedSigma)
SCORE_CASES = [(2, 1.5, 1, 0), (4, 1.0, 2, 0), (2, 2.0, 1, 1)]


def main():
    if not ref_build.available():
        ref_build.build()
    R = ref_build.load()
    g = {}

    # eSRRF_ST per-frame maps
    x = blinking_stack(2, 16, 20, 5, seed=11)
    g["esrrf_st/input"] = x
    for k, (m, r, s, iw) in enumerate(ESRRF_ST_CASES):
        out = R["eSRRF_ST"](verbose=False).run(x, magnification=m, radius=r, sensitivity=s,
                                               doIntensityWeighting=iw, run_type="Threaded")
        g[f"esrrf_st/{k}"] = np.asarray(out, dtype=np.float32)
    g["esrrf_st/cases"] = np.array(ESRRF_ST_CASES, dtype=np.float64)

    # full eSRRF(): timepoints of 5 frames (last one short), AVG/VAR/TAC2, MPC on/off
    x = blinking_stack(12, 24, 20, 6, seed=12)
    g["esrrf/input"] = x
    m, r, s, fpt = 5, 1.5, 2, 5
    for corr in ("AVG", "VAR", "TAC2"):
        for mpc in (True, False):
            outs = []
            for i in range(0, x.shape[0], fpt):
                st = R["eSRRF_ST"](verbose=False).run(x[i:i + fpt], magnification=m, radius=r,
                                                      sensitivity=s, run_type="Threaded")
                tc = np.asarray(R["calculate_eSRRF_temporal_correlations"](st, corr))
                if mpc:
                    tc = R["macro_pixel_corrector"](np.expand_dims(tc, 0), magnification=m)[0]
                outs.append(np.asarray(tc, dtype=np.float32))
            g[f"esrrf/{corr}/{int(mpc)}"] = np.stack(outs)

    # Catmull-Rom ShiftAndMagnify
    x = blinking_stack(2, 9, 11, 2, seed=13)
    g["cr/input"] = x
    cr = R["CRShiftAndMagnify"](verbose=False)
    g["cr/0"] = cr.run(x, 0, 0, 5, 5, run_type="Threaded")
    g["cr/1"] = cr.run(x, 0.3, -1.2, 2.5, 3.0, run_type="Threaded")
    g["cr/2"] = cr.run(x, 0, 0, 10, 10, run_type="Threaded")

    # Roberts-Cross
    gc, gr = R["GradientRobertsCross"](verbose=False).run(x, run_type="Threaded")
    g["robx/gc"] = np.asarray(gc)
    g["robx/gr"] = np.asarray(gr)

    # standalone RGC on the reference's own magnified gradients
    x = blinking_stack(2, 12, 14, 3, seed=14)
    g["rgc/input"] = x
    m = 4
    gc, gr = R["GradientRobertsCross"](verbose=False).run(x, run_type="Threaded")
    gci = cr.run(gc, 0, 0, 2 * m, 2 * m, run_type="Threaded")
    gri = cr.run(gr, 0, 0, 2 * m, 2 * m, run_type="Threaded")
    mag = cr.run(x, 0, 0, m, m, run_type="Threaded")
    g["rgc/gci"], g["rgc/gri"], g["rgc/mag"] = gci, gri, mag
    rgc = R["RadialGradientConvergence"](verbose=False)
    g["rgc/0"] = rgc.run(gci, gri, mag, magnification=m, radius=1.5, sensitivity=1,
                         run_type="Threaded")
    g["rgc/1"] = rgc.run(gci, gri, mag, magnification=m, radius=1.5, sensitivity=2,
                         pad_edges=True, run_type="Threaded")
    g["rgc/2"] = rgc.run(gci, gri, mag, magnification=m, radius=2.0, sensitivity=1,
                         doIntensityWeighting=False, run_type="Threaded")

    # SRRF radiality (+ the reference's CR-magnified intensity)
    x = blinking_stack(2, 14, 16, 3, seed=15)
    g["srrf/input"] = x
    rad = R["Radiality"](verbose=False)
    for k, (m, ring, border, pos) in enumerate([(5, 0.5, 0, True), (4, 1.0, 1, False),
                                                 (2, 0.5, 0, True)]):
        mag = cr.run(x, 0, 0, m, m, run_type="Threaded")
        out = rad.run(x, mag, magnification=m, ringRadius=ring, border=border,
                      radialityPositivityConstraint=pos, run_type="Threaded")
        g[f"srrf/{k}"] = np.asarray(out)
        g[f"srrf/{k}/mpc"] = np.asarray(R["macro_pixel_corrector"](np.asarray(out), magnification=m))

    # temporal correlations
    rng = np.random.default_rng(16)
    x = (rng.random((7, 10, 12)) * 3 + 0.5).astype(np.float32)
    g["temporal/input"] = x
    for corr in ("AVG", "VAR", "TAC2"):
        g[f"temporal/{corr}"] = np.asarray(R["calculate_eSRRF_temporal_correlations"](x, corr))
    xs = (rng.random((9, 8, 10)) * 2 - 0.5).astype(np.float32)
    g["srrf_temporal/input"] = xs
    for order in (0, 1, -1, 2, 3, 4):
        g[f"srrf_temporal/{order}"] = np.asarray(
            R["calculate_SRRF_temporal_correlations"](xs, order), dtype=np.float32)
    # ACRF with lag-time integration (sr_temporal_correlations.py:159-200) at frame
    # counts the reference accepts (orders 3 and 4 raise IndexError at others)
    rng_lag = np.random.default_rng(17)
    for T, orders in ((12, (2, 3, 4)), (39, (3,)), (40, (2, 4))):
        xl = (rng_lag.random((T, 8, 10)) * 2 - 0.5).astype(np.float32)
        g[f"srrf_lag/{T}/input"] = xl
        for order in orders:
            g[f"srrf_lag/{T}/{order}"] = np.asarray(
                R["calculate_SRRF_temporal_correlations"](xl, order, True), dtype=np.float32)

    # FHT interpolation and eSRRF_ST(use_fht=True) (interpolation.py, _le_esrrf.pyx:183-188)
    xf = blinking_stack(2, 24, 20, 6, seed=18)
    g["fht/input"] = xf
    for mag in (2, 5, 10):
        g[f"fht/{mag}"] = np.asarray(R["fht_space_interpolation"](xf, mag), dtype=np.float32)
    xt = blinking_stack(1, 260, 40, 20, seed=19)
    g["fht/tiled_input"] = xt
    g["fht/tiled_2"] = np.asarray(R["fht_space_interpolation"](xt, 2), dtype=np.float32)
    for k, (m, pad) in enumerate(((2, False), (3, True), (2, True))):
        g[f"fht/esrrf_st/{k}"] = np.asarray(R["eSRRF_ST"](verbose=False).run(
            xf, magnification=m, radius=1.5, sensitivity=1, use_fht=True, pad_edges=pad,
            run_type="Threaded"), dtype=np.float32)

    # macro-pixel correction
    x = (rng.random((2, 20, 25)) + 0.1).astype(np.float32)
    x[0, :, :3] = 0.0
    g["mpc/input"] = x
    g["mpc/5"] = np.asarray(R["macro_pixel_corrector"](x, magnification=5))

    # parameter-sweep scoring (error_map.pyx, frc.pyx, parameter_sweep.py)
    xd = blinking_stack(1, 24, 20, 6, seed=20)[0]
    g["score/dht/input"] = xd
    for mag in (2, 4):
        g[f"score/dht/{mag}"] = np.asarray(R["dht_interpolation"](xd[None], mag)[0])
    xs = blinking_stack(20, 32, 32, 12, seed=21)
    g["score/stack"] = xs
    ref = np.mean(xs, axis=0)
    for k, (m, r, s, fixed) in enumerate(SCORE_CASES):
        rgc = np.asarray(R["eSRRF_ST"](verbose=False).run(xs, magnification=m, radius=r,
                                                           sensitivity=s, run_type="Threaded"))
        sr = np.mean(rgc, axis=0)
        em = R["ErrorMap"]()
        em.optimise(ref, sr, fixedSigma=fixed)
        g[f"score/em/{k}/sr"] = sr
        g[f"score/em/{k}/vals"] = np.array([em.get_sigma(), em._alpha, em._beta, em.getRSE(),
                                            em.getRSP()], dtype=np.float64)
        g[f"score/em/{k}/imRSE"] = np.asarray(em.imRSE)
        odd = np.mean(rgc[1::2], axis=0)
        even = np.mean(rgc[::2], axis=0)
        fc = R["FIRECalculator"]()
        g[f"score/frc/{k}/fire"] = np.array([fc.calculate_fire_number(odd, even)])
        g[f"score/frc/{k}/odd"] = odd
        g[f"score/frc/{k}/even"] = even
    # a non-square, odd-sided pair: the even-square crop
    a = blinking_stack(2, 37, 44, 10, seed=22)
    fc = R["FIRECalculator"]()
    g["score/frc/crop/images"] = a
    g["score/frc/crop/fire"] = np.array([fc.calculate_fire_number(a[0], a[1])])
    # the scored sweep: QnR over 2 x 2, all frames and with n_frames slices
    xq = blinking_stack(10, 32, 32, 12, seed=23)
    g["score/sweep/input"] = xq
    g["score/sweep/qnr"] = np.asarray(R["ParameterSweep"]().run(xq, 2, [1, 2], [1.0, 1.5]))
    g["score/sweep/qnr_nframes4"] = np.asarray(
        R["ParameterSweep"]().run(xq, 2, [1, 2], [1.0, 1.5], n_frames=4))

    # decorrelation analysis (decorr.pyx) on reconstructions, and the sweep scored by it
    dec = []
    for k, (T, h, w, m, seed) in enumerate(DECORR_CASES):
        xd = blinking_stack(T, h, w, 8, seed=seed)
        rec = np.mean(np.asarray(R["eSRRF_ST"](verbose=False).run(
            xd, magnification=m, radius=1.5, sensitivity=1, run_type="Threaded")), axis=0)
        g[f"score/decorr/{k}/image"] = rec
        dc = R["DecorrAnalysis"]()
        dc.run_analysis(rec)
        dec.append(dc.resolution)
    g["score/decorr/resolution"] = np.array(dec, dtype=np.float64)
    g["score/sweep/qnr_decorr"] = np.asarray(
        R["ParameterSweep"]().run(xq, 2, [1, 2], [1.0, 1.5], use_decorr=True))

    # eSRRF-3D (_le_esrrf3d.pyx, eSRRF3D_workflow.py)
    x3 = (np.random.default_rng(24).random((5, 6, 14, 12)) * 100 + 10).astype(np.float32)
    g["esrrf3d/input"] = x3
    for k, (mxy, mz, r, s, mode, iw) in enumerate(ESRRF3D_CASES):
        g[f"esrrf3d/{k}"] = np.asarray(R["eSRRF3D_ST"](verbose=False).run(
            x3[:3], magnification_xy=mxy, magnification_z=mz, radius=r, sensitivity=s,
            mode=mode, doIntensityWeighting=bool(iw), run_type="Threaded"))
    # the workflow: timepoints of 2 frames (last one short), per-slice MPC
    tps = []
    for t0 in range(0, 5, 2):
        v = R["eSRRF3D_ST"](verbose=False).run(x3[t0:t0 + 2], magnification_xy=2,
                                                magnification_z=2, radius=1.5, sensitivity=1,
                                                run_type="Threaded")
        tps.append(np.asarray(R["macro_pixel_corrector"](np.asarray(v), magnification=2)))
    g["esrrf3d/workflow"] = np.stack(tps)

    keep64 = ("esrrf_st/cases",)
    g = {k: (np.asarray(v, dtype=np.float32) if k not in keep64 and "/vals" not in k
             and not k.startswith("score/sweep/qnr") and k != "score/decorr/resolution"
             else np.asarray(v)) for k, v in g.items()}
    np.savez_compressed(OUT, **g)
    print(f"wrote {OUT}: {len(g)} arrays, {os.path.getsize(OUT) / 1e6:.2f} MB")


if __name__ == "__main__":
    main()
