"""Runs of the compiled reference (``oracle/_ref``) at configuration sizes.

TEST INFRASTRUCTURE: these helpers call the reference's own Cython path the
way ``nanopyx.eSRRF()`` does (``methods/esrrf/eSRRF_workflow.py:58-121``):
per timepoint ``eSRRF_ST`` -> ``calculate_eSRRF_temporal_correlations`` ->
``macro_pixel_corrector``.  ``eSRRF_ST`` is independent per frame
(``_le_esrrf.pyx:172-196``: every stage maps frame t to frame t), so it is run
on blocks of frames to bound the host memory of its 2m-magnified gradient
images (2 x 5120^2 floats per 512^2 frame at m=5); the per-frame maps are
concatenated before the temporal step, which sees the whole timepoint exactly
as in the reference.
"""
from __future__ import annotations

import numpy as np

from oracle import esrrf_np as O
from oracle import ref_build

BLOCK = 12


def load():
    assert ref_build.available() or ref_build.build(), \
        "the compiled reference (oracle/_ref) is needed for these comparisons"
    return ref_build.load()


def esrrf_st(R, x, magnification, radius, sensitivity, block=BLOCK):
    """Reference eSRRF_ST (Threaded) on frame blocks -> (T, H*m, W*m) float32."""
    T, H, W = x.shape
    out = np.empty((T, H * magnification, W * magnification), dtype=np.float32)
    op = R["eSRRF_ST"](verbose=False)
    for a in range(0, T, block):
        out[a:a + block] = op.run(np.ascontiguousarray(x[a:a + block]),
                                  magnification=magnification, radius=radius,
                                  sensitivity=sensitivity, run_type="Threaded")
    return out


def esrrf_from_maps(R, st, magnification, frames_per_timepoint, correlation, mpc):
    """eSRRF()'s per-timepoint temporal step and macro-pixel correction on the
    per-frame maps ``st`` -> (n_tp, H*m, W*m) float32 (not squeezed)."""
    T = st.shape[0]
    fpt = frames_per_timepoint if 0 < frames_per_timepoint <= T else T
    n_tp = -(-T // fpt)
    out = np.zeros((n_tp,) + st.shape[1:], dtype=np.float32)
    for i in range(n_tp):
        tc = np.asarray(R["calculate_eSRRF_temporal_correlations"](st[i * fpt:(i + 1) * fpt],
                                                                   correlation))
        if mpc:
            out[i] = R["macro_pixel_corrector"](np.expand_dims(tc, 0),
                                                magnification=magnification)[0]
        else:
            out[i] = tc
    return out


def fp64_from_maps(st, magnification, frames_per_timepoint, correlation, mpc):
    """The same temporal step and macro-pixel correction through the FP64
    oracle (``oracle.esrrf_np.temporal_correlation`` / ``macro_pixel_correct``)
    applied to the given per-frame maps."""
    T = st.shape[0]
    fpt = frames_per_timepoint if 0 < frames_per_timepoint <= T else T
    n_tp = -(-T // fpt)
    out = np.zeros((n_tp,) + st.shape[1:], dtype=np.float64)
    for i in range(n_tp):
        v = O.temporal_correlation(st[i * fpt:(i + 1) * fpt], correlation)
        out[i] = O.macro_pixel_correct(v, magnification)[0] if mpc else v
    return out
