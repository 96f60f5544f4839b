"""The C-ABI library loads and exports every entry point include/*.h declares.

No compute call is made here (no GPU needed); the host-only weight-table entry
point is checked against an independent NumPy evaluation of the reference's
distance weight (_c_sr_radial_gradient_convergence.c:4-6).
"""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from conftest import ROOT
from nanopyx_gb300 import _build, _native


def _declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(nx_\w+)\s*\(", src))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_build.LIB):
        _build.build()
    return _native.lib()


def test_library_exports_every_declared_symbol(lib):
    declared = _declared_symbols()
    assert len(declared) >= 20
    raw = ctypes.CDLL(_build.LIB)
    missing = [n for n in declared if not hasattr(raw, n)]
    assert not missing, missing
    assert sorted(_native.exported_symbols()) == declared


def test_abi_version(lib):
    assert lib.nx_abi_version() == 1


def _weights_numpy(m, radius):
    sigma = np.float32(radius / 2.355)
    tSS = np.float32(np.float32(2) * sigma * sigma)
    tSO = np.float32(np.float32(2) * sigma + np.float32(1))
    J = int(np.float32(2.0) * np.float32(radius))
    W2 = 2 * J + 1
    out = np.zeros((m, m, W2, W2))
    for py in range(m):
        cy = (2 * py + 1) // m
        for px in range(m):
            cx = (2 * px + 1) // m
            for jj in range(W2):
                dy = (cy + jj - J) / 2 - (py + 0.5) / m
                for ii in range(W2):
                    dx = (cx + ii - J) / 2 - (px + 0.5) / m
                    d = float(np.float32(np.hypot(dx, dy)))
                    if d != 0 and d <= tSO:
                        out[py, px, jj, ii] = (d * np.exp(-d * d / float(tSS))) ** 4
    return J, out


@pytest.mark.parametrize("m,radius", [(5, 1.5), (2, 1.0), (4, 2.5), (3, 1.25)])
def test_weight_table_matches_numpy(lib, m, radius):
    J, ref = _weights_numpy(m, radius)
    buf = np.zeros(ref.size, dtype=np.float32)
    got_J = lib.nx_esrrf_weight_table(m, radius, buf.ctypes.data, buf.size)
    assert got_J == J
    got = buf.reshape(ref.shape)
    assert np.allclose(got, ref, rtol=2e-7, atol=0)


def test_weight_table_rejects_bad_args(lib):
    assert lib.nx_esrrf_weight_table(0, 1.5, None, 0) == _native.NX_ERR_INVALID_ARG
    assert lib.nx_esrrf_weight_table(5, -1.0, None, 0) == _native.NX_ERR_INVALID_ARG
    assert "radius" in lib.nx_last_error().decode()


def test_argument_checks_run_before_any_device_work(lib):
    """Entry points reject bad arguments on the host, before touching a device."""
    P = ctypes.c_void_p
    # the failure-detection self-test needs a status workspace and a short limit
    assert lib.nx_selftest_wait_timeout(None, 0, 1000, None) == _native.NX_ERR_WORKSPACE
    assert lib.nx_selftest_wait_timeout(P(256), 64, 1000, None) == _native.NX_ERR_WORKSPACE
    assert lib.nx_selftest_wait_timeout(P(256), 256, 2_000_000_000, None) == \
        _native.NX_ERR_INVALID_ARG
    # temporal correlation: shape and correlation code
    assert lib.nx_temporal_correlation(None, 0, 10, _native.NX_CORR_AVG, None, None) == \
        _native.NX_ERR_INVALID_ARG
    assert lib.nx_temporal_correlation(None, 5, 10, 3, None, None) == _native.NX_ERR_INVALID_ARG
    # allocation-free macro-pixel correction: shape, magnification, static scratch size
    assert lib.nx_macro_pixel_correct_static(None, 1, 10, 10, 5, None) == \
        _native.NX_ERR_INVALID_ARG
    assert lib.nx_macro_pixel_correct_static(P(256), 1, 10, 10, 0, None) == \
        _native.NX_ERR_INVALID_ARG
    assert lib.nx_macro_pixel_correct_static(P(256), 100000, 10, 10, 5, None) == \
        _native.NX_ERR_INVALID_ARG
    assert b"static scratch" in lib.nx_last_error()
    # fused-kernel abort self-test: a plan is required before anything runs
    assert lib.nx_selftest_fused_abort(None, None, 1, None, None, 0, 20_000_000, None) == \
        _native.NX_ERR_INVALID_ARG
    # ACRF with lag-time integration: bad order, and the reference's IndexError
    # frame counts, are rejected on the host
    assert lib.nx_srrf_acrf_integrated(None, 12, 10, 5, None, None, 0, None) == \
        _native.NX_ERR_INVALID_ARG
    assert lib.nx_srrf_acrf_integrated(None, 7, 10, 3, None, None, 0, None) == \
        _native.NX_ERR_INDEX
    assert b"out of bounds" in lib.nx_last_error()
    assert lib.nx_srrf_acrf_integrated(None, 12, 10, 3, None, None, 0, None) == \
        _native.NX_ERR_INVALID_ARG
    # tile variants need a plan
    assert lib.nx_esrrf_plan_set_tile_variant(None, 1) == _native.NX_ERR_INVALID_ARG
    assert lib.nx_esrrf_plan_tile_variant(None) == _native.NX_ERR_INVALID_ARG
    # Fourier interpolation: plan arguments are checked on the host
    h = ctypes.c_void_p()
    assert lib.nx_fht_plan_create(None, 8, 8, 2) == _native.NX_ERR_INVALID_ARG
    assert lib.nx_fht_plan_create(ctypes.byref(h), 0, 8, 2) == _native.NX_ERR_INVALID_ARG
    assert lib.nx_fht_plan_create(ctypes.byref(h), 8, 8, 0) == _native.NX_ERR_INVALID_ARG
    assert lib.nx_fht_interpolate(None, None, 1, None, None, 0, None) == \
        _native.NX_ERR_INVALID_ARG
    # eSRRF-3D: the slice index of a window sample is formed by a multiply-high
    # that is exact while S * magnification_z^2 < 2^32; deeper stacks are
    # refused on the host (the pointers here are never dereferenced)
    big = ctypes.c_size_t(2 ** 63)
    assert lib.nx_esrrf3d_st(P(256), 1, 65536, 8, 8, 1, 256, 1.5, 1.05, 1.0, 0, 1, P(256),
                             P(256), big, None) == _native.NX_ERR_INVALID_ARG
    assert b"2^32" in lib.nx_last_error()
    assert lib.nx_esrrf3d_st(P(256), 1, 4, 8, 8, 0, 2, 1.5, 1.05, 1.0, 0, 1, P(256), P(256),
                             big, None) == _native.NX_ERR_INVALID_ARG
