"""FP64 NumPy restatement of the reference's eSRRF / SRRF CPU path.

TEST INFRASTRUCTURE ONLY: the oracle.  Only ``tests/``, ``__graft_entry__.smoke``
and ``bench.py``'s CPU-baseline legs import it, to check results; the product
package ``nanopyx_gb300`` never does.

Every function restates, in float64 arithmetic, one reference routine (paths
inside the reference project):

* ``cubic`` / ``cr_resample`` / ``cr_points``  -- Catmull-Rom (Keys, a = 0.5)
  ``src/include/_c_interpolation_catmull_rom.c:6-18`` (``_c_cubic``) and
  ``:21-52`` (``_c_interpolate``): pixel-centre convention, taps outside the
  image are skipped (not renormalised), 0 outside ``[0, rows) x [0, cols)``;
  sampling grid of ``ShiftAndMagnify`` (``row = i / mag - shift``,
  ``src/nanopyx/core/transform/_le_interpolation_catmull_rom.pyx:143-160``).
* ``roberts_cross``  -- ``src/include/_c_gradients.c:53-73``.
* ``rgc_params`` / ``radial_gradient_convergence``  --
  ``src/nanopyx/core/transform/_le_radial_gradient_convergence.pyx:85-115``
  and ``src/include/_c_sr_radial_gradient_convergence.c:4-90``.
* ``esrrf_st``  -- ``src/nanopyx/core/transform/_le_esrrf.pyx:172-196``.
* ``temporal_correlation``  --
  ``src/nanopyx/core/transform/sr_temporal_correlations.py:46-75,205-221``.
* ``acrf_lag_levels`` / ``srrf_acrf_integrated``  -- the ACRF with lag-time
  integration, ``sr_temporal_correlations.py:111-121,159-200``.
* ``macro_pixel_correct``  -- ``src/nanopyx/core/transform/mpcorrector.pyx:26-73``.
* ``esrrf``  -- ``src/nanopyx/methods/esrrf/eSRRF_workflow.py:58-121``.
* ``mirror_square`` / ``fht_interpolate_frame`` / ``fht_space_interpolation`` /
  ``esrrf_st_fht``  -- the use_fht=True path,
  ``src/nanopyx/core/transform/interpolation.py:22-290`` and
  ``_le_esrrf.pyx:183-188``.
* ``gradient_radiality`` / ``radiality`` / ``srrf``  --
  ``src/include/_c_gradients.c:3-25``, ``src/include/_c_sr_radiality.c:6-51``,
  ``src/nanopyx/core/transform/_le_radiality.pyx:86-125`` and
  ``src/nanopyx/methods/srrf/SRRF_workflow.py:50-76``.

Scalar parameters are taken exactly as the reference forms them (its float32
``sigma``, ``tSS``, ``tSO``, ring coordinates); the arithmetic on pixel data
is float64 throughout, so this is the "exact" answer the float32 reference and
the GPU path are both measured against.

The RGC reads the 2m-magnified gradient images only at rows / columns that are
multiples of ``m`` (plus the clamped last row / column), so ``esrrf_st``
evaluates the gradient interpolation at exactly those positions instead of
materialising the full ``(2Hm, 2Wm)`` images; the values are the same ones the
reference reads.
"""
from __future__ import annotations

import numpy as np

F32 = np.float32


# ----------------------------------------------------------------------------
# Catmull-Rom
# ----------------------------------------------------------------------------
def cubic(v):
    v = np.abs(np.asarray(v, dtype=np.float64))
    a = 0.5
    z = np.zeros_like(v)
    m1 = v < 1
    m2 = (v >= 1) & (v < 2)
    z[m1] = v[m1] * v[m1] * (v[m1] * (-a + 2) + (a - 3)) + 1
    vv = v[m2]
    z[m2] = -a * vv * vv * vv + 5 * a * vv * vv - 8 * a * vv + 4 * a
    return z


def _cr_weight_matrix(coords, n):
    """(len(coords), n) tap-weight matrix of _c_interpolate along one axis."""
    coords = np.asarray(coords, dtype=np.float64)
    Wm = np.zeros((coords.size, n), dtype=np.float64)
    inside = (coords >= 0) & (coords < n)
    base = np.floor(coords - 0.5).astype(np.int64)
    for t in range(4):
        nb = base - 1 + t
        ok = inside & (nb >= 0) & (nb < n)
        idx = np.nonzero(ok)[0]
        Wm[idx, nb[idx]] += cubic(coords[idx] - (nb[idx] + 0.5))
    return Wm, inside


def cr_resample(img2d, row_coords, col_coords):
    """Separable CR evaluation of one frame on a (rows x cols) coordinate grid."""
    img = np.asarray(img2d, dtype=np.float64)
    Wr, _ = _cr_weight_matrix(row_coords, img.shape[0])
    Wc, _ = _cr_weight_matrix(col_coords, img.shape[1])
    return Wr @ img @ Wc.T


def cr_shift_magnify(stack, shift_row, shift_col, mag_row, mag_col):
    """ShiftAndMagnify (reference sampling grid) for a (T, H, W) stack."""
    stack = np.asarray(stack)
    T, H, W = stack.shape
    rowsM = int(H * F32(mag_row))
    colsM = int(W * F32(mag_col))
    rr = np.arange(rowsM, dtype=np.float64) / float(F32(mag_row)) - float(F32(shift_row))
    cc = np.arange(colsM, dtype=np.float64) / float(F32(mag_col)) - float(F32(shift_col))
    out = np.empty((T, rowsM, colsM), dtype=np.float64)
    for t in range(T):
        out[t] = cr_resample(stack[t], rr, cc)
    return out


def cr_points(img2d, r, c):
    """Pointwise CR evaluation at coordinate arrays r, c (same shape)."""
    img = np.asarray(img2d, dtype=np.float64)
    rows, cols = img.shape
    r = np.asarray(r, dtype=np.float64)
    c = np.asarray(c, dtype=np.float64)
    inside = (r >= 0) & (r < rows) & (c >= 0) & (c < cols)
    r_int = np.floor(r - 0.5).astype(np.int64)
    c_int = np.floor(c - 0.5).astype(np.int64)
    q = np.zeros(r.shape, dtype=np.float64)
    for j in range(4):
        cn = c_int - 1 + j
        okc = (cn >= 0) & (cn < cols)
        wc = cubic(c - (cn + 0.5))
        p = np.zeros(r.shape, dtype=np.float64)
        for i in range(4):
            rn = r_int - 1 + i
            ok = okc & (rn >= 0) & (rn < rows)
            vals = np.where(ok, img[np.clip(rn, 0, rows - 1), np.clip(cn, 0, cols - 1)], 0.0)
            p += vals * cubic(r - (rn + 0.5))
        q += np.where(okc, p * wc, 0.0)
    return np.where(inside, q, 0.0)


# ----------------------------------------------------------------------------
# gradients
# ----------------------------------------------------------------------------
def roberts_cross(stack):
    """Roberts-Cross with top/left clamp; returns (gradient_col, gradient_row)."""
    a = np.asarray(stack, dtype=np.float64)
    if a.ndim == 2:
        a = a[None]
    up = np.concatenate([a[:, :1], a[:, :-1]], axis=1)          # [r0, c1]
    left = np.concatenate([a[:, :, :1], a[:, :, :-1]], axis=2)  # [r1, c0]
    upleft = np.concatenate([up[:, :, :1], up[:, :, :-1]], axis=2)  # [r0, c0]
    gc = up - left + a - upleft
    gr = -up + left + a - upleft
    return gc, gr


def gradient_radiality(frame):
    """Central differences on rows/cols 1..n-2, zero elsewhere (_c_gradients.c:3-25)."""
    f = np.asarray(frame, dtype=np.float64)
    gx = np.zeros_like(f)
    gy = np.zeros_like(f)
    gx[1:-1, 1:-1] = -f[1:-1, :-2] + f[1:-1, 2:]
    gy[1:-1, 1:-1] = -f[:-2, 1:-1] + f[2:, 1:-1]
    return gx, gy


# ----------------------------------------------------------------------------
# RGC
# ----------------------------------------------------------------------------
def rgc_params(radius):
    """Scalars exactly as _le_radial_gradient_convergence.pyx:85-92 forms them."""
    sigma = F32(float(radius) / 2.355)
    fwhm = F32(radius)
    tSS = F32(F32(2) * sigma * sigma)
    tSO = F32(F32(2) * sigma + F32(1))
    start = -int(F32(2.0) * fwhm)
    end = int(F32(2.0) * fwhm + F32(1))
    return dict(sigma=sigma, fwhm=fwhm, tSS=tSS, tSO=tSO, start=start, end=end)


def rgc_margin(radius, magnification, pad_edges=False):
    return 0 if pad_edges else int(float(F32(radius)) * magnification)


def _rgc_frame(gx_at, gy_at, rowsM, colsM, m, p, margin):
    """One frame of RGC (before intensity weighting).

    ``gx_at(py_idx, px_idx)`` returns gradient values at integer positions of the
    2m-magnified grid (arrays broadcast against each other).
    """
    yM = np.arange(margin, rowsM - margin)
    xM = np.arange(margin, colsM - margin)
    out = np.zeros((rowsM, colsM), dtype=np.float64)
    if yM.size == 0 or xM.size == 0:
        return out
    yc = ((yM + 0.5) / m)[:, None]
    xc = ((xM + 0.5) / m)[None, :]
    tSS = float(p["tSS"])
    tSO = float(p["tSO"])
    rgc = np.zeros((yM.size, xM.size))
    wsum = np.zeros((yM.size, xM.size))
    by = np.trunc(2.0 * yc).astype(np.int64)
    bx = np.trunc(2.0 * xc).astype(np.int64)
    for j in range(p["start"], p["end"]):
        vy = (by + j) / 2.0
        oky = (vy > 0) & (vy <= rowsM - 1)
        posy = np.clip(vy * m * 2, 0, rowsM * 2 - 1).astype(np.int64)
        for i in range(p["start"], p["end"]):
            vx = (bx + i) / 2.0
            okx = (vx > 0) & (vx <= colsM - 1)
            dx = vx - xc
            dy = vy - yc
            d = np.sqrt(dx * dx + dy * dy)
            ok = oky & okx & (d != 0) & (d <= tSO)
            if not ok.any():
                continue
            posx = np.clip(vx * m * 2, 0, colsM * 2 - 1).astype(np.int64)
            Gx = gx_at(posy, posx)
            Gy = gy_at(posy, posx)
            dsafe = np.where(d == 0, 1.0, d)
            w = (dsafe * np.exp(-(dsafe * dsafe) / tSS)) ** 4
            w = np.where(ok, w, 0.0)
            wsum += w
            gdotr = Gx * dx + Gy * dy
            gn = np.sqrt(Gx * Gx + Gy * Gy)
            with np.errstate(invalid="ignore", divide="ignore"):
                dk = np.abs(Gy * dx - Gx * dy) / gn
            dk = np.where(np.isnan(dk), dsafe, dk)
            dk = 1.0 - dk / dsafe
            rgc += np.where(ok & (gdotr < 0), dk * w, 0.0)
    with np.errstate(invalid="ignore", divide="ignore"):
        rgc = np.where(wsum > 0, rgc / np.where(wsum > 0, wsum, 1.0), 0.0)
    s = float(F32(p["sensitivity"]))
    rgc = np.where(rgc < 0, 0.0, rgc)
    if s > 1:
        rgc = rgc ** s
    out[margin:rowsM - margin, margin:colsM - margin] = rgc
    return out


def radial_gradient_convergence(gc_interp, gr_interp, image_interp, magnification=5,
                                radius=1.5, sensitivity=1, doIntensityWeighting=True,
                                pad_edges=False):
    """Standalone RGC op on given 2m-magnified gradients and m-magnified image."""
    gc_interp = np.asarray(gc_interp, dtype=np.float64)
    gr_interp = np.asarray(gr_interp, dtype=np.float64)
    image_interp = np.asarray(image_interp, dtype=np.float64)
    if gc_interp.ndim == 2:
        gc_interp, gr_interp = gc_interp[None], gr_interp[None]
    if image_interp.ndim == 2:
        image_interp = image_interp[None]
    T, rowsM, colsM = image_interp.shape
    p = rgc_params(radius)
    p["sensitivity"] = sensitivity
    margin = rgc_margin(radius, magnification, pad_edges)
    gw = int(colsM * 2)
    out = np.zeros((T, rowsM, colsM))
    for t in range(T):
        gcf = gc_interp[t].reshape(-1)
        grf = gr_interp[t].reshape(-1)
        f = _rgc_frame(lambda y, x: gcf[y * gw + x], lambda y, x: grf[y * gw + x],
                       rowsM, colsM, magnification, p, margin)
        out[t] = f * image_interp[t] if doIntensityWeighting else f
    return out


def esrrf_st(stack, magnification=5, radius=1.5, sensitivity=1, doIntensityWeighting=True):
    """eSRRF single task: (T, H, W) -> per-frame RGC maps (T, H*m, W*m)."""
    stack = np.asarray(stack)
    if stack.ndim == 2:
        stack = stack[None]
    T, H, W = stack.shape
    m = int(magnification)
    rowsM, colsM = H * m, W * m
    p = rgc_params(radius)
    p["sensitivity"] = sensitivity
    margin = rgc_margin(radius, m)
    # magnified intensity
    rr = np.arange(rowsM) / float(m)
    cc = np.arange(colsM) / float(m)
    # gradient interpolation only where RGC reads: rows/cols k*m (k >= 0),
    # clamped to 2*m*H - 1 by the RGC kernel
    ky = np.unique(np.clip(np.arange(0, 2 * H + 2) * m, 0, 2 * rowsM - 1))
    kx = np.unique(np.clip(np.arange(0, 2 * W + 2) * m, 0, 2 * colsM - 1))
    ry = ky / (2.0 * m)
    rx = kx / (2.0 * m)
    lut_y = np.full(2 * rowsM, -1, dtype=np.int64)
    lut_y[ky] = np.arange(ky.size)
    lut_x = np.full(2 * colsM, -1, dtype=np.int64)
    lut_x[kx] = np.arange(kx.size)
    gcs, grs = roberts_cross(stack)
    out = np.zeros((T, rowsM, colsM))
    for t in range(T):
        mag = cr_resample(stack[t], rr, cc)
        gxi = cr_resample(gcs[t], ry, rx)
        gyi = cr_resample(grs[t], ry, rx)
        f = _rgc_frame(lambda y, x: gxi[lut_y[y], lut_x[x]],
                       lambda y, x: gyi[lut_y[y], lut_x[x]],
                       rowsM, colsM, m, p, margin)
        out[t] = f * mag if doIntensityWeighting else f
    return out


# ----------------------------------------------------------------------------
# FHT (Fourier) interpolation, the use_fht=True path of eSRRF_ST
# (src/nanopyx/core/transform/interpolation.py:22-290, _le_esrrf.pyx:183-188)
# ----------------------------------------------------------------------------
def _pow2_ceil(n):
    return 1 if n <= 1 else 1 << int(np.ceil(np.log2(n)))


def mirror_square(img):
    """The frame tiled with alternating mirror images (an odd number of copies
    per axis, the centre copy upright) and cropped centrally to the smallest
    power-of-two square covering both sides (interpolation.py:22-55)."""
    h, w = img.shape
    n = max(_pow2_ceil(h), _pow2_ceil(w))
    copies = []
    for dim, axis_len in ((0, h), (1, w)):
        k = -(-n // axis_len)
        k += 1 - k % 2                       # odd
        mid = (k - 1) // 2
        idx = np.concatenate([np.arange(axis_len) if (c - mid) % 2 == 0
                              else np.arange(axis_len)[::-1] for c in range(k)])
        start = (k * axis_len - n) // 2
        copies.append(idx[start:start + n])
    return img[np.ix_(copies[0], copies[1])]


def fht_interpolate_frame(img, mag):
    """Zero-padded-spectrum interpolation of one frame (interpolation.py:58-111):
    the mirrored square's spectrum (real FFT along x, full along y) is moved
    into a mag-times larger zero spectrum (the y frequencies at or above half
    the size go to the top end), inverted, rescaled onto the frame's own
    [min, max] and cropped to the frame's magnified extent.  float64."""
    img = np.asarray(img, dtype=np.float64)
    lo, hi = float(np.float32(img.min())), float(np.float32(img.max()))
    sq = mirror_square(img)
    n = sq.shape[0]
    L = n * mag
    spec = np.fft.rfft2(sq)
    big = np.zeros((L, L // 2 + 1), dtype=np.complex128)
    keep = (n + 1) // 2
    big[:keep, :spec.shape[1]] = spec[:keep]
    big[L - (n - keep):, :spec.shape[1]] = spec[keep:]
    z = np.fft.irfft2(big, s=(L, L))
    zlo, zhi = z.min(), z.max()
    if zhi != zlo:
        z = (z - zlo) * ((hi - lo) / (zhi - zlo)) + lo
    y0 = (L - mag * img.shape[0]) // 2
    x0 = (L - mag * img.shape[1]) // 2
    return z[y0:y0 + mag * img.shape[0], x0:x0 + mag * img.shape[1]]


def _tile_starts(dim, ts, step):
    s = list(range(0, dim, step))
    if s and s[-1] + ts < dim:
        s.append(max(0, dim - ts))
    return s


def fht_space_interpolation(stack, mag, tile=256, overlap=16):
    """Per frame: frames up to `tile` pixels a side in one piece; larger ones in
    overlapping tile x tile pieces blended with Hann windows (float32 windows,
    as the reference; interpolation.py:117-181,250-290)."""
    stack = np.asarray(stack, dtype=np.float64)
    if stack.ndim == 2:
        stack = stack[None]
    T, h, w = stack.shape
    mag = int(mag)
    out = np.zeros((T, h * mag, w * mag))
    for t in range(T):
        f = stack[t]
        if h <= tile and w <= tile:
            out[t] = fht_interpolate_frame(f, mag)
            continue
        step = max(1, tile - 2 * overlap)
        acc = np.zeros((h * mag, w * mag))
        wgt = np.zeros((h * mag, w * mag))
        for r0 in _tile_starts(h, tile, step):
            r1 = min(r0 + tile, h)
            for c0 in _tile_starts(w, tile, step):
                c1 = min(c0 + tile, w)
                piece = fht_interpolate_frame(f[r0:r1, c0:c1], mag)
                wr = np.hanning(piece.shape[0] + 2)[1:-1].astype(np.float32).astype(np.float64)
                wc = np.hanning(piece.shape[1] + 2)[1:-1].astype(np.float32).astype(np.float64)
                win = np.outer(wr, wc)
                acc[r0 * mag:r1 * mag, c0 * mag:c1 * mag] += piece * win
                wgt[r0 * mag:r1 * mag, c0 * mag:c1 * mag] += win
        nz = wgt > 0
        acc[nz] /= wgt[nz]
        out[t] = acc
    return out


def esrrf_st_fht(stack, magnification=5, radius=1.5, sensitivity=1, doIntensityWeighting=True,
                 pad_edges=False):
    """eSRRF_ST with use_fht=True (_le_esrrf.pyx:183-188): FHT-magnified
    intensity (x m) and Roberts-Cross gradients (x 2m), then RGC with pad_edges."""
    stack = np.asarray(stack, dtype=np.float64)
    if stack.ndim == 2:
        stack = stack[None]
    m = int(magnification)
    mag = fht_space_interpolation(stack, m)
    gc, gr = roberts_cross(stack)
    return radial_gradient_convergence(fht_space_interpolation(gc, 2 * m),
                                       fht_space_interpolation(gr, 2 * m), mag, m, radius,
                                       sensitivity, doIntensityWeighting, pad_edges)


# ----------------------------------------------------------------------------
# temporal correlations and macro-pixel correction
# ----------------------------------------------------------------------------
def temporal_correlation(stack, correlation):
    x = np.asarray(stack, dtype=np.float64)
    if correlation == "AVG":
        return x.mean(axis=0)
    if correlation == "VAR":
        return x.var(axis=0)
    if correlation == "TAC2":
        c = x - x.mean(axis=0)
        return (c[:-1] * c[1:]).mean(axis=0)
    raise ValueError("Type of correlation must be AVG, VAR or TAC2")


def acrf_lag_levels(T, order):
    """Loop control of the reference's ACRF with lag-time integration
    (``sr_temporal_correlations.py:159-200``), replayed without the data.

    Returns one ``(n_iter, n_bin, n_binned)`` per level: the level runs
    ``t = 0 .. n_iter - 1`` (``t < n_binned - order``), re-bins frame ``t`` for
    ``t < n_bin`` (``t * order < n_binned``) and divides by ``n_binned`` (the
    frame count ``T`` at the first level, then ``T / order**k`` as a Python
    float).  Raises ``IndexError`` exactly where the reference's binning would
    read past the last frame (``im[t * order + order - 2]`` with that index
    ``>= T``: orders 3 and 4 at many frame counts).
    """
    levels = []
    n_b = T
    while n_b > order:
        t, n_bin = 0, 0
        while t < n_b - order:
            if t * order < n_b:
                if t * order + order - 2 >= T:
                    raise IndexError(f"index {t * order + order - 2} is out of bounds for "
                                     f"axis 0 with size {T}")
                n_bin = t + 1
            t += 1
        levels.append((t, n_bin, n_b))
        n_b = n_b / order
    return levels


def srrf_acrf_integrated(stack, order):
    """ACRF of order 2, 3 or 4 with lag-time integration, float64 arithmetic,
    the reference's steps (``sr_temporal_correlations.py:111-121,159-200``):
    per level, the lag products over ``t < n_binned - order`` (``ab`` restarts
    at each level; ``abc`` and the order-4 sums run on across levels), then
    frame ``t`` is replaced by ``sum_{k < order-1} frame[t*order + k] / order``
    (in place, after being zeroed, for ``t * order < n_binned``; else 0); the
    last level's ``|ab|`` (order 2), ``|abc|`` (3) or
    ``|abcd - ab cd - ac bd - ad bc|`` (4) over ``n_binned`` is the result
    (zeros when no level runs)."""
    im = np.array(stack, dtype=np.float64)
    T = im.shape[0]
    levels = acrf_lag_levels(T, order)
    mean = im.mean(axis=0)
    z = np.zeros(im.shape[1:])
    out = z.copy()
    abc, abcd, cd, ac, bd, ad, bc = (z.copy() for _ in range(7))
    for n_iter, n_bin, n_b in levels:
        ab = z.copy()
        for t in range(n_iter):
            a = im[t] - mean
            b = im[t + 1] - mean
            ab = ab + a * b
            if order == 3:
                abc = abc + a * b + (im[t + 2] - mean)
            if order == 4:
                c = im[t + 2] - mean
                d = im[t + 3] - mean
                abcd = abcd + a * b * c * d
                cd, ac, bd, ad, bc = cd + c * d, ac + a * c, bd + b * d, ad + a * d, bc + b * c
            im[t] = 0.0
            if t < n_bin:
                for k in range(order - 1):
                    im[t] = im[t] + im[t * order + k] / order
        if order == 3:
            out = np.abs(abc) / n_b
        elif order == 4:
            out = np.abs(abcd - ab * cd - ac * bd - ad * bc) / n_b
        else:
            out = np.abs(ab) / n_b
    return out


def macro_pixel_correct(img, magnification):
    a = np.array(img, dtype=np.float64)
    if a.ndim == 2:
        a = a[None]
    S, rowsM, colsM = a.shape
    m = int(magnification)
    rows, cols = rowsM // m, colsM // m
    for s in range(S):
        blk = a[s, :rows * m, :cols * m].reshape(rows, m, cols, m)
        cmap = blk.sum(axis=(0, 2)) / (rows * cols)
        corr = np.tile(cmap, (rowsM // m + 1, colsM // m + 1))[:rowsM, :colsM]
        nz = corr != 0
        a[s][nz] /= corr[nz]
    return a


def esrrf(stack, magnification=5, radius=1.5, sensitivity=1, frames_per_timepoint=0,
          temporal_correlation_name="AVG", doIntensityWeighting=True,
          macro_pixel_correction=True):
    stack = np.asarray(stack)
    if stack.ndim == 2:
        stack = stack[None]
    T = stack.shape[0]
    fpt = T if frames_per_timepoint == 0 or frames_per_timepoint > T else frames_per_timepoint
    ntp = T // fpt + (1 if T % fpt else 0)
    outs = []
    for i in range(ntp):
        rgc = esrrf_st(stack[fpt * i: fpt * (i + 1)], magnification, radius, sensitivity,
                       doIntensityWeighting)
        tc = temporal_correlation(rgc, temporal_correlation_name)
        if macro_pixel_correction:
            tc = macro_pixel_correct(tc, magnification)[0]
        outs.append(tc)
    return np.squeeze(np.stack(outs))


# ----------------------------------------------------------------------------
# SRRF radiality
# ----------------------------------------------------------------------------
def ring_coordinates(magnification, ring_radius, n=12):
    """Float32 ring offsets exactly as _le_radiality.pyx:92-104 forms them."""
    rr = F32(float(ring_radius) * magnification)
    step = F32((np.pi * 2.0) / n)
    xs = np.array([F32(np.cos(float(F32(step * F32(k)))) * float(rr)) for k in range(n)], dtype=np.float32)
    ys = np.array([F32(np.sin(float(F32(step * F32(k)))) * float(rr)) for k in range(n)], dtype=np.float32)
    return xs, ys, rr


def radiality(stack, image_interp, magnification=5, ringRadius=0.5, border=0,
              radialityPositivityConstraint=True, doIntensityWeighting=True):
    stack = np.asarray(stack)
    if stack.ndim == 2:
        stack = stack[None]
    image_interp = np.asarray(image_interp, dtype=np.float64)
    if image_interp.ndim == 2:
        image_interp = image_interp[None]
    T, h, w = stack.shape
    m = int(magnification)
    xs, ys, rr = ring_coordinates(m, ringRadius)
    out = np.zeros((T, h * m, w * m))
    j0, j1 = (1 + border) * m, (h - 1 - border) * m
    i0, i1 = (1 + border) * m, (w - 1 - border) * m
    if j1 <= j0 or i1 <= i0:
        return out
    jj = np.arange(j0, j1)[:, None].astype(np.float64)
    ii = np.arange(i0, i1)[None, :].astype(np.float64)
    yc = jj + 0.5
    xc = ii + 0.5
    for t in range(T):
        gx, gy = gradient_radiality(stack[t])
        acc = np.zeros((j1 - j0, i1 - i0))
        for k in range(xs.size):
            x0 = xc + float(xs[k])
            y0 = yc + float(ys[k])
            vgx = cr_points(gx, y0 / m + 0 * x0, x0 / m + 0 * y0)
            vgy = cr_points(gy, y0 / m + 0 * x0, x0 / m + 0 * y0)
            gmag = np.sqrt(vgx * vgx + vgy * vgy)
            with np.errstate(invalid="ignore", divide="ignore"):
                dk = 1 - (np.abs(vgy * (xc - x0) - vgx * (yc - y0)) / gmag) / float(rr)
            dk = np.where(gmag != 0, dk * dk, 0.0)
            sgn = (vgx * float(xs[k]) + vgy * float(ys[k])) > 0
            acc += np.where(sgn, -dk, dk)
        acc /= xs.size
        if radialityPositivityConstraint:
            acc = np.maximum(acc, 0)
        res = np.zeros((h * m, w * m))
        res[j0:j1, i0:i1] = acc
        out[t] = res * image_interp[t] if doIntensityWeighting else res
    return out


def srrf(stack, magnification=5, ringRadius=0.5, border=0, radialityPositivityConstraint=True,
         doIntensityWeighting=True, macro_pixel_correction=True):
    stack = np.asarray(stack)
    if stack.ndim == 2:
        stack = stack[None]
    mag = cr_shift_magnify(stack, 0, 0, magnification, magnification)
    rad = radiality(stack, mag, magnification, ringRadius, border,
                    radialityPositivityConstraint, doIntensityWeighting)
    if macro_pixel_correction:
        rad = macro_pixel_correct(rad, magnification)
    return rad


# ---------------------------------------------------------------------------
# eSRRF-3D (src/nanopyx/core/transform/_le_esrrf3d.pyx:65-140,
# src/nanopyx/core/transform/_interpolation.pyx:54-104,
# src/include/_c_gradients.c:75-116,
# src/include/_c_sr_radial_gradient_convergence.c:92-204,
# src/nanopyx/methods/esrrf_3d/eSRRF3D_workflow.py:8-107)
# ---------------------------------------------------------------------------
def interpolate_3d_zlinear(vol, mxy, mz):
    """Catmull-Rom x mxy in every slice, then the slices repeated mz times:
    the reference's "linear" z step takes slice sM // mz with weight 1 (its
    slice coordinate is an integer division)."""
    v = np.asarray(vol, dtype=np.float64)
    if mxy > 1:
        v = cr_shift_magnify(v, 0, 0, mxy, mxy)
    if mz > 1:
        v = np.repeat(v, mz, axis=0)
    return v


def gradient_3d(vol):
    """Central differences along x and y, the backward difference along z,
    halved, with indices clamped to the volume."""
    v = np.asarray(vol, dtype=np.float64)
    S, H, W = v.shape
    zi, yi, xi = np.arange(S), np.arange(H), np.arange(W)
    zm = np.maximum(zi - 1, 0)
    yp, ym = np.minimum(yi + 1, H - 1), np.maximum(yi - 1, 0)
    xp, xm = np.minimum(xi + 1, W - 1), np.maximum(xi - 1, 0)
    gc = (v[:, :, xp] - v[:, :, xm]) / 2
    gr = (v[:, yp, :] - v[:, ym, :]) / 2
    gs = (v - v[zm]) / 2
    return gc, gr, gs


def rgc3d_params(radius, radius_z):
    f32 = np.float32
    sigma = f32(radius / 2.355)
    sigma_z = f32(radius_z / 2.355)
    return dict(tSS=f32(f32(2) * sigma * sigma), tSO=f32(f32(2) * sigma + f32(1)),
                tSS_z=f32(f32(2) * sigma_z * sigma_z), tSO_z=f32(f32(2) * sigma_z + f32(1)),
                fwhm=f32(radius), fwhm_z=f32(radius_z))


def rgc3d_frame(gc, gr, gs, S, H, W, mxy, mz, radius, radius_z, sensitivity):
    """RGC-3D of one frame at every output voxel inside the margins (float64
    weights and sums; sample geometry and gradient indices in float32 as the
    reference forms them)."""
    f32 = np.float32
    p = rgc3d_params(radius, radius_z)
    Sm, Hm, Wm = S * mz, H * mxy, W * mxy
    margin = int(radius * mxy)
    margin_z = int(radius_z * mz)
    out = np.zeros((Sm, Hm, Wm))
    sM, rM, cM = np.meshgrid(np.arange(margin_z, Sm - margin_z), np.arange(margin, Hm - margin),
                             np.arange(margin, Wm - margin), indexing="ij")
    if sM.size == 0:
        return out
    xc = (cM.astype(f32) / f32(mxy)).astype(f32)
    yc = (rM.astype(f32) / f32(mxy)).astype(f32)
    zc = (sM.astype(f32) / f32(mz)).astype(f32)
    rgc = np.zeros(sM.shape)
    wsum = np.zeros(sM.shape)
    s0, s1 = -int(p["fwhm"]), int(p["fwhm"] + f32(1))
    z0, z1 = -int(p["fwhm_z"]), int(p["fwhm_z"] + f32(1))
    tSS, tSS_z = float(p["tSS"]), float(p["tSS_z"])
    for j in range(s0, s1 + 1):
        vy = (yc + f32(j)).astype(f32)
        for i in range(s0, s1 + 1):
            vx = (xc + f32(i)).astype(f32)
            for k in range(z0, z1 + 1):
                vz = (zc + f32(k)).astype(f32)
                ok = (vy > 0) & (vy <= H - 1) & (vx > 0) & (vx <= W - 1) & (vz > 0) & (vz <= S - 1)
                dx = (vx - xc).astype(f32)
                dy = (vy - yc).astype(f32)
                dz = (vz - zc).astype(f32)
                dxy2 = (dx * dx + dy * dy).astype(f32)
                dist = np.sqrt((dxy2 + dz * dz).astype(f32).astype(np.float64)).astype(f32)
                dxy = np.sqrt(dxy2.astype(np.float64)).astype(f32)
                ok &= (dist != 0) & (dxy <= p["tSO"]) & (dz <= p["tSO_z"])
                if not ok.any():
                    continue
                zi = (vz * f32(mz)).astype(f32).astype(np.int64)
                yi = (f32(mxy) * vy).astype(f32).astype(np.int64)
                xi = (f32(mxy) * vx).astype(f32).astype(np.int64)
                zi, yi, xi = (np.where(ok, a, 0) for a in (zi, yi, xi))
                Gx, Gy, Gz = gc[zi, yi, xi], gr[zi, yi, xi], gs[zi, yi, xi]
                d, x_, y_, z_ = (a.astype(np.float64) for a in (dist, dx, dy, dz))
                w = (d * np.exp(-x_ * x_ / tSS - y_ * y_ / tSS) * np.exp(-z_ * z_ / tSS_z)) ** 4
                w = np.where(ok, w, 0.0)
                wsum += w
                gdr = Gx * x_ + Gy * y_ + Gz * z_
                c1, c2, c3 = Gy * z_ - Gz * y_, Gz * x_ - Gx * z_, Gx * y_ - Gy * x_
                gm = np.sqrt(Gx * Gx + Gy * Gy + Gz * Gz)
                with np.errstate(invalid="ignore", divide="ignore"):
                    dk = np.sqrt(c1 * c1 + c2 * c2 + c3 * c3) / gm
                dk = np.where(np.isnan(dk), d, dk)
                dk = 1 - dk / d
                rgc += np.where(ok & (gdr < 0), dk * w, 0.0)
    with np.errstate(invalid="ignore", divide="ignore"):
        rgc = rgc / wsum
    if sensitivity > 1:
        rgc = np.where(rgc >= 0, np.abs(rgc) ** sensitivity, rgc)
    rgc = np.where(rgc < 0, 0.0, rgc)
    out[margin_z:Sm - margin_z, margin:Hm - margin, margin:Wm - margin] = rgc
    return out


def esrrf3d_st(stack, magnification_xy=2, magnification_z=2, radius=1.5, PSF_ratio=2.8,
               voxel_ratio=4.0, sensitivity=1, mode="average", doIntensityWeighting=True):
    """eSRRF3D_ST.run on a (T, S, H, W) stack: per frame RGC-3D (times the
    interpolated intensity), then the frames' mean or standard deviation."""
    x = np.asarray(stack, dtype=np.float32)
    if x.ndim == 3:
        x = x[None]
    radius_z = radius * PSF_ratio / voxel_ratio
    T, S, H, W = x.shape
    mxy, mz = magnification_xy, magnification_z
    maps = []
    for f in range(T):
        v = x[f]
        g = gradient_3d(v)
        gm = [interpolate_3d_zlinear(a.astype(np.float32), mxy, mz) for a in g]
        r = rgc3d_frame(*gm, S, H, W, mxy, mz, radius, radius_z, sensitivity)
        if doIntensityWeighting:
            r = r * interpolate_3d_zlinear(v, mxy, mz)
        maps.append(r)
    maps = np.stack(maps)
    if mode == "std":
        return np.sqrt(maps.var(axis=0))
    return maps.mean(axis=0)


def esrrf3d(stack, magnification_xy=2, magnification_z=2, radius=1.5, PSF_ratio=2.8,
            voxel_ratio=4.0, sensitivity=1, frames_per_timepoint=0, mode="average",
            doIntensityWeighting=True, macro_pixel_correction=True):
    """The eSRRF3D workflow: per timepoint eSRRF3D_ST, then the per-slice
    macro-pixel correction; (n_tp, S*mz, H*mxy, W*mxy)."""
    x = np.asarray(stack, dtype=np.float32)
    T = x.shape[0]
    fpt = T if frames_per_timepoint == 0 or frames_per_timepoint > T else frames_per_timepoint
    outs = []
    for t0 in range(0, T, fpt):
        v = esrrf3d_st(x[t0:t0 + fpt], magnification_xy, magnification_z, radius, PSF_ratio,
                       voxel_ratio, sensitivity, mode, doIntensityWeighting)
        if macro_pixel_correction:
            v = macro_pixel_correct(v, magnification_xy)
        outs.append(v)
    return np.stack(outs)
