"""Float64 NumPy/SciPy restatement of the parameter sweep's scoring.

TEST INFRASTRUCTURE ONLY: the oracle.  Only ``tests/`` import it, as the
reference for the results; the product package ``nanopyx_gb300`` never does.

Each function restates one reference routine (paths inside the reference
project), in float64 where the reference mixes precisions:

* ``dht_interpolate``  -- the full-spectrum Fourier interpolation ErrorMap
  uses, ``src/nanopyx/core/transform/_interpolation.pyx:106-200``: mirrored
  power-of-two square, fft2, centred block in a zero spectrum, ifft2, real
  part, rescale onto the image's [min, max], central crop.
* ``error_map``  -- ``src/nanopyx/core/transform/error_map.pyx:33-100,127-146``:
  Brent search (``scipy.optimize.brent``, bracket (0, 4 m / 2.35482)) of the
  RMSE between the reference interpolation and the linearly fitted, Gaussian-
  blurred SR image; RSE, RSP (Pearson,
  ``src/nanopyx/core/analysis/pearson_correlation.pyx:44-77``).
* ``frc_curve`` / ``fire_number``  -- ``src/nanopyx/core/analysis/frc.pyx:
  38-275``: even-square crop, Tukey(0.25) taper, centred FFTs, bilinear ring
  sampling at the reference's float32 positions, Savitzky-Golay smoothing,
  crossing of the 1/7 threshold.
* ``qnr``  -- ``src/nanopyx/core/analysis/parameter_sweep.py:113-139``.
"""
from __future__ import annotations

import numpy as np

from .esrrf_np import mirror_square


def dht_interpolate(img, mag):
    """Full-spectrum Fourier interpolation of one 2-D image (float64)."""
    img = np.asarray(img, dtype=np.float64)
    lo, hi = float(np.float32(img.min())), float(np.float32(img.max()))
    sq = mirror_square(img)
    n = sq.shape[0]
    L = n * mag
    spec = np.fft.fftshift(np.fft.fft2(sq))
    big = np.zeros((L, L), dtype=np.complex128)
    o = (L - n) // 2
    big[o:o + n, o:o + n] = spec
    z = np.real(np.fft.ifft2(np.fft.ifftshift(big)))
    zlo, zhi = z.min(), z.max()
    if zhi != zlo:
        z = (z - zlo) * ((hi - lo) / (zhi - zlo)) + lo
    y0 = (L - mag * img.shape[0]) // 2
    x0 = (L - mag * img.shape[1]) // 2
    return z[y0:y0 + mag * img.shape[0], x0:x0 + mag * img.shape[1]]


def _blur(img, sigma):
    from scipy.ndimage import gaussian_filter

    return gaussian_filter(np.asarray(img, dtype=np.float64), sigma)


def _fit(sigma, ref, sr):
    g = _blur(sr, sigma).ravel()
    y = ref.ravel()
    gm, ym = g.mean(), y.mean()
    slope = np.dot(g - gm, y - ym) / np.dot(g - gm, g - gm)
    intercept = ym - slope * gm
    return slope, intercept


def _rmse(sigma, ref, sr):
    a, b = _fit(sigma, ref, sr)
    return float(np.sqrt(np.mean((_blur(sr * a + b, sigma) - ref) ** 2)))


def pearson(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    da, db = a - a.mean(), b - b.mean()
    s11, s22 = np.dot(da, da), np.dot(db, db)
    if s11 == 0 or s22 == 0:
        return 0.0
    return float(np.dot(da, db) / np.sqrt(s11 * s22))


def error_map(img_ref, img_sr, fixed_sigma=0):
    """(sigma, alpha, beta, RSE, RSP, imRSE) of the reference's ErrorMap."""
    from scipy.optimize import brent

    ref = np.asarray(img_ref, np.float32).astype(np.float64)
    sr = np.asarray(img_sr, np.float32).astype(np.float64)
    m = int(sr.shape[0] / ref.shape[0])
    ref_int = dht_interpolate(ref, m) if m > 1 else ref
    max_sigma = (4 / 2.35482) * m
    sigma = fixed_sigma * m
    if fixed_sigma == 0:
        sigma = brent(_rmse, args=(ref_int, sr), brack=(0, max_sigma), maxiter=1000)
    a, b = _fit(sigma, ref_int, sr)
    blurred = _blur(a * sr + b, sigma)
    diff = blurred - ref_int
    return dict(sigma=float(sigma), alpha=float(a), beta=float(b),
                rse=float(np.sqrt(np.mean(diff ** 2))), rsp=pearson(blurred, ref_int),
                imRSE=np.abs(diff), ref_int=ref_int)


def _tukey(M, alpha=0.25):
    w = np.ones(M)
    if M <= 1:
        return w
    width = int(np.floor(alpha * (M - 1) / 2.0))
    n = np.arange(M)
    lo = n <= width
    hi = n >= M - width - 1
    w[lo] = 0.5 * (1 + np.cos(np.pi * (-1 + 2.0 * n[lo] / alpha / (M - 1))))
    w[hi] = 0.5 * (1 + np.cos(np.pi * (-2.0 / alpha + 1 + 2.0 * n[hi] / alpha / (M - 1))))
    return w


def ring_positions(N):
    """The reference's float32 sample positions per ring r = 1 .. N/2 - 2."""
    max_r = N // 2 - 1
    limit = np.float32(np.pi * 2)
    rings = []
    for r in range(1, max_r):
        step = np.float32(1.0 / r)
        ang = np.arange(0, float(limit), float(step), dtype=np.float32)
        ca = np.cos(ang.astype(np.float64)).astype(np.float32)
        sn = np.sqrt((np.float32(1) - ca * ca).astype(np.float64))
        sn = np.where(ang.astype(np.float64) > np.pi, -sn, sn).astype(np.float32)
        x = np.float32(max_r + 1) + np.float32(r) * ca
        y = np.float32(max_r + 1) + np.float32(r) * sn
        rings.append((x.astype(np.float32), y.astype(np.float32)))
    return rings


def frc_curve(img1, img2, pixel_size=1.0):
    """The reference's FRC curve (max_r, 3): frequency, FRC, samples (float64
    spectra and sums; positions as the reference computes them)."""
    a = np.asarray(img1, np.float32).astype(np.float64)
    b = np.asarray(img2, np.float32).astype(np.float64)
    h, w = a.shape
    size = min(h, w)
    size -= size % 2
    r0, c0 = (h - size) // 2, (w - size) // 2
    a = a[r0:r0 + size, c0:c0 + size]
    b = b[r0:r0 + size, c0:c0 + size]
    t = _tukey(size).astype(np.float32).astype(np.float64)
    win = np.outer(t, t)
    f1 = np.fft.fftshift(np.fft.fft2(a * win))
    f2 = np.fft.fftshift(np.fft.fft2(b * win))
    imgs = np.stack([(f1.real * f2.real + f1.imag * f2.imag),
                     np.abs(f1) ** 2, np.abs(f2) ** 2]).reshape(3, -1)
    max_r = size // 2 - 1
    freq = np.linspace(0, 1 / (2 * pixel_size), max_r, dtype=np.float32)
    res = np.zeros((max_r, 3))
    res[0] = (0, 1, 1)
    for r, (x, y) in enumerate(ring_positions(size), start=1):
        xb, yb = x.astype(np.int64), y.astype(np.int64)
        fx = np.maximum(x.astype(np.float64) - xb, 0)
        fy = np.maximum(y.astype(np.float64) - yb, 0)
        ll = yb * size + xb
        v = []
        for k in range(3):
            im = imgs[k]
            up = im[ll + size] + fx * (im[ll + size + 1] - im[ll + size])
            lo = im[ll] + fx * (im[ll + 1] - im[ll])
            v.append(np.sum(lo + fy * (up - lo)))
        res[r] = (freq[r], v[0] / np.sqrt(v[1] * v[2]), len(x))
    return res


def fire_number(img1, img2, pixel_size=1.0):
    """(fire number, smoothed curve) of the reference's FIRECalculator."""
    from scipy.signal import savgol_filter

    curve = frc_curve(img1, img2, pixel_size)
    window = int(0.0707 * curve.shape[0])
    if 3 >= window:
        window = 4
    curve[:, 1] = savgol_filter(curve[:, 1], window_length=window, polyorder=3)
    thr = 1.0 / 7.0
    for i in range(1, curve.shape[0]):
        y1, y2 = curve[i - 1, 1], curve[i, 1]
        if not ((thr >= y1 and thr < y2) or (y1 >= thr and y2 < thr)):
            continue
        x1, x2 = curve[i - 1, 0], curve[i, 0]
        # the crossing of the segment with the flat threshold
        px = x1 + (thr - y1) * (x2 - x1) / (y2 - y1) if y2 != y1 else x1
        return 1.0 / px, curve
    return 0.0, curve


def qnr(rsp, frc):
    rsp, frc = np.asarray(rsp, np.float64), np.asarray(frc, np.float64)
    lo, hi = frc.min(), frc.max()
    M1, M2 = 0.075, 0.925
    A1, A2 = np.log((1 - M1) / M1), np.log((1 - M2) / M2)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        x0 = (A2 * hi - A1 * lo) / (A2 - A1)
        k = 1 / (x0 - hi) * A1
        n = 1 / (np.exp(-k * (frc - x0)) + 1)
        return 2 * rsp * n / (rsp + n)


# ---------------------------------------------------------------------------
# decorrelation analysis (src/nanopyx/core/analysis/decorr.pyx:23-393 with
# transform/edges.pyx:9-49, transform/normalize.pyx:13-29,
# generate/mask.pyx:32-47, utils/array.pyx:8-40)
# ---------------------------------------------------------------------------
def apodize_edges(img):
    """Cosine roll-off of the 20-pixel border towards the mean of the pixels
    outside the inscribed circle of radius w/2 - 20."""
    a = np.asarray(img, np.float32).astype(np.float64)
    h, w = a.shape
    off = 20
    radius = np.float32(w // 2 - off)
    yy, xx = np.meshgrid(np.arange(h), np.arange(w), indexing="ij")
    dist = (yy - h // 2) ** 2 + (xx - w // 2) ** 2
    sel = dist > float(radius) ** 2
    edge_mean = a[sel].mean() if sel.any() else np.nan
    x0 = np.abs(xx - w // 2).astype(np.float64)
    y0 = np.abs(yy - h // 2).astype(np.float64)
    ex, ey = np.abs(x0 - w // 2), np.abs(y0 - h // 2)
    near = (ex <= off) | (ey <= off)
    d = np.minimum(ex, ey)
    c = (np.cos(d * np.pi / off - np.pi) + 1) / 2
    out = a.copy()
    out[near] = (c * (a - edge_mean) + edge_mean)[near]
    far = ~near & (np.abs(xx - w // 2) > w // 2) & (np.abs(yy - h // 2) > h // 2)
    out[far] = edge_mean
    return out


def decorr_pad(img):
    """The power-of-two square filled with the first pixel, the image placed at
    column (N - w) // 2 and row 0 (the reference's copy loop keeps the row
    offset at 0)."""
    a = np.asarray(img, np.float64)
    h, w = a.shape
    n = int(2 ** np.ceil(np.log(max(h, w)) / np.log(2.0)))
    out = np.full((n, n), a.ravel()[0])
    ox = (n - w) // 2
    out[:h, ox:ox + w] = a
    return out


def _decorr_coefs(img, crmin, crmax, n_r, zero_dc=False):
    """cr and the ring coefficients of one square image."""
    n = img.shape[0]
    F = np.fft.fftshift(np.fft.fft2(img))
    if zero_dc:
        F[n // 2, n // 2] = 0
    mag = np.abs(F)
    yy, xx = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    mask = ((yy - n / 2) ** 2 + (xx - n / 2) ** 2) < n * n / 4
    cr = np.sqrt(np.sum(mag[mask] ** 2))
    f32 = np.float32
    ox = int(f32(n) * (f32(1) - f32(crmax)) / f32(2))
    w = int(f32(n) * f32(crmax))
    coef = np.zeros(2 * n_r)
    kmax = n * n // 2 + n // 2
    xs, ys = np.meshgrid(np.arange(ox, ox + w), np.arange(ox, ox + w), indexing="ij")
    xs, ys = xs.ravel(), ys.ravel()  # x-major: the reference's loop order
    keep = (xs * n + ys) <= kmax
    xs, ys = xs[keep], ys[keep]
    dist = np.sqrt(4.0 * ((xs - n // 2) ** 2 + (ys - n // 2) ** 2) / (n * n))
    ok = dist <= crmax
    xs, ys, dist = xs[ok], ys[ok], dist[ok]
    dm = (dist - crmin) / (crmax - crmin) * (n_r - 1)
    dm = np.maximum(dm, 0)
    d = np.floor(dm + 0.5).astype(np.int64)
    ok = d < n_r
    xs, ys, d = xs[ok], ys[ok], d[ok]
    m = mag[ys, xs]
    np.add.at(coef, d, m)
    np.add.at(coef, d + n_r, (m != 0).astype(np.float64))
    return cr, coef


def _d_curve(cr, coef, n_r):
    D = np.cumsum(coef[:n_r])
    Cc = np.cumsum(coef[n_r:])
    with np.errstate(invalid="ignore", divide="ignore"):
        out = np.where((cr == 0) | (Cc == 0), np.nan, np.sqrt(2) * D / (cr * np.sqrt(Cc)))
    if np.isnan(out[0]):
        out[0] = 0
    return out


def _get_max(arr, x1, x2):
    i, v = x1, arr[x1]
    for k in range(x1, x2):
        if arr[k] > v:
            i, v = k, arr[k]
    return [i, v]


def _get_min(arr, x1, x2):
    i, v = x1, arr[x1]
    for k in range(x1, x2):
        if arr[k] < v:
            i, v = k, arr[k]
    return [i, v]


def _d_corr_max(d, r1, r2, n_r):
    t = np.array(d, dtype=np.float64)
    out = _get_max(d, 0, n_r)
    length = len(t)
    dt = 0.001
    while out[0] == length - 1:
        t[length - 1] = 0
        length -= 1
        if length == 0:
            out = [0, 0]
            break
        out = _get_max(t, 0, n_r)
        tmin = _get_min(t, int(out[0]), length - 1)
        if t[int(out[0])] - tmin[1] > dt:
            break
        t[int(out[0])] = tmin[1]
        out[0] = length - 1
    return [r1 + (r2 - r1) * out[0] / (n_r - 1), out[1]]


def _scores(kc, a):
    best, gm_max = [0.0, 0.0, 0.0], 0.0
    for k in range(len(kc)):
        if kc[k] * a[k] > gm_max:
            gm_max = kc[k] * a[k]
            best = [kc[k], a[k], k]
    top, kc_max = [0.0, 0.0, 0.0], 0.0
    for k in range(len(kc)):
        if kc[k] > kc_max:
            kc_max = kc[k]
            top = [kc[k], a[k], k]
    return best, top


def decorr_resolution(img, rmin=0.0, rmax=1.0, n_r=50, n_g=10, pixel_size=1.0):
    """DecorrAnalysis(...).run_analysis(img).resolution.  Sums and spectra in
    float64; the padded image, its Gaussian blurs and the high-pass
    differences in float32 as the reference forms them -- at the smallest blur
    widths the high-pass image is a cancellation (the float32 blur equals the
    image), and the decisions that follow depend on it -- and the search
    state (band limits, blur widths) in float32."""
    from scipy.ndimage import gaussian_filter

    f32 = np.float32
    temp = decorr_pad(apodize_edges(img)).astype(np.float32)
    n = temp.shape[0]
    cr, coef = _decorr_coefs(temp.astype(np.float64), rmin, rmax, n_r, zero_dc=True)
    d0 = _d_curve(cr, coef, n_r).astype(np.float32)
    kc0 = f32(_d_corr_max(d0, 0, 1, n_r)[0])
    g_max = f32(n // 2) if kc0 == 0 else f32(f32(2) / kc0)
    g_min = f32(0.14)
    crmin, crmax = f32(rmin), f32(rmax)
    kc_max = f32(0)

    def widths(lo, hi):
        return [float(np.exp(np.log(np.float64(lo)) + (np.log(np.float64(hi)) - np.log(np.float64(lo))) *
                             np.float64(f32(f32(k) / f32(n_g - 1))))) for k in range(n_g)]

    for refine in range(2):
        curves = []
        for sig in widths(g_min, g_max):
            hp = (temp - gaussian_filter(temp, sig)).astype(np.float32)
            c_, coef_ = _decorr_coefs(hp.astype(np.float64), float(crmin), float(crmax), n_r)
            curves.append(_d_curve(c_, coef_, n_r).astype(np.float32))
        res = [_d_corr_max(c, float(crmin), float(crmax), n_r) for c in curves]
        kc = [f32(r[0]) for r in res]
        a = [f32(r[1]) for r in res]
        if refine == 0:
            r0 = _d_corr_max(d0, float(crmin), float(crmax), n_r)
            kc.append(f32(r0[0]))
            a.append(f32(r0[1]))
            gm, mx = _scores(kc, a)
            crmin = f32(max(f32(np.float64(min(gm[0], mx[0])) - 0.05), f32(rmin)))
            crmax = f32(min(f32(np.float64(max(gm[0], mx[0])) + 0.3), f32(rmax)))
            ind1 = f32(min(gm[2], mx[2]) - 1)
            ind2 = f32(max(gm[2], mx[2]))
            if ind2 < n_g:
                lg0, lg1 = np.log(np.float64(g_min)), np.log(np.float64(g_max))
                g_temp = f32(np.exp(lg0 + (lg1 - lg0) * np.float64(f32(ind1 / f32(n_g - 1)))))
                g_max = f32(np.exp(lg0 + (lg1 - lg0) * np.float64(f32(ind2 / f32(n_g - 1)))))
                g_min = g_temp
            else:
                g_max = g_min
                g_min = f32(2 / n)
        else:
            gm, mx = _scores(kc, a)
            kc_max = f32(mx[0])
    with np.errstate(divide="ignore"):
        return float(f32(2) * f32(pixel_size) / kc_max) if kc_max else float("inf")
