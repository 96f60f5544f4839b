"""Scoring of the eSRRF parameter sweep: ErrorMap (RSP / RSE), FIRECalculator
(FRC resolution), QnR, and the sweep driver that scores every
(sensitivity, radius) pair.

The image-sized work runs in the CUDA library -- Fourier interpolation of the
reference image, Gaussian blurs, float64 moment sums, the 2-D FFTs and ring
sums of the FRC -- while the host keeps the reference's scalar control: the
Brent search over the blur width (the same ``scipy.optimize.brent`` call the
reference makes), the Savitzky-Golay smoothing of the FRC curve and its
threshold crossing, and the logistic QnR map over the (S, R) grid.

Reference (paths inside the NanoPyx tree):
    src/nanopyx/core/transform/error_map.pyx:21-146          ErrorMap
    src/nanopyx/core/analysis/frc.pyx:17-294                 FIRECalculator
    src/nanopyx/core/analysis/pearson_correlation.pyx:44-77  Pearson correlation
    src/nanopyx/core/analysis/parameter_sweep.py:11-139      ParameterSweep
    src/nanopyx/methods/esrrf/parameter_sweep.py:6-81        run_esrrf_parameter_sweep
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _native as N
from ._device import FHT_FULL_SPECTRUM, require_cuda, stream_ptr, workspace

_SUMS = 6  # sx, sy, sxx, sxy, syy, s(x-y)^2 of nx_moment_sums


def _to_device(img) -> tuple[torch.Tensor, bool]:
    """float32 C-contiguous CUDA tensor, and whether the input was a CUDA tensor."""
    dev = require_cuda()
    if isinstance(img, torch.Tensor):
        return img.detach().to(device=dev, dtype=torch.float32).contiguous(), img.is_cuda
    return torch.from_numpy(np.ascontiguousarray(np.asarray(img, dtype=np.float32))).to(dev), False


def gaussian_blur_batch(stack: torch.Tensor, sigmas, index=None, alpha=None,
                       beta=None, float64_sums: bool = False) -> torch.Tensor:
    """scipy.ndimage.gaussian_filter of images of a (B, H, W) CUDA float32 stack
    (mode 'reflect', truncate 4), each with its own sigma: output i blurs image
    ``index[i]`` (default i), of ``alpha[i] * x + beta[i]`` when given (float32)."""
    B, H, W = stack.shape
    n = len(sigmas)
    idx = list(range(n)) if index is None else [int(i) for i in index]
    if any(not 0 <= i < B for i in idx):
        raise IndexError("image index outside the stack")
    out = torch.empty((n, H, W), dtype=torch.float32, device=stack.device)
    if n == 0:
        return out
    L = N.lib()
    ws = workspace(L.nx_gaussian_blur_batch_workspace_bytes(H, W, n), stack.device)
    sig = (C.c_double * n)(*[float(v) for v in sigmas])
    ix = (C.c_int * n)(*idx)
    al = be = None
    if alpha is not None:
        al = (C.c_float * n)(*[float(v) for v in alpha])
        be = (C.c_float * n)(*[float(v) for v in beta])
    N.check(L.nx_gaussian_blur_batch_ex(stack.data_ptr(), H, W, n, C.cast(ix, C.c_void_p),
                                        C.cast(sig, C.c_void_p),
                                        C.cast(al, C.c_void_p) if al is not None else None,
                                        C.cast(be, C.c_void_p) if be is not None else None,
                                        1 if float64_sums else 0, out.data_ptr(),
                                        ws.data_ptr(), ws.numel(), stream_ptr()),
            "Gaussian blur")
    return out


def gaussian_blur(img: torch.Tensor, sigma: float, alpha: float | None = None,
                  beta: float | None = None) -> torch.Tensor:
    """scipy.ndimage.gaussian_filter(img, sigma) of a 2-D CUDA float32 image,
    optionally of ``alpha * img + beta`` (float32)."""
    return gaussian_blur_batch(img[None], [sigma], None,
                               None if alpha is None else [alpha],
                               None if beta is None else [beta])[0]


def moment_sums(x: torch.Tensor, y: torch.Tensor) -> np.ndarray:
    """float64 moments of each image of ``x`` ((B, n) or (n,)) against ``y``
    (n,): (sum x, sum y, Sxx, Sxy, Syy, sum (x-y)^2) with S the second moments
    about the means; returns (B, 6) on the host."""
    xs = x.reshape(-1, y.numel())
    B = xs.shape[0]
    L = N.lib()
    out = torch.empty((B, _SUMS), dtype=torch.float64, device=x.device)
    ws = workspace(L.nx_moment_sums_workspace_bytes(B), x.device)
    N.check(L.nx_moment_sums(xs.data_ptr(), y.data_ptr(), y.numel(), B, out.data_ptr(),
                             ws.data_ptr(), ws.numel(), stream_ptr()), "moment sums")
    return out.cpu().numpy()


def _pearson(s, n: int) -> float:
    """Pearson correlation from the moments; 0 where a variance vanishes
    (pearson_correlation.pyx:60-77)."""
    cxx, cxy, cyy = s[2], s[3], s[4]
    if cxx <= 0 or cyy <= 0:
        return 0.0
    return float(np.float32(cxy / np.sqrt(cxx * cyy)))


def _regression(s, n: int):
    """scipy.stats.linregress(x, y) slope and intercept from the moments, and
    the RMSE of ``slope * x + intercept`` against y."""
    mx, my = s[0] / n, s[1] / n
    cxx, cxy, cyy = s[2], s[3], s[4]
    slope = cxy / cxx if cxx != 0 else np.nan
    intercept = my - slope * mx
    resid = cyy - 2 * slope * cxy + slope * slope * cxx
    return slope, intercept, float(np.sqrt(max(resid, 0.0) / n))


_GOLD = 1.618034       # bracket growth ratio
_GROW_LIMIT = 110.0    # furthest parabolic extrapolation, in bracket widths
_TINY = 1e-21
_CGOLD = 0.3819660     # golden-section fraction
_ZEPS = 1e-11          # absolute tolerance floor
_XTOL = 1.48e-8        # relative tolerance on the minimiser


def _brent_search(brack, maxiter: int = 1000):
    """Brent's minimisation (R. P. Brent, "Algorithms for Minimization without
    Derivatives", 1973, ch. 5, in the form of Numerical Recipes' mnbrak and
    brent) as a generator: it yields each abscissa to evaluate, is sent the
    function value, and returns the minimiser.  The search the reference runs
    through scipy.optimize.brent(f, brack=(a, b)) -- downhill bracketing from
    the two starting points by golden-ratio growth and limited parabolic
    extrapolation, then parabolic steps safeguarded by golden sections, to a
    relative tolerance of 1.48e-8."""
    # bracketing: a, b, c with f(b) below f(a) and f(c)
    a, b = float(brack[0]), float(brack[1])
    fa = yield a
    fb = yield b
    if fb > fa:
        a, b, fa, fb = b, a, fb, fa
    c = b + _GOLD * (b - a)
    fc = yield c
    it = 0
    while fc < fb:
        r = (b - a) * (fb - fc)
        q = (b - c) * (fb - fa)
        den = q - r
        den = 2.0 * (_TINY if abs(den) < _TINY else den)
        u = b - ((b - c) * q - (b - a) * r) / den
        ulim = b + _GROW_LIMIT * (c - b)
        it += 1
        if it > maxiter:
            raise RuntimeError("Too many iterations.")
        if (b - u) * (u - c) > 0.0:  # parabolic minimum between b and c
            fu = yield u
            if fu < fc:
                a, b, fa, fb = b, u, fb, fu
                break
            if fu > fb:
                c, fc = u, fu
                break
            u = c + _GOLD * (c - b)
            fu = yield u
        elif (u - ulim) * (ulim - c) >= 0.0:  # at or beyond the growth limit
            u = ulim
            fu = yield u
        elif (c - u) * (u - ulim) > 0.0:  # between c and the limit
            fu = yield u
            if fu < fc:
                b, c, fb, fc = c, u, fc, fu
                u = c + _GOLD * (c - b)
                fu = yield u
        else:  # parabola useless: grow by the golden ratio
            u = c + _GOLD * (c - b)
            fu = yield u
        a, b, c = b, c, u
        fa, fb, fc = fb, fc, fu
    # Brent's method inside the bracket
    lo, hi = (a, c) if a < c else (c, a)
    x = w = v = b
    fx = fw = fv = fb
    d = e = 0.0
    for _ in range(maxiter):
        xm = 0.5 * (lo + hi)
        tol1 = _XTOL * abs(x) + _ZEPS
        tol2 = 2.0 * tol1
        if abs(x - xm) < tol2 - 0.5 * (hi - lo):
            break
        golden = True
        if abs(e) > tol1:  # try a parabola through x, w, v
            r = (x - w) * (fx - fv)
            q = (x - v) * (fx - fw)
            p = (x - v) * q - (x - w) * r
            q = 2.0 * (q - r)
            if q > 0.0:
                p = -p
            q = abs(q)
            e_prev, e = e, d
            if q * (lo - x) < p < q * (hi - x) and abs(p) < abs(0.5 * q * e_prev):
                d = p / q
                u = x + d
                if u - lo < tol2 or hi - u < tol2:
                    d = tol1 if xm - x >= 0 else -tol1
                golden = False
        if golden:
            e = (lo - x) if x >= xm else (hi - x)
            d = _CGOLD * e
        u = x + d if abs(d) >= tol1 else (x + tol1 if d >= 0 else x - tol1)
        fu = yield u
        if fu > fx:
            if u < x:
                lo = u
            else:
                hi = u
            if fu <= fw or w == x:
                v, w, fv, fw = w, u, fw, fu
            elif fu <= fv or v == x or v == w:
                v, fv = u, fu
        else:
            if u >= x:
                lo = x
            else:
                hi = x
            v, w, x = w, x, u
            fv, fw, fx = fw, fx, fu
    return x


def _lockstep_brent(brackets, evaluate):
    """Brent searches (``_brent_search``) over several objectives at once:
    every step gathers the abscissae all live searches wait on and evaluates
    them in one call, ``evaluate({i: x, ...}) -> {i: f}``, so each step is one
    batch of device work.  Returns the minimisers."""
    gens = [_brent_search(b) for b in brackets]
    out = [None] * len(gens)
    pending = {i: next(g) for i, g in enumerate(gens)}
    while pending:
        vals = evaluate(pending)
        nxt = {}
        for i, f in vals.items():
            try:
                nxt[i] = gens[i].send(float(f))
            except StopIteration as stop:
                out[i] = stop.value
        pending = nxt
    return out


def _reference_interp(ref: torch.Tensor, m: int) -> torch.Tensor:
    """The reference image on the super-resolution grid (_interpolation.pyx's
    full-spectrum Fourier interpolation, as error_map.pyx:52-57 calls it)."""
    if m <= 1:
        return ref
    from .transform import _fht_device

    return _fht_device(ref[None], m, FHT_FULL_SPECTRUM)[0]


def _magnification(ref_shape, sr_shape) -> int:
    m = int(sr_shape[0] / ref_shape[0])
    if m != int(sr_shape[1] / ref_shape[1]):
        raise AssertionError("the magnification differs between the axes")
    return m


def error_maps(ref: torch.Tensor, srs: torch.Tensor, fixed_sigmas=None, ref_int=None):
    """Error maps of several super-resolution images (B, H, W) against one
    reference image (h, w), all on the device; the Brent searches advance in
    lockstep (one batched blur and one batched moment sum per step).

    Returns a dict of per-image lists ``sigma``, ``alpha``, ``beta``, ``rse``,
    ``rsp``, ``evaluations`` and the device tensors ``blurred`` and ``imRSE``
    (B, H, W), and ``ref_int``.
    """
    B, H, W = srs.shape
    m = _magnification(ref.shape, (H, W))
    if ref_int is None:
        ref_int = _reference_interp(ref, m)
    if tuple(ref_int.shape) != (H, W):
        raise ValueError(f"super-resolution image {(H, W)} is not the reference "
                         f"{tuple(ref.shape)} magnified {m}x")
    n = H * W
    y = ref_int.reshape(-1)
    fixed = [0] * B if fixed_sigmas is None else list(fixed_sigmas)
    evals = [0] * B

    def fits(batch):  # {image: sigma} -> {image: (slope, intercept, rmse)}
        keys = list(batch)
        for k in keys:
            evals[k] += 1
        g = gaussian_blur_batch(srs, [batch[k] for k in keys], keys)
        sums = moment_sums(g, y)
        return {k: _regression(sums[j], n) for j, k in enumerate(keys)}

    max_sigma_boundary = (4 / 2.35482) * m
    sig = [f * m for f in fixed]
    search = [i for i in range(B) if fixed[i] == 0]
    if search:
        def objective(batch):  # {search position: sigma} -> {search position: RMSE}
            res = fits({search[p]: x for p, x in batch.items()})
            return {p: res[search[p]][2] for p in batch}

        found = _lockstep_brent([(0, max_sigma_boundary)] * len(search), objective)
        for i, v in zip(search, found):
            sig[i] = v
    for v in sig:
        if abs(v - max_sigma_boundary) < 0.0001:
            print("RSF constrained, as no good minimum found")
    fit = fits({i: sig[i] for i in range(B)})
    # the reference keeps these as C floats
    alpha = [float(np.float32(fit[i][0])) for i in range(B)]
    beta = [float(np.float32(fit[i][1])) for i in range(B)]
    sigma = [float(np.float32(v)) for v in sig]
    blurred = gaussian_blur_batch(srs, sigma, None, alpha, beta)
    sums = moment_sums(blurred, y)
    return dict(sigma=sigma, alpha=alpha, beta=beta,
                rse=[float(np.float32(np.sqrt(sums[i][5] / n))) for i in range(B)],
                rsp=[_pearson(sums[i], n) for i in range(B)], evaluations=evals,
                blurred=blurred, imRSE=(blurred - ref_int).abs_(), ref_int=ref_int)


class ErrorMap:
    """Resolution-scaled error map of a super-resolution image against its
    diffraction-limited reference (error_map.pyx:21-100).

    ``optimise(img_ref, img_sr)`` Fourier-interpolates the reference to the
    super-resolution grid, finds the Gaussian blur width (Brent search of the
    RMSE of the linearly fitted, blurred SR image), and computes the RSE, the
    RSP (Pearson correlation) and the error map ``imRSE``.  NumPy inputs give
    NumPy maps, CUDA tensors give CUDA tensors.
    """

    def __init__(self):
        self._vRSE = 0.0
        self._vRSP = 0.0
        self._alpha = 0.0
        self._beta = 0.0
        self._sigma = 0.0
        self.imRSE = None
        self.img_ref = None
        self.img_sr = None
        self.im_sr_intensity_scaled_blurred = None
        self.n_evaluations = 0

    def optimise(self, img_ref, img_sr, fixedSigma=0) -> None:
        ref, on_dev = _to_device(img_ref)
        sr, _ = _to_device(img_sr)
        if ref.ndim != 2 or sr.ndim != 2:
            raise ValueError("ErrorMap takes 2-D images")
        r = error_maps(ref, sr[None], [fixedSigma])
        self._set(r, 0, ref, sr, on_dev)

    def _set(self, r, i, ref, sr, on_dev):
        self._sigma, self._alpha, self._beta = r["sigma"][i], r["alpha"][i], r["beta"][i]
        self._vRSE, self._vRSP = r["rse"][i], r["rsp"][i]
        self.n_evaluations = r["evaluations"][i]
        conv = (lambda t: t) if on_dev else (lambda t: t.cpu().numpy())
        self.img_ref, self.img_sr = conv(ref), conv(sr)
        self.im_sr_intensity_scaled_blurred = conv(r["blurred"][i])
        self.imRSE = conv(r["imRSE"][i])

    def getRSE(self) -> float:
        return self._vRSE

    def getRSP(self) -> float:
        return self._vRSP

    def get_sigma(self) -> float:
        return self._sigma


class _FrcPlan:
    __slots__ = ("handle", "N")

    def __init__(self, n: int):
        h = C.c_void_p()
        N.check(N.lib().nx_frc_plan_create(C.byref(h), n), "FRC plan")
        self.handle, self.N = h, n

    def __del__(self):
        try:
            if self.handle:
                N.lib().nx_frc_plan_destroy(self.handle)
        except Exception:
            pass


_frc_plans: dict = {}


def _frc_plan(n: int) -> _FrcPlan:
    key = (torch.cuda.current_device(), int(n))
    p = _frc_plans.get(key)
    if p is None:
        if len(_frc_plans) >= 8:
            _frc_plans.pop(next(iter(_frc_plans)))
        p = _frc_plans[key] = _FrcPlan(int(n))
    return p


def _even_square_window(h: int, w: int):
    """Size and origin of the reference's central even-square crop
    (ccm_helper_functions.pyx:37-78)."""
    size = min(w, h)
    if size % 2:
        size -= 1
    return size, (h - size) // 2, (w - size) // 2


def frc_curves(img1: torch.Tensor, img2: torch.Tensor, pixel_size: float = 1.0):
    """Unsmoothed FRC curves (max_r, 3) -- frequency, FRC, samples -- of image
    pairs (P, H, W) on the device, all pairs in one batch of FFTs and ring
    sums; the reference's float32 steps from the ring sums on
    (frc.pyx:150-179)."""
    P, h, w = img1.shape
    if tuple(img2.shape) != (P, h, w):
        raise ValueError("FRC images must have the same shape")
    img1, img2 = img1.contiguous(), img2.contiguous()
    size, r0, c0 = _even_square_window(h, w)
    plan = _frc_plan(size)
    L = N.lib()
    n_rings = L.nx_frc_rings(plan.handle)
    sums = torch.empty((P, n_rings + 1, 4), dtype=torch.float64, device=img1.device)
    ws = workspace(L.nx_frc_workspace_bytes(plan.handle, P), img1.device)
    N.check(L.nx_frc_ring_sums(plan.handle, img1.data_ptr(), img2.data_ptr(), P, h * w, w, r0,
                               c0, sums.data_ptr(), ws.data_ptr(), ws.numel(), stream_ptr()),
            "FRC ring sums")
    s_all = sums.cpu().numpy()
    max_r = size // 2 - 1
    ps = np.float32(pixel_size)
    freq = np.linspace(0, float(np.float32(1) / (np.float32(2) * ps)), max_r, dtype=np.float32)
    curves = []
    for s in s_all:
        res = np.zeros((max_r, 3), dtype=np.float32)
        res[0] = (0, 1, 1)
        with np.errstate(over="ignore", invalid="ignore", divide="ignore"):
            s0 = s[1:max_r, 0].astype(np.float32)
            s1 = s[1:max_r, 1].astype(np.float32)
            s2 = s[1:max_r, 2].astype(np.float32)
            prod = (s1 * s2).astype(np.float32)  # float32 product, as the reference
            res[1:, 1] = (s0.astype(np.float64) / np.sqrt(prod.astype(np.float64))).astype(
                np.float32)
        res[1:, 0] = freq[1:]
        res[1:, 2] = s[1:max_r, 3]
        curves.append(res)
    return curves, size


class FIRECalculator:
    """Fourier ring correlation and its 1/7-threshold resolution (frc.pyx:17-294)."""

    def __init__(self, pixel_size: float = 1, units: str = "pixel"):
        self.pixel_size = float(np.float32(pixel_size))
        self.units = units
        self.threshold = float(np.float32(1 / 7))
        self.fire_number = 0.0
        self.field_of_view = 0
        self.frc_curve = None
        self.threshold_curve = None
        self.intersections = None

    def _frc_curve(self, img1: torch.Tensor, img2: torch.Tensor) -> np.ndarray:
        curves, self.field_of_view = frc_curves(img1[None], img2[None], self.pixel_size)
        return curves[0]

    def _from_curve(self, curve: np.ndarray, size: int) -> float:
        self.field_of_view = size
        self.frc_curve = curve
        self._smooth()
        self.threshold_curve = np.full(self.frc_curve.shape[0], 1.0 / 7.0, dtype=np.float32)
        self._intersections()
        if self.intersections.shape[0] > 0:
            with np.errstate(divide="ignore"):
                self.fire_number = float(np.float32(1) / self.intersections[0, 0])
        else:
            self.fire_number = 0.0
        return self.fire_number

    def _smooth(self):
        from scipy.signal import savgol_filter

        window = int(0.0707 * self.frc_curve.shape[0])
        if 3 >= window:
            window = 4
        self.frc_curve[:, 1] = savgol_filter(self.frc_curve[:, 1], window_length=window,
                                             polyorder=3)

    def _intersections(self):
        f = self.frc_curve
        t = self.threshold_curve
        out = []
        f32 = np.float32
        # segments where the curve crosses the threshold (the reference's test,
        # vectorised), then its float32 intersection arithmetic on those only
        fy = f[:, 1].astype(np.float32)
        ty = np.asarray(t, dtype=np.float32)
        y1v, y2v, y3v, y4v = fy[:-1], fy[1:], ty[:-1], ty[1:]
        cross = ((y3v >= y1v) & (y4v < y2v)) | ((y1v >= y3v) & (y2v < y4v))
        for i in np.nonzero(cross)[0] + 1:
            y1, y2, y3, y4 = f32(f[i - 1, 1]), f32(f[i, 1]), f32(t[i - 1]), f32(t[i])
            x1, x2 = f32(f[i - 1, 0]), f32(f[i, 0])
            x3, x4 = x1, x2
            x1_x2, x3_x4, y1_y2, y3_y4 = x1 - x2, x3 - x4, y1 - y2, y3 - y4
            den = f32(f32(x1_x2 * y3_y4) - f32(y1_y2 * x3_x4))
            if den == 0:
                if y1 == y3:
                    out.append((x1, y1))
            else:
                num = f32(f32(f32(x1 * y2) - f32(y1 * x2)) * x3_x4) - f32(
                    x1_x2 * f32(f32(x3 * y4) - f32(y3 * x4)))
                px = f32(num / den)
                if x1 <= px < x2:
                    mm = f32(f32(y4 - y3) / f32(x2 - x1))
                    c = f32(y3 - f32(mm * x1))
                    out.append((px, f32(f32(mm * px) + c)))
                else:
                    out.append((px, y1))
        self.intersections = np.array(out, dtype=np.float32).reshape(-1, 2)

    def calculate_fire_number(self, img_1, img_2) -> float:
        a, _ = _to_device(img_1)
        b, _ = _to_device(img_2)
        if a.ndim != 2:
            raise ValueError("FRC takes 2-D images")
        curves, size = frc_curves(a[None], b[None], self.pixel_size)
        return self._from_curve(curves[0], size)

    def plot_frc_curve(self):
        import io

        from matplotlib import pyplot as plt

        fig, ax = plt.subplots(dpi=150)
        ax.plot(self.frc_curve[:, 0], self.frc_curve[:, 1])
        ax.axhline(y=1.0 / 7.0, color="r", linestyle="-")
        ax.set_xlabel(f"Spatial frequency [1/{self.units}]")
        ax.set_ylabel("FRC")
        ax.set_title(f"FRC resolution: {np.round(self.fire_number, 1)} {self.units}")
        with io.BytesIO() as buf:
            fig.savefig(buf, format="raw", dpi=150)
            buf.seek(0)
            data = np.frombuffer(buf.getvalue(), dtype=np.uint8)
        w, h = fig.canvas.get_width_height()
        plt.close(fig)
        return data.reshape((int(h), int(w), -1))


def logistic_image_conversion(im, min_val=None, max_val=None):
    """The logistic normalisation of the FRC map (parameter_sweep.py:113-134)."""
    im = np.asarray(im)
    if min_val is None:
        min_val = np.min(im)
    if max_val is None:
        max_val = np.max(im)
    M1, M2 = 0.075, 0.925
    A1 = np.log((1 - M1) / M1)
    A2 = np.log((1 - M2) / M2)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        x0 = (A2 * max_val - A1 * min_val) / (A2 - A1)
        k = 1 / (x0 - max_val) * A1
        return np.asarray([1 / (np.exp(-k * (image - x0)) + 1) for image in im])


def calculate_qnr_score(RSP, FRC):
    """QnR = 2 RSP nFRC / (RSP + nFRC) (parameter_sweep.py:136-139)."""
    RSP, FRC = np.asarray(RSP), np.asarray(FRC)
    if RSP.shape != FRC.shape:
        raise AssertionError("RSP and FRC maps differ in shape")
    nFRC = logistic_image_conversion(FRC)
    with np.errstate(divide="ignore", invalid="ignore"):
        return (2 * RSP * nFRC) / (RSP + nFRC)


class ParameterSweep:
    """The scored eSRRF parameter sweep (parameter_sweep.py:11-139).

    The reconstructions of every (sensitivity, radius) pair -- over all frames,
    the odd frames and the even frames -- run as one batch on the GPU (one RGC
    pass per radius and frame serves up to four sensitivities for AVG); each
    pair is then scored: RSP of the ErrorMap of the all-frames reconstruction
    against the frame mean, FRC resolution of the odd against the even
    reconstruction, and the QnR map over the grid.
    """

    def __init__(self, doErrorMapping: bool = True, doFRCMapping: bool = True):
        self.doErrorMapping = doErrorMapping
        self.doFRCMapping = doFRCMapping
        self.RSP_map = None
        self.FRC_map = None
        self.sigma_map = None

    def calculate_rsp(self, im, reconstruction) -> float:
        em = ErrorMap()
        em.optimise(_frame_mean(_to_device(im)[0]), reconstruction)
        return em.getRSP()

    def calculate_frc(self, im_odd, im_even) -> float:
        return FIRECalculator().calculate_fire_number(im_odd, im_even)

    def _decorr_grid(self, rec_all):
        """Decorrelation resolution of every pair's all-frames reconstruction
        (the whole stack, as the reference's n_frames path also uses)."""
        S, R = rec_all.shape[:2]
        return np.array([[DecorrAnalysis().run_analysis(rec_all[s, r, 0]) for r in range(R)]
                         for s in range(S)])

    def _fire_grid(self, rec_odd, rec_even):
        """FRC resolution of every (sensitivity, radius) pair, one batch."""
        S, R = rec_odd.shape[:2]
        H, W = rec_odd.shape[-2:]
        curves, size = frc_curves(rec_odd[:, :, 0].reshape(S * R, H, W),
                                  rec_even[:, :, 0].reshape(S * R, H, W))
        return np.array([FIRECalculator()._from_curve(c, size) for c in curves]).reshape(S, R)

    def logistic_image_conversion(self, im, min_val=None, max_val=None):
        return logistic_image_conversion(im, min_val, max_val)

    def calculate_qnr_score(self, RSP, FRC):
        return calculate_qnr_score(RSP, FRC)

    def reconstructions(self, stack: torch.Tensor, magnification: int, sensitivity_array,
                        radius_array, temporal_correlation: str = "AVG", frames_per_timepoint=0):
        """(all, odd, even) reconstruction grids, each (S, R, n_tp, H m, W m) on
        the device (all: per timepoint of ``frames_per_timepoint`` frames)."""
        from .engine import EsrrfBatch

        T = stack.shape[0]
        if T < 2:
            raise ValueError("the sweep's FRC needs at least two frames")
        even = stack[0::2].contiguous()
        odd = stack[1::2].contiguous()
        S, R = len(sensitivity_array), len(radius_array)
        b = EsrrfBatch()
        avg_shared = temporal_correlation == "AVG" and frames_per_timepoint == 0
        idx = {}
        groups = [list(sensitivity_array[i:i + 4]) for i in range(0, S, 4)]
        for ri, r in enumerate(radius_array):
            if avg_shared:
                for gi, g in enumerate(groups):
                    for part, st in (("odd", odd), ("even", even)):
                        idx[(part, ri, gi)] = b.add(st, magnification, r, g, 0, "AVG", True,
                                                    False)
            else:
                for si, s in enumerate(sensitivity_array):
                    for part, st, fpt in (("all", stack, frames_per_timepoint), ("odd", odd, 0),
                                          ("even", even, 0)):
                        idx[(part, ri, si)] = b.add(st, magnification, r, s, fpt,
                                                    temporal_correlation, True, False)
        outs = b.run()
        grid = {}
        for part in ("all", "odd", "even"):
            rows = []
            for si in range(S):
                row = []
                for ri in range(R):
                    if avg_shared:
                        if part == "all":
                            continue
                        row.append(outs[idx[(part, ri, si // 4)]][si % 4])
                    else:
                        row.append(outs[idx[(part, ri, si)]][0])
                if row:
                    rows.append(torch.stack(row))
            if rows:
                grid[part] = torch.stack(rows)
        if avg_shared:
            n_e, n_o = even.shape[0], odd.shape[0]
            grid["all"] = ((grid["even"].double() * n_e + grid["odd"].double() * n_o) / T).to(
                torch.float32)
        return grid["all"], grid["odd"], grid["even"]

    def run(self, im, magnification: int, sensitivity_array: list, radius_array: list,
            temporal_correlation: str = "AVG", use_decorr: bool = False, n_frames=None):
        stack, _ = _to_device(im)
        if stack.ndim != 3:
            raise ValueError("the sweep takes a (T, H, W) stack")
        T = stack.shape[0]
        S, R = len(sensitivity_array), len(radius_array)
        fpt = 0 if n_frames is None else int(n_frames)
        rec_all, rec_odd, rec_even = self.reconstructions(
            stack, magnification, list(sensitivity_array), list(radius_array),
            temporal_correlation, fpt)
        RSP_map = np.zeros((S, R))
        FRC_map = np.zeros((S, R))
        if n_frames is None:
            if self.doErrorMapping:
                # one reference interpolation and one lockstep Brent search for
                # the whole grid (the reference repeats both per pair)
                H, W = rec_all.shape[-2:]
                em = error_maps(_frame_mean(stack), rec_all[:, :, 0].reshape(S * R, H, W))
                RSP_map = np.asarray(em["rsp"], dtype=np.float64).reshape(S, R)
                self.sigma_map = np.asarray(em["sigma"]).reshape(S, R)
            if self.doFRCMapping:
                FRC_map = self._decorr_grid(rec_all) if use_decorr else \
                    self._fire_grid(rec_odd, rec_even)
        else:
            n_slices = T // fpt + (1 if T % fpt else 0)
            for s in range(S):
                for r in range(R):
                    # as written in the reference (parameter_sweep.py:53-67), the
                    # per-slice map is re-created for every pair and averaged into
                    # RSP_map, so only the last pair's mean RSP survives
                    slices = np.zeros((n_slices, S, R))
                    if self.doErrorMapping and s == S - 1 and r == R - 1:
                        for i in range(n_slices):
                            em = ErrorMap()
                            em.optimise(_frame_mean(stack[i * fpt:(i + 1) * fpt]),
                                        rec_all[s, r, i])
                            slices[i, s, r] = em.getRSP()
                    if s == S - 1 and r == R - 1:
                        RSP_map = np.mean(slices, axis=0)
            if self.doFRCMapping:
                if use_decorr:  # the whole stack's reconstruction, as the reference
                    full = self.reconstructions(stack, magnification, list(sensitivity_array),
                                                list(radius_array), temporal_correlation, 0)[0]
                    FRC_map = self._decorr_grid(full)
                else:
                    FRC_map = self._fire_grid(rec_odd, rec_even)
            if not self.doErrorMapping:
                RSP_map = np.zeros((S, R))
        self.RSP_map, self.FRC_map = RSP_map, FRC_map
        return self.calculate_qnr_score(RSP_map, FRC_map)


def _frame_mean(stack: torch.Tensor) -> torch.Tensor:
    """numpy.mean(stack, axis=0) of a float32 stack: float32 sums frame by
    frame, then the division (the temporal AVG kernel)."""
    from .transform import calculate_eSRRF_temporal_correlations

    return calculate_eSRRF_temporal_correlations(stack, "AVG")


def run_esrrf_parameter_sweep(img, magnification: int = 2, sensitivities: list = [1, 2],
                              radii: list = [1, 1.5], temporal_correlation: str = "AVG",
                              use_decorr: bool = False, plot_sweep=False, return_qnr=False,
                              n_frames=None):
    """Scored eSRRF parameter sweep (methods/esrrf/parameter_sweep.py:6-81):
    the QnR map over (sensitivities x radii) if ``return_qnr``, else the
    (sensitivity, radius) pair with the highest QnR."""
    out = ParameterSweep().run(img, magnification, sensitivity_array=sensitivities,
                               radius_array=radii, temporal_correlation=temporal_correlation,
                               use_decorr=use_decorr, n_frames=n_frames)
    if plot_sweep:
        from matplotlib import pyplot as plt

        fig, ax = plt.subplots()
        ax.imshow(out, cmap="plasma")
        ax.set_xticks(np.arange(len(radii)), labels=radii)
        ax.set_yticks(np.arange(len(sensitivities)), labels=sensitivities)
        for i in range(len(sensitivities)):
            for j in range(len(radii)):
                ax.text(j, i, round(out[i, j], 2), ha="center", va="center", color="w")
        ax.set_title("Parameter Sweep QnR")
        ax.set_xlabel("Radii")
        ax.set_ylabel("Sensitivities")
        fig.tight_layout()
        plt.show()
    if return_qnr:
        return out
    sens_idx, rad_idx = np.unravel_index(np.argmax(out), out.shape)
    return sensitivities[sens_idx], radii[rad_idx]


def calculate_error_map(img_ref, img_sr):
    """(error map, RSE, RSP) of a super-resolution image against its reference
    (methods/squirrel/error_map.py:5-36)."""
    em = ErrorMap()
    em.optimise(img_ref, img_sr)
    rse_map = em.imRSE
    if isinstance(rse_map, torch.Tensor):
        rse_map = rse_map.cpu().numpy()
    return np.asarray(rse_map, dtype=np.float32), em.getRSE(), em.getRSP()


def calculate_frc(frame_1, frame_2, pixel_size: float = 1, units: str = "pixel",
                  plot_frc_curve: bool = False):
    """FRC resolution of two frames (methods/squirrel/resolution.py:7-44)."""
    fc = FIRECalculator(pixel_size=pixel_size, units=units)
    res = fc.calculate_fire_number(frame_1, frame_2)
    if plot_frc_curve:
        from matplotlib import pyplot as plt

        plt.axis("off")
        plt.subplots_adjust(left=0, right=1, top=1, bottom=0, wspace=0, hspace=0)
        plt.imshow(fc.plot_frc_curve())
        plt.show()
    return res


# ---------------------------------------------------------------------------
# decorrelation analysis (src/nanopyx/core/analysis/decorr.pyx:23-393)
# ---------------------------------------------------------------------------
def _d_curve32(cr, coef, n_r):
    """d(k) = sqrt(2) D_k / (cr sqrt(C_k)) with D, C the running ring sums, in
    the reference's float32 (nan where cr or C_k is 0, d(0) nan -> 0)."""
    f32 = np.float32
    D = np.cumsum(coef[:n_r].astype(np.float32), dtype=np.float32)
    Cc = np.cumsum(coef[n_r:].astype(np.float32), dtype=np.float32)
    crf = f32(np.sqrt(np.float64(f32(cr))))
    with np.errstate(invalid="ignore", divide="ignore"):
        out = (np.sqrt(2.0) * D.astype(np.float64) /
               (np.float64(crf) * np.sqrt(Cc.astype(np.float64)))).astype(np.float32)
    out[(crf == 0) | (Cc == 0)] = np.nan
    if np.isnan(out[0]):
        out[0] = 0
    return out


def _argmax_from(arr, x1, x2):
    i, v = x1, arr[x1]
    for k in range(x1, x2):
        if arr[k] > v:
            i, v = k, arr[k]
    return [i, v]


def _argmin_from(arr, x1, x2):
    i, v = x1, arr[x1]
    for k in range(x1, x2):
        if arr[k] < v:
            i, v = k, arr[k]
    return [i, v]


def _d_corr_max(d, r1, r2, n_r):
    """Peak of a decorrelation curve, walking back from a maximum at the last
    point while it is not 0.001 above the following minimum (decorr.pyx:
    216-246); returns (frequency, amplitude) in float32."""
    f32 = np.float32
    t = np.array(d, dtype=np.float32)
    out = _argmax_from(t, 0, n_r)
    length = len(t)
    while out[0] == length - 1:
        t[length - 1] = 0
        length -= 1
        if length == 0:
            out = [0, f32(0)]
            break
        out = _argmax_from(t, 0, n_r)
        tmin = _argmin_from(t, int(out[0]), length - 1)
        if f32(t[int(out[0])] - tmin[1]) > f32(0.001):
            break
        t[int(out[0])] = tmin[1]
        out[0] = length - 1
    return f32(f32(r1) + f32(f32(f32(r2) - f32(r1)) * f32(out[0])) / f32(n_r - 1)), f32(out[1])


def _best_and_max(kc, a):
    best, gm_max = [0.0, 0.0, 0.0], np.float32(0)
    top, kc_max = [0.0, 0.0, 0.0], np.float32(0)
    for k in range(len(kc)):
        g = np.float32(kc[k] * a[k])
        if g > gm_max:
            gm_max = g
            best = [kc[k], a[k], k]
        if kc[k] > kc_max:
            kc_max = kc[k]
            top = [kc[k], a[k], k]
    return best, top


class DecorrAnalysis:
    """Image decorrelation analysis (Descloux et al.), the reference's
    DecorrAnalysis (decorr.pyx:23-393): resolution = 2 pixel_size / kc_max.

    The image-sized work -- edge apodisation and padding, the Gaussian
    high-pass images (float64 sums rounded to float32, as scipy does: at the
    smallest widths the high-pass image is an exact cancellation), their
    spectra and ring sums -- runs on the GPU, the 2 x n_g high-pass images of
    a refinement round in one batch; the curve maxima and the refinement of
    the band run on the host in the reference's float32.  ``roi`` is accepted
    and, as in the reference, does not change the result (the analysis uses
    the whole image)."""

    def __init__(self, rmin: float = 0, rmax: float = 1, n_r: int = 50, n_g: int = 10,
                 pixel_size: float = 1, units: str = "pixel", roi: tuple = (0, 0, 0, 0)):
        self.rmin = self.rmin2 = float(np.float32(rmin))
        self.rmax = self.rmax2 = float(np.float32(rmax))
        self.n_r, self.n_g = int(n_r), int(n_g)
        self.pixel_size = float(np.float32(pixel_size))
        self.units = units
        self.x0, self.x1, self.y0, self.y1 = roi
        self.d0 = np.zeros(self.n_r, np.float32)
        self.d = np.zeros((self.n_r, 2 * self.n_g), np.float32)
        self.kc = np.zeros(2 * self.n_g, np.float32)
        self.a_g = np.zeros(2 * self.n_g, np.float32)
        self.kc0 = self.a0 = self.kc_gm = self.agm = self.kc_max = self.a_max = 0.0
        self.resolution = 0.0

    def _coefs(self, plan, base, sub, B, zero_dc, crmin, crmax):
        L = N.lib()
        cr = torch.empty(B, dtype=torch.float64, device=base.device)
        coef = torch.empty((B, 2 * self.n_r), dtype=torch.float64, device=base.device)
        ws = workspace(L.nx_decorr_coefs_workspace_bytes(plan.handle, B, self.n_r), base.device)
        N.check(L.nx_decorr_coefs(plan.handle, base.data_ptr(),
                                  sub.data_ptr() if sub is not None else None, B,
                                  1 if zero_dc else 0, float(crmin), float(crmax), self.n_r,
                                  cr.data_ptr(), coef.data_ptr(), ws.data_ptr(), ws.numel(),
                                  stream_ptr()), "decorrelation coefficients")
        return cr.cpu().numpy(), coef.cpu().numpy()

    def run_analysis(self, img):
        f32 = np.float32
        t, _ = _to_device(img)
        if t.ndim != 2:
            raise ValueError("decorrelation analysis takes a 2-D image")
        h, w = t.shape
        n = 1 << int(np.ceil(np.log(max(h, w)) / np.log(2.0)))
        L = N.lib()
        temp = torch.empty((n, n), dtype=torch.float32, device=t.device)
        ws = workspace(L.nx_decorr_prepare_workspace_bytes(h, w), t.device)
        N.check(L.nx_decorr_prepare(t.data_ptr(), h, w, temp.data_ptr(), n, ws.data_ptr(),
                                    ws.numel(), stream_ptr()), "decorrelation image")
        plan = _frc_plan(n)
        n_r, n_g = self.n_r, self.n_g
        cr, coef = self._coefs(plan, temp, None, 1, True, self.rmin, self.rmax)
        self.d0 = _d_curve32(cr[0], coef[0], n_r)
        self.kc0, self.a0 = _d_corr_max(self.d0, 0, 1, n_r)
        g_max = f32(n // 2) if self.kc0 == 0 else f32(f32(2) / self.kc0)
        g_min = f32(0.14)
        crmin, crmax = f32(self.rmin), f32(self.rmax)
        d_curve = np.zeros((n_r, 2 * n_g), np.float32)
        for refine in range(2):
            lg0, lg1 = np.log(np.float64(g_min)), np.log(np.float64(g_max))
            sig = [float(np.exp(lg0 + (lg1 - lg0) * np.float64(f32(f32(k) / f32(n_g - 1)))))
                   for k in range(n_g)]
            blurred = gaussian_blur_batch(temp[None], sig, [0] * n_g, float64_sums=True)
            crs, coefs = self._coefs(plan, temp, blurred, n_g, False, crmin, crmax)
            kc, a = [], []
            for k in range(n_g):
                d_curve[:, refine * n_g + k] = _d_curve32(crs[k], coefs[k], n_r)
                r = _d_corr_max(d_curve[:, refine * n_g + k], crmin, crmax, n_r)
                kc.append(r[0])
                a.append(r[1])
                self.kc[k], self.a_g[k] = r
            if refine == 0:
                r0 = _d_corr_max(self.d0, crmin, crmax, n_r)
                kc.append(r0[0])
                a.append(r0[1])
                self.kc[n_g], self.a_g[n_g] = r0
                gm, mx = _best_and_max(kc, a)
                crmin = f32(max(f32(np.float64(min(gm[0], mx[0])) - 0.05), f32(self.rmin)))
                crmax = f32(min(f32(np.float64(max(gm[0], mx[0])) + 0.3), f32(self.rmax)))
                self.rmin2, self.rmax2 = float(crmin), float(crmax)
                ind1 = f32(min(gm[2], mx[2]) - 1)
                ind2 = f32(max(gm[2], mx[2]))
                if ind2 < n_g:
                    g_temp = f32(np.exp(lg0 + (lg1 - lg0) * np.float64(f32(ind1 / f32(n_g - 1)))))
                    g_max = f32(np.exp(lg0 + (lg1 - lg0) * np.float64(f32(ind2 / f32(n_g - 1)))))
                    g_min = g_temp
                else:
                    g_max = g_min
                    g_min = f32(2 / n)
            else:
                gm, mx = _best_and_max(kc, a)
                self.kc_gm, self.agm = float(gm[0]), float(gm[1])
                self.kc_max, self.a_max = float(mx[0]), float(mx[1])
        self.d = d_curve
        with np.errstate(divide="ignore"):
            # every kc 0: the reference divides by a value it never set (its
            # result varies run to run); here 2 pixel_size / 0 = inf
            self.resolution = float(f32(2) * f32(self.pixel_size) / f32(self.kc_max)) \
                if self.kc_max else float("inf")
        return self.resolution


def calculate_decorr_analysis(frame, rmin: float = 0.0, rmax: float = 1.0, n_r: int = 50,
                              n_g: int = 10, pixel_size: float = 1, units: str = "pixel",
                              roi: tuple = (0, 0, 0, 0), plot_decorr_analysis: bool = False):
    """Decorrelation resolution of a frame (methods/squirrel/resolution.py:47-104)."""
    dc = DecorrAnalysis(rmin=rmin, rmax=rmax, n_r=n_r, n_g=n_g, pixel_size=pixel_size,
                        units=units, roi=roi)
    dc.run_analysis(frame)
    if plot_decorr_analysis:
        raise NotImplementedError("plotting needs matplotlib")
    return dc.resolution
