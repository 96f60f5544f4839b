"""Seeded synthetic blinking-emitter stacks (the input of every workload here).

There is no public dataset on this path: the reference's own tests use a
network-downloaded SMLM dataset that is not available offline, so every
workload is generated here from a fixed recipe:

* ``n_emitters`` point emitters at uniform positions in ``[0, H) x [0, W)``
  (pixel-edge coordinates: pixel ``r`` spans ``[r, r + 1)``);
* each emitter follows a 2-state Markov blink chain, starting OFF, with
  ``p_off_on = 0.05`` and ``p_on_off = 0.5`` per frame;
* an ON emitter contributes ``photons`` (500) photons through a Gaussian PSF of
  ``sigma`` (1.3 px), **pixel-integrated** (the fraction of the Gaussian that
  falls inside each pixel, via ``erf`` differences, over an 11 x 11 patch);
* a flat background of ``background`` (100) photons / pixel;
* Poisson shot noise on the total, then Gaussian read noise N(0, 2^2);
* float32, C-contiguous ``(T, H, W)``.

Everything comes from one ``numpy.random.default_rng(seed)`` stream, so the
same arguments always give bit-identical stacks.
"""
from __future__ import annotations

import math

import numpy as np

__all__ = ["blinking_stack", "emitters_for_density"]

_HALF = 5  # PSF patch half-size (11 x 11 patch, > 3.8 sigma at sigma = 1.3)


def _erf_vec(x: np.ndarray) -> np.ndarray:
    return np.vectorize(math.erf, otypes=[np.float64])(x)


def blinking_stack(T: int, H: int, W: int, n_emitters: int, seed: int = 0, *,
                   photons: float = 500.0, sigma: float = 1.3, background: float = 100.0,
                   read_noise: float = 2.0, p_off_on: float = 0.05, p_on_off: float = 0.5,
                   ) -> np.ndarray:
    """Return a ``(T, H, W)`` float32 stack of blinking emitters (see module doc)."""
    if T < 0 or H < 1 or W < 1:
        raise ValueError("T must be >= 0 and H, W >= 1")
    rng = np.random.default_rng(seed)
    ey = rng.uniform(0.0, H, n_emitters)
    ex = rng.uniform(0.0, W, n_emitters)

    # blink chains: state[t, e]
    state = np.zeros((T, n_emitters), dtype=bool)
    on = np.zeros(n_emitters, dtype=bool)
    u = rng.random((T, n_emitters))
    for t in range(T):
        on = np.where(on, u[t] >= p_on_off, u[t] < p_off_on)
        state[t] = on

    # per-emitter separable pixel-integrated PSF profiles on an 11 x 11 patch
    iy0 = np.floor(ey).astype(np.int64) - _HALF
    ix0 = np.floor(ex).astype(np.int64) - _HALF
    k = np.arange(2 * _HALF + 2, dtype=np.float64)
    s2 = sigma * math.sqrt(2.0)
    edges_y = _erf_vec(((iy0[:, None] + k[None, :]) - ey[:, None]) / s2)
    edges_x = _erf_vec(((ix0[:, None] + k[None, :]) - ex[:, None]) / s2)
    py = 0.5 * np.diff(edges_y, axis=1)          # (E, 11)
    px = 0.5 * np.diff(edges_x, axis=1)          # (E, 11)
    patches = photons * py[:, :, None] * px[:, None, :]   # (E, 11, 11)

    # render the noiseless expectation with a padded canvas, then crop
    pad = _HALF + 1
    out = np.empty((T, H, W), dtype=np.float32)
    canvas = np.empty((H + 2 * pad, W + 2 * pad), dtype=np.float64)
    oy = iy0 + pad
    ox = ix0 + pad
    n = 2 * _HALF + 1
    for t in range(T):
        canvas.fill(background)
        for e in np.nonzero(state[t])[0]:
            canvas[oy[e]:oy[e] + n, ox[e]:ox[e] + n] += patches[e]
        lam = canvas[pad:pad + H, pad:pad + W]
        frame = rng.poisson(lam).astype(np.float64)
        frame += rng.normal(0.0, read_noise, size=(H, W))
        out[t] = frame.astype(np.float32)
    return out


def emitters_for_density(H: int, W: int, density: float) -> int:
    """Emitter count for a density in emitters / px^2 (rounded, at least 1)."""
    return max(1, int(round(density * H * W)))
