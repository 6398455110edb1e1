"""Seeded synthetic SLC pairs with a known offset field.

There is no public dataset for dense ampcor; these scenes stand in for real
SLCs with the reference's shapes and value distributions:

* speckle: circular complex Gaussian ``(N(0,1) + i N(0,1)) / sqrt(2)``;
* low-pass to 80 % of the band (2-D FFT bins with ``|f| > 0.4`` cycles/sample
  zeroed on each axis);
* the secondary is the reference moved by an offset field through exact
  band-limited separable shears: a per-row FFT phase ramp moves row ``r`` by
  ``d_r(r)`` across, then a per-column ramp moves column ``c`` by ``d_a(c)``
  down.  The true offset (down, across) of reference pixel (r, c) is then
  ``(d_a(c + d_r(r)), d_r(r))``;
* complex Gaussian noise at a stated SNR (noise power = mean|z|^2 / 10^(SNR/10)).
"""
from __future__ import annotations

import dataclasses
from typing import Callable

import numpy as np
import scipy.fft as sfft


@dataclasses.dataclass
class Scene:
    reference: np.ndarray          # complex64 (H, W)
    secondary: np.ndarray          # complex64 (H, W)
    d_down: Callable               # d_a(col) -> azimuth (down) offset
    d_across: Callable             # d_r(row) -> range (across) offset

    def truth(self, row: np.ndarray, col: np.ndarray):
        """True (down, across) offset at reference pixel (row, col)."""
        dr = self.d_across(np.asarray(row, np.float64))
        da = self.d_down(np.asarray(col, np.float64) + dr)
        return da, dr


def speckle(shape, seed: int, band: float = 0.8) -> np.ndarray:
    rng = np.random.default_rng(seed)
    z = (rng.standard_normal(shape, dtype=np.float32)
         + 1j * rng.standard_normal(shape, dtype=np.float32)).astype(np.complex64)
    z *= np.float32(1.0 / np.sqrt(2.0))
    Z = sfft.fft2(z, workers=-1)
    half = band / 2.0
    Z[np.abs(sfft.fftfreq(shape[0])) > half, :] = 0
    Z[:, np.abs(sfft.fftfreq(shape[1])) > half] = 0
    return sfft.ifft2(Z, workers=-1).astype(np.complex64)


def shear(z: np.ndarray, shifts: np.ndarray, axis: int, block: int = 512) -> np.ndarray:
    """Move each line along ``axis`` by ``shifts[line]`` pixels (content moves
    towards larger index for positive shifts) with an exact FFT phase ramp."""
    out = np.empty_like(z)
    n = z.shape[axis]
    f = sfft.fftfreq(n)
    nlines = z.shape[1 - axis]
    for s0 in range(0, nlines, block):
        sl = slice(s0, min(nlines, s0 + block))
        if axis == 1:
            seg = z[sl, :]
            ramp = np.exp(-2j * np.pi * shifts[sl, None] * f[None, :]).astype(np.complex64)
            out[sl, :] = sfft.ifft(sfft.fft(seg, axis=1, workers=-1) * ramp, axis=1, workers=-1)
        else:
            seg = z[:, sl]
            ramp = np.exp(-2j * np.pi * shifts[None, sl] * f[:, None]).astype(np.complex64)
            out[:, sl] = sfft.ifft(sfft.fft(seg, axis=0, workers=-1) * ramp, axis=0, workers=-1)
    return out


def add_noise(z: np.ndarray, snr_db: float, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    p = float(np.mean(np.abs(z) ** 2)) / (10.0 ** (snr_db / 10.0))
    s = np.float32(np.sqrt(p / 2.0))
    n = (rng.standard_normal(z.shape, dtype=np.float32)
         + 1j * rng.standard_normal(z.shape, dtype=np.float32)).astype(np.complex64)
    return (z + s * n).astype(np.complex64)


def make_pair(shape, d_down: Callable, d_across: Callable, snr_db: float,
              seed_ref: int, seed_noise: int, reference: np.ndarray | None = None) -> Scene:
    H, W = shape
    ref = speckle(shape, seed_ref) if reference is None else reference
    dr = d_across(np.arange(H, dtype=np.float64))
    da = d_down(np.arange(W, dtype=np.float64))
    sec = shear(ref, dr, axis=1)
    sec = shear(sec, da, axis=0)
    sec = add_noise(sec, snr_db, seed_noise)
    return Scene(ref, sec, d_down, d_across)


# --------------------------------------------------------------------------
# the named workloads
# --------------------------------------------------------------------------
def scene_plain_small(n: int = 2048) -> Scene:
    """2048^2 plain case: +1.30 across / -0.70 down plus 0.5 px ramps, 10 dB."""
    return make_pair((n, n),
                     d_down=lambda c: -0.70 + 0.5 * c / (n - 1),
                     d_across=lambda r: 1.30 + 0.5 * r / (n - 1),
                     snr_db=10.0, seed_ref=1, seed_noise=2)


def scene_burst(H: int = 12000, W: int = 8000) -> Scene:
    """12000 x 8000 burst: quadratic field, max 3 px, 5 dB."""
    return make_pair((H, W),
                     d_down=lambda c: -3.0 * (c / (W - 1)) ** 2,
                     d_across=lambda r: 3.0 * (r / (H - 1)) ** 2,
                     snr_db=5.0, seed_ref=11, seed_noise=12)


def scene_precision(n: int = 4096, n_targets: int = 200) -> Scene:
    """60 dB dynamic range: speckle + bright point targets (1e3 x mean) + a
    dark water rectangle (1e-3 x) covering 10 % of the area."""
    z = speckle((n, n), 41)
    m = float(np.mean(np.abs(z)))
    rng = np.random.default_rng(42)
    r = rng.integers(0, n, n_targets)
    c = rng.integers(0, n, n_targets)
    ph = rng.uniform(0, 2 * np.pi, n_targets)
    z[r, c] += (1e3 * m * np.exp(1j * ph)).astype(np.complex64)
    rng = np.random.default_rng(43)
    side = int(np.sqrt(0.1) * n)
    r0, c0 = rng.integers(0, n - side, 2)
    z[r0:r0 + side, c0:c0 + side] *= np.float32(1e-3)
    return make_pair((n, n),
                     d_down=lambda cc: -0.70 + 0.5 * cc / (n - 1),
                     d_across=lambda rr: 1.30 + 0.5 * rr / (n - 1),
                     snr_db=10.0, seed_ref=41, seed_noise=44, reference=z)


def scene_job(seed: int, H: int, W: int, snr_db: float = 10.0) -> Scene:
    """One job of the mixed-size batch: constant U(-3,3) px + ramp U(0,1) px."""
    rng = np.random.default_rng(seed)
    c_d, c_a = rng.uniform(-3, 3, 2)
    r_d, r_a = rng.uniform(0, 1, 2)
    return make_pair((H, W),
                     d_down=lambda c: c_d + r_d * c / max(W - 1, 1),
                     d_across=lambda r: c_a + r_a * r / max(H - 1, 1),
                     snr_db=snr_db, seed_ref=seed, seed_noise=seed + 7919)
