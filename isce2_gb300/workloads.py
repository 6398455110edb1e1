"""Named workloads beyond the single burst: the uneven batch of many jobs and
the served request stream, plus a device-side scene generator for them.

Both follow the synthetic recipe of ``synth`` (seeded circular complex
Gaussian speckle low-passed to 80 % of the band, exact separable FFT shears
by the offset field, complex Gaussian noise at a stated SNR).  The device
generator draws its speckle with torch's CUDA generator, so its pixels differ
from ``synth``'s NumPy draws for the same seed; the recipe, the sizes and the
value distributions are the same.  It exists because the uneven batch holds
about 90 GB of images, which only the GPU generates in seconds.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

WINDOW_SIDES = (32, 48, 64, 96, 128)
OVS_CHOICES = (16, 32, 64)


@dataclasses.dataclass
class JobSpec:
    """One offset-tracking job: image pair geometry, ampcor parameters and
    the linear offset field d_down(col) = cD + rD col/(W-1),
    d_across(row) = cA + rA row/(H-1)."""
    seed: int
    H: int
    W: int
    Wh: int
    Ww: int
    hs: int
    skipD: int
    skipA: int
    ovs: int
    cD: float
    cA: float
    rD: float
    rA: float
    snr_db: float = 10.0
    raw: int = 2
    zoom: int = 16
    deramp: int = 0

    @property
    def n_down(self) -> int:
        return (self.H - 2 * self.hs - self.Wh) // self.skipD

    @property
    def n_across(self) -> int:
        return (self.W - 2 * self.hs - self.Ww) // self.skipA

    @property
    def windows(self) -> int:
        return max(self.n_down, 0) * max(self.n_across, 0)

    def params(self) -> dict:
        """PyCuAmpcor properties of the job (reference start = half search)."""
        return dict(referenceImageHeight=self.H, referenceImageWidth=self.W, secondaryImageHeight=self.H,
                    secondaryImageWidth=self.W, windowSizeHeight=self.Wh, windowSizeWidth=self.Ww,
                    halfSearchRangeDown=self.hs, halfSearchRangeAcross=self.hs, skipSampleDown=self.skipD,
                    skipSampleAcross=self.skipA, rawDataOversamplingFactor=self.raw,
                    corrSurfaceOverSamplingFactor=self.ovs, corrSurfaceZoomInWindow=self.zoom,
                    derampMethod=self.deramp, referenceStartPixelDownStatic=self.hs,
                    referenceStartPixelAcrossStatic=self.hs, numberWindowDown=self.n_down,
                    numberWindowAcross=self.n_across)

    def d_down(self, col):
        return self.cD + self.rD * col / max(self.W - 1, 1)

    def d_across(self, row):
        return self.cA + self.rA * row / max(self.H - 1, 1)


def _field(rng):
    cD, cA = rng.uniform(-3.0, 3.0, 2)
    rD, rA = rng.uniform(0.0, 1.0, 2)
    return float(cD), float(cA), float(rD), float(rA)


def uneven_jobs(n: int = 256, seed0: int = 1000) -> list[JobSpec]:
    """The uneven batch: job j (seed seed0+j) has sides uniform in
    [1024, 8192], window sides from {32, 48, 64, 96, 128} (height and width
    drawn independently), one half search range uniform in [8, 48] for both
    axes, skips uniform in [16, 128] per axis, correlation oversampling from
    {16, 32, 64}, raw oversampling 2, zoom 16, 10 dB, and a field of a
    constant U(-3, 3) px plus a ramp U(0, 1) px per axis."""
    jobs = []
    for j in range(n):
        rng = np.random.default_rng(seed0 + j)
        H, W = (int(x) for x in rng.integers(1024, 8193, 2))
        Wh, Ww = (int(x) for x in rng.choice(WINDOW_SIDES, 2))
        hs = int(rng.integers(8, 49))
        sD, sA = (int(x) for x in rng.integers(16, 129, 2))
        ovs = int(rng.choice(OVS_CHOICES))
        jobs.append(JobSpec(seed0 + j, H, W, Wh, Ww, hs, sD, sA, ovs, *_field(rng)))
    return jobs


def serving_requests(rate: float, n: int, seed: int = 77, seed0: int = 5_000_000,
                     max_side: int = 16384) -> tuple[np.ndarray, list[JobSpec]]:
    """Poisson arrivals at `rate` requests/s (arrival seed `seed`); request k
    (seed seed0+k) has sides log-uniform in [1024, max_side], a square window
    uniform in [32, 256] rounded to even, a half search uniform in [8, 48],
    skip equal to the window, correlation oversampling 32, zoom 16."""
    arr = np.random.default_rng(seed)
    t = np.cumsum(arr.exponential(1.0 / rate, n))
    jobs = []
    for k in range(n):
        rng = np.random.default_rng(seed0 + k)
        H, W = (int(round(math.exp(x))) for x in rng.uniform(math.log(1024), math.log(max_side), 2))
        w = int(rng.integers(32, 257)) // 2 * 2
        hs = int(rng.integers(8, 49))
        jobs.append(JobSpec(seed0 + k, H, W, w, w, hs, w, w, 32, *_field(rng)))
    return t, jobs


# --------------------------------------------------------------------------
# device-side scene generator (torch on the GPU)
# --------------------------------------------------------------------------
def _speckle_t(H, W, seed, device, band=0.8):
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    z = torch.complex(torch.randn(H, W, generator=g, device=device),
                      torch.randn(H, W, generator=g, device=device))
    z.mul_(1.0 / math.sqrt(2.0))
    Z = torch.fft.fft2(z)
    del z
    half = band / 2.0
    Z[torch.fft.fftfreq(H, device=device).abs() > half, :] = 0
    Z[:, torch.fft.fftfreq(W, device=device).abs() > half] = 0
    return torch.fft.ifft2(Z)


def _shear_t(z, shifts, axis: int, block: int = 2048):
    """Move each line along `axis` by shifts[line] px with an FFT phase ramp."""
    import torch
    n = z.shape[axis]
    f = torch.fft.fftfreq(n, device=z.device, dtype=torch.float64)
    out = torch.empty_like(z)
    nl = z.shape[1 - axis]
    for s0 in range(0, nl, block):
        s1 = min(nl, s0 + block)
        sh = shifts[s0:s1].to(torch.float64)
        if axis == 1:
            ph = (-2.0 * math.pi) * sh[:, None] * f[None, :]
            seg = torch.fft.fft(z[s0:s1, :], dim=1)
            out[s0:s1, :] = torch.fft.ifft(seg * torch.polar(torch.ones_like(ph), ph).to(z.dtype), dim=1)
        else:
            ph = (-2.0 * math.pi) * sh[None, :] * f[:, None]
            seg = torch.fft.fft(z[:, s0:s1], dim=0)
            out[:, s0:s1] = torch.fft.ifft(seg * torch.polar(torch.ones_like(ph), ph).to(z.dtype), dim=0)
    return out


def make_pair_device(spec: JobSpec, device):
    """(reference, secondary) complex64 tensors of the job on `device`."""
    import torch
    H, W = spec.H, spec.W
    ref = _speckle_t(H, W, spec.seed, device)
    rows = torch.arange(H, device=device, dtype=torch.float64)
    cols = torch.arange(W, device=device, dtype=torch.float64)
    sec = _shear_t(ref, spec.d_across(rows), axis=1)
    sec = _shear_t(sec, spec.d_down(cols), axis=0)
    p = float((sec.abs() ** 2).mean()) / (10.0 ** (spec.snr_db / 10.0))
    g = torch.Generator(device=device)
    g.manual_seed(int(spec.seed) + 7919)
    s = math.sqrt(p / 2.0)
    sec.real.add_(torch.randn(H, W, generator=g, device=device), alpha=s)
    sec.imag.add_(torch.randn(H, W, generator=g, device=device), alpha=s)
    return ref.contiguous(), sec.contiguous()
