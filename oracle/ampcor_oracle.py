"""FP64 NumPy restatement of ISCE2 PyCuAmpcor's dense offset estimator.

TEST INFRASTRUCTURE: this module is the parity oracle.  The product package
never imports it.  Every stage cites the reference file:line it restates
(paths relative to ``contrib/PyCuAmpcor/src`` in ISCE2 2.6.5).  The oracle
computes in float64 where the reference computes in float32 (cuFFT and FP32
kernels); the reference's quirks are reproduced on purpose:

* Q1 swapped half-ranges in the search-chip size (cuAmpcorParameter.cpp:90-91)
  while the secondary start uses hsD down / hsA across (:161,164).
* Q2 deramp method 1 applies the row-derived phase to the column index and
  vice versa (cuDeramp.cu:79-113); Q13 the float2 ``*=`` operator updates the
  real part before using it for the imaginary part (float2.h:71-75).
* Q3 arg-max tie rule of the 512-thread tree reduction (cuOffset.cu:23-63):
  among equal maxima the winner is the one whose ``idx % 512`` has the
  smallest 9-bit bit-reversal, then the smallest ``idx``; NaN never wins.
* Q4 NCC normalisation ``c * rsqrt((S2 - S1^2/n) * R2 + FLT_EPSILON)`` with
  only the reference chip mean-subtracted (cuCorrNormalization.cu:286-312).
* Q5/Q6 spectral zero-padding by moving (h/2, w/2) quadrants to the corners,
  scale 1/(h*w), inverse transform first (cuArraysPadding.cu:223-267,
  cuOverSampler.cpp:72-78).
* Q7 the last row/column of the oversampled correlation is dropped
  (cuAmpcorChunk.cpp:168-169) and the remaining surface is zero-padded to the
  zoom window the R2R oversampler was built for (cuAmpcorChunk.cpp:542-546,
  cuOverSampler.cpp:141-148).
* Q8 SNR box / Q9 covariance sentinels (cuArraysCopy.cu:249-304,
  cuEstimateStats.cu:20-128), Q10 zoom clamp (cuAmpcorParameter.cpp:80-85,
  cuOffset.cu:190-241), Q12 output convention (cuAmpcorController.cpp:129-158).
"""
from __future__ import annotations

import dataclasses
import numpy as np

FLT_EPSILON = float(np.finfo(np.float32).eps)
NTHREADS_MAXLOC = 512  # cudaUtil.h:18, the block size of cudaKernel_maxloc2D


# ---------------------------------------------------------------------------
# parameters and geometry (cuAmpcorParameter.cpp)
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class OracleParams:
    """Subset of cuAmpcorParameter used by the estimator (defaults :18-64)."""
    referenceImageHeight: int = 1000
    referenceImageWidth: int = 1000
    secondaryImageHeight: int = 1000
    secondaryImageWidth: int = 1000
    numberWindowDown: int = 1
    numberWindowAcross: int = 1
    windowSizeHeight: int = 64        # windowSizeHeightRaw
    windowSizeWidth: int = 64         # windowSizeWidthRaw
    halfSearchRangeDown: int = 20
    halfSearchRangeAcross: int = 20
    skipSampleDown: int = 64
    skipSampleAcross: int = 64
    referenceStartPixelDownStatic: int = 0
    referenceStartPixelAcrossStatic: int = 0
    rawDataOversamplingFactor: int = 2
    corrStatWindowSize: int = 21
    corrSurfaceZoomInWindow: int = 16
    corrSurfaceOverSamplingFactor: int = 16
    corrSurfaceOverSamplingMethod: int = 0
    derampMethod: int = 1
    mergeGrossOffset: int = 0

    def derived(self) -> dict:
        """cuAmpcorParameter::setupParameters (cuAmpcorParameter.cpp:70-109)."""
        raw = self.rawDataOversamplingFactor
        hsD, hsA = self.halfSearchRangeDown, self.halfSearchRangeAcross
        Wh, Ww = self.windowSizeHeight, self.windowSizeWidth
        zoom = min(self.corrSurfaceZoomInWindow, min(hsA, hsD) * 2 * raw)
        hz = zoom // (2 * raw)
        d = dict(
            corrRawZoomInHeight=min(self.corrStatWindowSize, 2 * hsD + 1),
            corrRawZoomInWidth=min(self.corrStatWindowSize, 2 * hsA + 1),
            zoom=zoom, hz=hz,
            searchWidthRaw=Ww + 2 * hsD,      # Q1
            searchHeightRaw=Wh + 2 * hsA,     # Q1
            searchWidthZoomIn=Ww + 2 * hz,
            searchHeightZoomIn=Wh + 2 * hz,
        )
        return d

    def constant_gross_starts(self, goD: int, goA: int):
        """setStartPixels(int,int,int,int) (cuAmpcorParameter.cpp:189-205)."""
        nD, nA = self.numberWindowDown, self.numberWindowAcross
        row = np.arange(nD)[:, None]
        col = np.arange(nA)[None, :]
        refD = np.broadcast_to(self.referenceStartPixelDownStatic + row * self.skipSampleDown, (nD, nA))
        refA = np.broadcast_to(self.referenceStartPixelAcrossStatic + col * self.skipSampleAcross, (nD, nA))
        gD = np.full((nD, nA), goD, np.int64)
        gA = np.full((nD, nA), goA, np.int64)
        return self.starts_from(refD, refA, gD, gA)

    def varying_gross_starts(self, gD, gA):
        """setStartPixels(int,int,int*,int*) (cuAmpcorParameter.cpp:170-186)."""
        nD, nA = self.numberWindowDown, self.numberWindowAcross
        row = np.arange(nD)[:, None]
        col = np.arange(nA)[None, :]
        refD = np.broadcast_to(self.referenceStartPixelDownStatic + row * self.skipSampleDown, (nD, nA))
        refA = np.broadcast_to(self.referenceStartPixelAcrossStatic + col * self.skipSampleAcross, (nD, nA))
        return self.starts_from(refD, refA, np.reshape(gD, (nD, nA)), np.reshape(gA, (nD, nA)))

    def starts_from(self, refD, refA, gD, gA):
        """setStartPixels(int*,int*,int*,int*) (cuAmpcorParameter.cpp:155-167)."""
        refD = np.asarray(refD, np.int64).reshape(-1)
        refA = np.asarray(refA, np.int64).reshape(-1)
        gD = np.asarray(gD, np.int64).reshape(-1)
        gA = np.asarray(gA, np.int64).reshape(-1)
        secD = refD + gD - self.halfSearchRangeDown
        secA = refA + gA - self.halfSearchRangeAcross
        return dict(refD=refD, refA=refA, secD=secD, secA=secA, grossD=gD, grossA=gA)

    def check_range(self, st) -> None:
        """checkPixelInImageRange (cuAmpcorParameter.cpp:275-331); raises instead of exit."""
        d = self.derived()
        if (st["refD"] < 0).any() or (st["refA"] < 0).any():
            raise ValueError("reference window start pixel out of range")
        if (st["refD"] + self.windowSizeHeight >= self.referenceImageHeight).any():
            raise ValueError("reference window end pixel out of range in down")
        if (st["refA"] + self.windowSizeWidth >= self.referenceImageWidth).any():
            raise ValueError("reference window end pixel out of range in across")
        if (st["secD"] < 0).any() or (st["secA"] < 0).any():
            raise ValueError("secondary window start pixel out of range")
        if (st["secD"] + d["searchHeightRaw"] >= self.secondaryImageHeight).any():
            raise ValueError("secondary window end pixel out of range in down")
        if (st["secA"] + d["searchWidthRaw"] >= self.secondaryImageWidth).any():
            raise ValueError("secondary window end pixel out of range in across")


# ---------------------------------------------------------------------------
# kernels restated
# ---------------------------------------------------------------------------
def _bitrev9_table() -> np.ndarray:
    t = np.arange(NTHREADS_MAXLOC)
    r = np.zeros_like(t)
    for b in range(9):
        r |= ((t >> b) & 1) << (8 - b)
    return r


_BITREV9 = _bitrev9_table()


def maxloc(vals: np.ndarray):
    """cudaKernel_maxloc2D<512> (cuOffset.cu:23-84) on a batch (B, N).

    Returns (flat index, max value).  Tie rule Q3; NaN never wins; an all-NaN
    surface returns index 0 with -FLT_MAX (the reference leaves the location
    uninitialised there).
    """
    B, N = vals.shape
    v = np.where(np.isnan(vals), -np.inf, vals)
    m = v.max(axis=1)
    idx = np.arange(N, dtype=np.int64)
    key = _BITREV9[idx % NTHREADS_MAXLOC].astype(np.int64) * (N + 1) + idx
    tied = v == m[:, None]
    big = np.iinfo(np.int64).max
    best = np.where(tied, key[None, :], big).argmin(axis=1)
    allnan = ~np.isfinite(m) & (m < 0)
    best = np.where(allnan, 0, best)
    mval = np.where(allnan, -np.finfo(np.float32).max, m)
    return best.astype(np.int64), mval


def second_best_gap(vals: np.ndarray, best: np.ndarray) -> np.ndarray:
    """max - (largest value at any other index): small gaps flag near-ties."""
    v = np.where(np.isnan(vals), -np.inf, vals).copy()
    m = v[np.arange(v.shape[0]), best]
    v[np.arange(v.shape[0]), best] = -np.inf
    return m - v.max(axis=1)


def deramp_method1(x: np.ndarray) -> np.ndarray:
    """cuDerampMethod1_kernel (cuDeramp.cu:67-114) with quirks Q2 and Q13."""
    dY = (x[:, :, :-1] * np.conj(x[:, :, 1:])).sum(axis=(1, 2))
    dX = (x[:, :-1, :] * np.conj(x[:, 1:, :])).sum(axis=(1, 2))
    phaseY = np.arctan2(dY.imag, dY.real)
    phaseX = np.arctan2(dX.imag, dX.real)
    nx, ny = x.shape[1:]
    col = np.arange(ny)[None, None, :]
    row = np.arange(nx)[None, :, None]
    phase = col * phaseX[:, None, None] + row * phaseY[:, None, None]
    c, s = np.cos(phase), np.sin(phase)
    xr = x.real * c - x.imag * s
    xi = x.imag * c + xr * s
    return xr + 1j * xi


def oversample_c2c(x: np.ndarray, r: int) -> np.ndarray:
    """cuOverSamplerC2C::execute (cuOverSampler.cpp:72-78) without deramp.

    INVERSE FFT (unnormalised), quadrant padding with 1/(n1*n2)
    (cuArraysPadding.cu:223-267), FORWARD FFT of the r-times larger grid.
    """
    B, n1, n2 = x.shape
    X = np.fft.ifft2(x) * (n1 * n2)
    m1, m2 = r * n1, r * n2
    h1, h2 = n1 // 2, n2 // 2
    Y = np.zeros((B, m1, m2), np.complex128)
    Y[:, :h1, :h2] = X[:, :h1, :h2]
    Y[:, m1 - h1:, :h2] = X[:, n1 - h1:, :h2]
    Y[:, :h1, m2 - h2:] = X[:, :h1, n2 - h2:]
    Y[:, m1 - h1:, m2 - h2:] = X[:, n1 - h1:, n2 - h2:]
    Y *= 1.0 / (n1 * n2)
    return np.fft.fft2(Y)


def correlate(template: np.ndarray, search: np.ndarray) -> np.ndarray:
    """cuFreqCorrelator::execute (cuCorrFrequency.cu:63-79).

    c(u,v) = sum_ij t(i,j) s(i+u, j+v) for u <= Hs-Ht, v <= Ws-Wt.  The
    reference's circular FFT correlation of the zero-padded template equals
    this exactly because no index wraps; FP64 FFTs keep it to ~1e-15.
    """
    B, th, tw = template.shape
    _, sh, sw = search.shape
    tp = np.zeros((B, sh, sw))
    tp[:, :th, :tw] = template
    c = np.fft.irfft2(np.conj(np.fft.rfft2(tp)) * np.fft.rfft2(search), s=(sh, sw))
    return c[:, : sh - th + 1, : sw - tw + 1]


def normalize(corr: np.ndarray, template: np.ndarray, search: np.ndarray) -> np.ndarray:
    """cuCorrNormalize_kernel (cuCorrNormalization.cu:230-314), in FP64.

    norm2 = (S2 - S1^2 / n) * R2 over each template-sized box of the search
    chip; c *= 1/sqrt(norm2 + FLT_EPSILON).
    """
    B, th, tw = template.shape
    n = th * tw
    R2 = (template * template).sum(axis=(1, 2))
    sat = np.zeros((B, search.shape[1] + 1, search.shape[2] + 1))
    sat2 = np.zeros_like(sat)
    sat[:, 1:, 1:] = search.cumsum(1).cumsum(2)
    sat2[:, 1:, 1:] = (search * search).cumsum(1).cumsum(2)
    U, V = corr.shape[1:]

    def box(s):
        return (s[:, th:th + U, tw:tw + V] - s[:, :U, tw:tw + V]
                - s[:, th:th + U, :V] + s[:, :U, :V])

    S1 = box(sat)
    S2 = box(sat2)
    norm2 = (S2 - S1 * S1 / n) * R2[:, None, None]
    return corr / np.sqrt(norm2 + FLT_EPSILON)


def estimate_cov(corr: np.ndarray, loc: np.ndarray, peak: np.ndarray, templateSize: int) -> np.ndarray:
    """cudaKernel_estimateVar (cuEstimateStats.cu:49-128)."""
    B, NX, NY = corr.shape
    out = np.zeros((B, 3))
    px, py = loc[:, 0], loc[:, 1]
    edge = (px - 1 < 0) | (py - 1 < 0) | (px + 1 >= NX) | (py + 1 >= NY)
    out[:] = (99.0, 99.0, 0.0)
    ok = np.nonzero(~edge)[0]
    if ok.size:
        c = corr[ok]
        x, y = px[ok], py[ok]
        b = np.arange(ok.size)

        def at(dx, dy):
            return c[b, x + dx, y + dy]

        dxx = -(at(1, 0) + at(-1, 0) - 2.0 * at(0, 0))
        dyy = -(at(0, 1) + at(0, -1) - 2.0 * at(0, 0))
        dxy = (at(1, 1) + at(-1, -1) - at(1, -1) - at(-1, 1)) * 0.25
        n2 = np.maximum(1.0 - peak[ok], 0.0)
        dxx = dxx * templateSize
        dyy = dyy * templateSize
        dxy = dxy * templateSize
        n4 = n2 * n2
        n2 = n2 * 2
        n4 = n4 * 0.5 * templateSize
        u = dxy * dxy - dxx * dyy
        u2 = u * u
        small = np.abs(u) < 1e-2
        with np.errstate(divide="ignore", invalid="ignore"):
            cxx = (-n2 * u * dyy + n4 * (dyy * dyy + dxy * dxy)) / u2
            cyy = (-n2 * u * dxx + n4 * (dxx * dxx + dxy * dxy)) / u2
            cxy = (n2 * u * dxy - n4 * (dxx + dyy) * dxy) / u2
        res = np.stack([cxx, cyy, cxy], axis=1)
        res[small] = (99.0, 99.0, 0.0)
        out[ok] = res
    return out


def estimate_snr(corr: np.ndarray, loc: np.ndarray, peak: np.ndarray, outNX: int, outNY: int) -> np.ndarray:
    """cuArraysCopyExtractCorr + cuArraysSumCorr + cudaKernel_estimateSnr
    (cuArraysCopy.cu:249-304, cuCorrNormalization.cu:143-192, cuEstimateStats.cu:20-46)."""
    B, NX, NY = corr.shape
    ox = np.arange(outNX)[None, :, None] + loc[:, 0, None, None] - outNX // 2
    oy = np.arange(outNY)[None, None, :] + loc[:, 1, None, None] - outNY // 2
    valid = (ox >= 0) & (oy >= 0) & (ox < NX) & (oy < NY)
    oxc = np.clip(ox, 0, NX - 1)
    oyc = np.clip(oy, 0, NY - 1)
    b = np.arange(B)[:, None, None]
    vals = np.where(valid, corr[b, oxc, oyc], 0.0)
    s = (vals * vals).sum(axis=(1, 2))
    cnt = valid.sum(axis=(1, 2))
    with np.errstate(divide="ignore", invalid="ignore"):
        mean = (s - peak * peak) / (cnt - 1)
        return peak * peak / mean


def adjust_offset(old_range: int, new_range: int, maxloc_: np.ndarray):
    """dev_adjustOffset (cuOffset.cu:190-224): returns (start, shift)."""
    start = maxloc_ - new_range
    rbound = 2 * (old_range - new_range)
    shift = np.zeros_like(start)
    lo = start < 0
    hi = (~lo) & (start > rbound)
    shift = np.where(lo, -start, np.where(hi, start - rbound, 0))
    start = np.where(lo, 0, np.where(hi, rbound, start))
    return start, shift


def sinc_oversample(surf: np.ndarray, shift: np.ndarray, ovs: int, raw: int, out_n: int) -> np.ndarray:
    """cuSincOverSamplerR2R::execute (cuSincOverSampler.cu:168-195, kernel
    :83-160), in FP64.

    The output is zero except the (4 ovs + 1)^2 points at
    out_n/2 - 2 ovs + i + shift * ovs * raw (the execute call passes
    oversamplingFactor * rawDataOversamplingFactor as the shift multiplier,
    cuAmpcorChunk.cpp:181-184), wrapped once past out_n.  Each is a
    Hamming-weighted sinc (beta 0.75, relative length 6, 4096 phases) sum over
    8 x 8 surface samples with wrapped indices (the row wrap subtracts inNY, as
    the reference does), divided by the sum of the weights.
    """
    i_sincwindow, beta, relfiltlen, decfactor = 2, 0.75, 6.0, 4096
    intplength = int(relfiltlen / beta + 0.5)
    filtercoef = intplength * decfactor
    wgthgt = 0.5
    soff = (filtercoef - 1.0) / 2.0
    i = np.arange(filtercoef + 1, dtype=np.float64)
    wa = i - soff
    wgt = (1.0 - wgthgt) + wgthgt * np.cos(np.pi * wa / soff)
    s = wa * beta / decfactor * np.pi
    with np.errstate(invalid="ignore", divide="ignore"):
        fct = np.where(s != 0.0, np.sin(s) / np.where(s != 0, s, 1.0), 1.0)
    filt = fct * wgt
    B, inNX, inNY = surf.shape
    out = np.zeros((B, out_n, out_n))
    rng = i_sincwindow * ovs
    start = out_n // 2 - rng
    size = 2 * rng + 1
    k = np.arange(intplength)

    def taps(o, n_in, n_wrap):
        # output coordinate -> (input indices, coefficients), per cuSincOverSampler.cu:113-150
        r = o / ovs
        io = r.astype(np.int64)
        frac = ((r - io) * decfactor).astype(np.int64)
        idx = io[:, None] - k[None, :] + intplength // 2
        idx = np.where(idx < 0, idx + n_in, idx)
        idx = np.where(idx >= n_in, idx - n_wrap, idx)
        return idx, filt[k[None, :] * decfactor + frac[:, None]]

    for b in range(B):
        ox = np.arange(size) + start + shift[b, 0] * ovs * raw
        ox = np.where(ox >= out_n, ox - out_n, ox)
        oy = np.arange(size) + start + shift[b, 1] * ovs * raw
        oy = np.where(oy >= out_n, oy - out_n, oy)
        ixs, cxs = taps(ox, inNX, inNY)
        iys, cys = taps(oy, inNY, inNY)
        # acc[a, c] = sum_kl surf[ix[a,k], iy[c,l]] cx[a,k] cy[c,l]
        g = surf[b][ixs[:, :, None, None], iys[None, None, :, :]]      # (size, 8, size, 8)
        w = cxs[:, :, None, None] * cys[None, None, :, :]
        out[b][np.ix_(ox, oy)] = (g * w).sum(axis=(1, 3)) / w.sum(axis=(1, 3))
    return out


# ---------------------------------------------------------------------------
# the per-chunk pipeline (cuAmpcorChunk::run, cuAmpcorChunk.cpp:12-217)
# ---------------------------------------------------------------------------
def _gather(img: np.ndarray, d0: np.ndarray, a0: np.ndarray, h: int, w: int) -> np.ndarray:
    rows = d0[:, None, None] + np.arange(h)[None, :, None]
    cols = a0[:, None, None] + np.arange(w)[None, None, :]
    return img[rows, cols].astype(np.complex128)


def run_windows(ref_img: np.ndarray, sec_img: np.ndarray, p: OracleParams, st: dict,
                sel: np.ndarray | None = None, batch: int | None = None, surfaces: bool = False) -> dict:
    """Run the estimator for the windows ``sel`` (flat indices; all if None).

    ``surfaces`` also returns the normalised raw correlation surface
    (``raw_surface``, after cuCorrNormalize, cuAmpcorChunk.cpp:57) and the
    normalised oversampled one before its last row and column are dropped
    (``os_surface``, cuAmpcorChunk.cpp:161), flattened per window."""
    d = p.derived()
    Wh, Ww = p.windowSizeHeight, p.windowSizeWidth
    hsD, hsA = p.halfSearchRangeDown, p.halfSearchRangeAcross
    raw = p.rawDataOversamplingFactor
    ovs = p.corrSurfaceOverSamplingFactor
    zoom, hz = d["zoom"], d["hz"]
    Hs, Ws = d["searchHeightRaw"], d["searchWidthRaw"]
    Hz, Wz = d["searchHeightZoomIn"], d["searchWidthZoomIn"]
    nwin = st["refD"].size
    sel = np.arange(nwin) if sel is None else np.asarray(sel, np.int64)
    if batch is None:
        per = (zoom * ovs) ** 2 * 16 * 3 + (raw * raw) * Hs * Ws * 16 * 6
        batch = int(max(1, min(512, 4e8 // per)))
    keys = ["offset", "snr", "cov", "offset_init", "zoom_start", "zoom_shift",
            "zoom_loc", "maxval", "raw_gap", "zoom_gap", "zoom_maxval"]
    if surfaces:
        keys += ["raw_surface", "os_surface"]
    outs = {k: [] for k in keys}
    for b0 in range(0, sel.size, batch):
        s = sel[b0:b0 + batch]
        res = _run_batch(ref_img, sec_img, p, st, s, Wh, Ww, hsD, hsA, raw, ovs, zoom, hz, Hs, Ws, Hz, Wz, d)
        for k in outs:
            outs[k].append(res[k])
    return {k: np.concatenate(v, axis=0) for k, v in outs.items()}


def _run_batch(ref_img, sec_img, p, st, s, Wh, Ww, hsD, hsA, raw, ovs, zoom, hz, Hs, Ws, Hz, Wz, d):
    B = s.size
    # loadReferenceChunk / loadSecondaryChunk (cuAmpcorChunk.cpp:260-372)
    ref_c = _gather(ref_img, st["refD"][s], st["refA"][s], Wh, Ww)
    sec_c = _gather(sec_img, st["secD"][s], st["secA"][s], Hs, Ws)
    if p.derampMethod == 0:  # K2 stores (|z|, 0)
        ref_c = np.abs(ref_c) + 0j
        sec_c = np.abs(sec_c) + 0j
    # cuArraysAbs + cuArraysSubtractMean (cuAmpcorChunk.cpp:20-39)
    ref_a = np.abs(ref_c)
    ref_a = ref_a - ref_a.mean(axis=(1, 2), keepdims=True)
    sec_a = np.abs(sec_c)
    # raw correlation + normalisation (:48-60)
    corr = normalize(correlate(ref_a, sec_a), ref_a, sec_a)
    NX, NY = corr.shape[1:]
    flat, peak = maxloc(corr.reshape(B, -1))                       # (:69)
    gap = second_best_gap(corr.reshape(B, -1), flat)
    loc = np.stack([flat // NY, flat % NY], axis=1)
    cov = estimate_cov(corr, loc, peak, Wh * Ww)                    # (:72)
    snr = estimate_snr(corr, loc, peak, d["corrRawZoomInHeight"], d["corrRawZoomInWidth"])  # (:76-90)
    sx, shx = adjust_offset(hsD, hz, loc[:, 0])                     # (:100-106)
    sy, shy = adjust_offset(hsA, hz, loc[:, 1])
    # oversample the reference (deramp inside the oversampler) (:115-126)
    rc = deramp_method1(ref_c) if p.derampMethod == 1 else ref_c
    ref_os = np.abs(oversample_c2c(rc, raw))
    ref_os = ref_os - ref_os.mean(axis=(1, 2), keepdims=True)
    # extract the zoom-in search chip at the clamped start and oversample (:134-137)
    bi = np.arange(B)[:, None, None]
    zr = sx[:, None, None] + np.arange(Hz)[None, :, None]
    zc = sy[:, None, None] + np.arange(Wz)[None, None, :]
    sz = sec_c[bi, zr, zc]
    if p.derampMethod == 1:
        sz = deramp_method1(sz)
    sec_os = np.abs(oversample_c2c(sz, raw))
    # oversampled correlation + normalisation, drop last row/col (:148-169)
    corr_os = normalize(correlate(ref_os, sec_os), ref_os, sec_os)
    zp = corr_os.shape[1] - 1
    adj = corr_os[:, :zp, :corr_os.shape[2] - 1]
    # correlation surface oversampling (:177-186)
    if p.corrSurfaceOverSamplingMethod:
        shifts = np.stack([shx, shy], axis=1)
        surf = sinc_oversample(adj, shifts, ovs, raw, zoom * ovs)
    else:
        pad = np.zeros((B, zoom, zoom), np.complex128)
        pad[:, :adj.shape[1], :adj.shape[2]] = adj
        surf = oversample_c2c(pad, ovs).real
    M = surf.shape[2]
    zflat, zmax = maxloc(surf.reshape(B, -1))                       # (:194)
    zgap = second_best_gap(surf.reshape(B, -1), zflat)
    zloc = np.stack([zflat // M, zflat % M], axis=1)
    # cuSubPixelOffset (cuOffset.cu:137-187): fma(OSratio, loc, start) - hs in FP32
    osr = np.float32(1.0) / np.float32(ovs * raw)
    offx = np.float32(np.float64(osr) * zloc[:, 0] + sx) - np.float32(hsD)
    offy = np.float32(np.float64(osr) * zloc[:, 1] + sy) - np.float32(hsA)
    return dict(
        offset=np.stack([offx, offy], axis=1).astype(np.float32),
        snr=snr.astype(np.float32), cov=cov.astype(np.float32),
        offset_init=loc, zoom_start=np.stack([sx, sy], 1), zoom_shift=np.stack([shx, shy], 1),
        zoom_loc=zloc, maxval=peak, raw_gap=gap, zoom_gap=zgap, zoom_maxval=zmax,
        raw_surface=corr.reshape(B, -1), os_surface=corr_os.reshape(B, -1),
    )


def dense_offsets(ref_img: np.ndarray, sec_img: np.ndarray, p: OracleParams,
                  gross=(0, 0), sel=None) -> dict:
    """Convenience: constant gross offset, all (or selected) windows; applies
    mergeGrossOffset on the host as cuAmpcorController.cpp:145-150 does."""
    st = p.constant_gross_starts(*gross)
    p.check_range(st)
    out = run_windows(ref_img, sec_img, p, st, sel)
    if p.mergeGrossOffset:
        s = np.arange(st["refD"].size) if sel is None else np.asarray(sel)
        out["offset"] = out["offset"] + np.stack([st["grossD"][s], st["grossA"][s]], 1).astype(np.float32)
    return out
