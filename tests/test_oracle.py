"""The FP64 oracle pinned by known answers and by literal re-enactments of
individual reference kernels (run on CPU)."""
import json
import os

import numpy as np
import pytest

from isce2_gb300 import synth
from oracle import ampcor_oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def params(H, W, Wh=32, Ww=32, hs=8, skip=24, raw=2, ovs=16, zoom=8, deramp=1):
    return O.OracleParams(referenceImageHeight=H, referenceImageWidth=W, secondaryImageHeight=H,
                          secondaryImageWidth=W, windowSizeHeight=Wh, windowSizeWidth=Ww,
                          halfSearchRangeDown=hs, halfSearchRangeAcross=hs, skipSampleDown=skip,
                          skipSampleAcross=skip, rawDataOversamplingFactor=raw,
                          corrSurfaceOverSamplingFactor=ovs, corrSurfaceZoomInWindow=zoom,
                          derampMethod=deramp, referenceStartPixelDownStatic=hs,
                          referenceStartPixelAcrossStatic=hs,
                          numberWindowDown=(H - 2 * hs - Wh) // skip, numberWindowAcross=(W - 2 * hs - Ww) // skip)


@pytest.mark.parametrize("deramp", [0, 1])
def test_integer_shift_is_exact(deramp):
    n = 200
    sc = synth.make_pair((n, n), d_down=lambda c: 2.0 + 0 * c, d_across=lambda r: -3.0 + 0 * r,
                         snr_db=120.0, seed_ref=1, seed_noise=2)
    p = params(n, n, deramp=deramp)
    out = O.dense_offsets(sc.reference, sc.secondary, p)
    assert (out["offset_init"] == [8 + 2, 8 - 3]).all()
    # amplitude chips (deramp 0) shift exactly; with deramp 1 the reference's
    # per-chip phase estimate and its in-place complex multiply perturb the
    # oversampled amplitudes, which moves the zoom peak by at most one step
    tol = 1e-6 if deramp == 0 else 1.0 / 32 + 1e-6
    np.testing.assert_allclose(out["offset"], np.tile([2.0, -3.0], (out["offset"].shape[0], 1)), atol=tol)


def test_subpixel_shift_recovered_with_complex_oversampling():
    n = 256
    sc = synth.make_pair((n, n), d_down=lambda c: 0.25 + 0 * c, d_across=lambda r: -0.375 + 0 * r,
                         snr_db=60.0, seed_ref=3, seed_noise=4)
    p = params(n, n, Wh=64, Ww=64, hs=12, skip=48, ovs=32, zoom=16, deramp=1)
    out = O.dense_offsets(sc.reference, sc.secondary, p)
    err = out["offset"] - np.array([0.25, -0.375])
    assert np.abs(err.mean(axis=0)).max() < 0.01
    assert np.abs(err).max() < 0.05


def test_constant_field_constant_output():
    n = 200
    sc = synth.make_pair((n, n), d_down=lambda c: 1.0 + 0 * c, d_across=lambda r: 1.0 + 0 * r,
                         snr_db=200.0, seed_ref=5, seed_noise=6)
    out = O.dense_offsets(sc.reference, sc.secondary, params(n, n, deramp=0))
    assert np.ptp(out["offset"], axis=0).max() == 0.0


def _maxloc_literal(img: np.ndarray):
    """cudaKernel_maxloc2D<512> (cuOffset.cu:23-84) step by step: every thread
    scans idx = tid, tid+512, ... keeping the first strictly larger value
    starting from -FLT_MAX, then the shared-memory tree keeps the lower slot
    unless the upper one is strictly larger."""
    B = 512
    fmax = np.finfo(np.float32).max
    shval = [-fmax] * B
    shloc = [0] * B
    for tid in range(B):
        for gid in range(tid, img.size, B):
            if shval[tid] < img[gid]:
                shval[tid] = img[gid]
                shloc[tid] = gid
    s = B // 2
    while s >= 1:
        for tid in range(s):
            if shval[tid] < shval[tid + s]:
                shval[tid] = shval[tid + s]
                shloc[tid] = shloc[tid + s]
        s //= 2
    return shloc[0], shval[0]


@pytest.mark.parametrize("n", [17 * 17, 41 * 41, 3000])
def test_maxloc_tie_rule_matches_reference_tree(n):
    rng = np.random.default_rng(n)
    for trial in range(6):
        v = np.round(rng.standard_normal(n), 1)  # many exact ties
        if trial == 5:
            v[:] = 0.0  # all tied
        if trial == 4:
            v[rng.integers(0, n, 5)] = np.nan
        idx, val = O.maxloc(v[None, :])
        ref_idx, ref_val = _maxloc_literal(v)
        assert idx[0] == ref_idx and val[0] == ref_val


def _padding_literal(X: np.ndarray, m1: int, m2: int) -> np.ndarray:
    """cuArraysPaddingMany_kernel (cuArraysPadding.cu:223-245), one thread at a time."""
    n1, n2 = X.shape
    Y = np.zeros((m1, m2), np.complex128)
    f = 1.0 / (n1 * n2)
    for tx in range(n1 // 2):
        for ty in range(n2 // 2):
            tx1, ty1, tx2, ty2 = n1 - 1 - tx, n2 - 1 - ty, m1 - 1 - tx, m2 - 1 - ty
            Y[tx, ty] = X[tx, ty] * f
            Y[tx2, ty] = X[tx1, ty] * f
            Y[tx, ty2] = X[tx, ty1] * f
            Y[tx2, ty2] = X[tx1, ty1] * f
    return Y


@pytest.mark.parametrize("shape,r", [((8, 6), 2), ((9, 7), 2), ((12, 10), 3), ((16, 16), 4)])
def test_oversampler_matches_literal_padding(shape, r):
    rng = np.random.default_rng(sum(shape))
    x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    X = np.fft.ifft2(x) * x.size
    lit = np.fft.fft2(_padding_literal(X, r * shape[0], r * shape[1]))
    np.testing.assert_allclose(O.oversample_c2c(x[None], r)[0], lit, rtol=0, atol=1e-12)


def test_even_oversampling_keeps_samples():
    rng = np.random.default_rng(0)
    x = rng.standard_normal((1, 10, 12)) + 0j
    y = O.oversample_c2c(x, 2)
    np.testing.assert_allclose(y[0, ::2, ::2], x[0], atol=1e-12)


def test_correlate_and_normalize_against_direct_sums():
    rng = np.random.default_rng(1)
    t = rng.random((2, 6, 5))
    s = rng.random((2, 11, 9))
    t = t - t.mean(axis=(1, 2), keepdims=True)
    c = O.correlate(t, s)
    n = O.normalize(c, t, s)
    for b in range(2):
        for u in range(6):
            for v in range(5):
                blk = s[b, u:u + 6, v:v + 5]
                direct = (t[b] * blk).sum()
                assert abs(c[b, u, v] - direct) < 1e-12
                norm2 = ((blk ** 2).sum() - blk.sum() ** 2 / 30) * (t[b] ** 2).sum()
                assert abs(n[b, u, v] - direct / np.sqrt(norm2 + O.FLT_EPSILON)) < 1e-12


def test_cov_sentinel_and_snr_box():
    corr = np.zeros((1, 9, 9))
    corr[0, 4, 4] = 1.0
    cov = O.estimate_cov(corr, np.array([[0, 4]]), np.array([1.0]), 64)
    assert tuple(cov[0]) == (99.0, 99.0, 0.0)  # peak on the margin
    snr = O.estimate_snr(corr + 0.1, np.array([[4, 4]]), np.array([1.1]), 5, 5)
    # 25 cells, peak 1.1, others 0.1
    assert abs(snr[0] - 1.21 / ((1.21 + 24 * 0.01 - 1.21) / 24)) < 1e-9


def test_adjust_offset_clamp():
    start, shift = O.adjust_offset(20, 2, np.array([0, 1, 2, 20, 38, 40]))
    assert start.tolist() == [0, 0, 0, 18, 36, 36]
    assert shift.tolist() == [2, 1, 0, 0, 0, 2]


@pytest.mark.parametrize("name", ["small_deramp0", "rect_deramp1"])
def test_golden_fixture_regression(name):
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    p = O.OracleParams(**json.loads(str(g["params"])))
    out = O.run_windows(g["reference"], g["secondary"], p, p.constant_gross_starts(0, 0))
    for k in ("offset", "snr", "cov", "offset_init", "zoom_start", "zoom_loc"):
        np.testing.assert_array_equal(out[k], g[k])


def test_check_range_rejects_edge_windows():
    p = params(100, 100, hs=8)
    st = p.constant_gross_starts(0, 0)
    p.check_range(st)
    with pytest.raises(ValueError):
        p.check_range(p.constant_gross_starts(100, 0))
