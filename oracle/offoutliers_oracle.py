"""CPU restatement of ISCE2's offset-field outlier culling (Offoutliers) and of
prepareGeometry's nearest-neighbour decimation.

TEST INFRASTRUCTURE ONLY: the tests, ``smoke()`` and bench's CPU baseline use
this module as the checker; the product path never imports it.

Follows, step by step:

* ``Offoutliers.py:268-276`` (``addOffsets``): the SNR pre-cull through
  ``OffsetField.cull`` (``isceobj/Location/Offset.py:364-378``: an offset is
  dropped when its SNR is below the threshold, kept otherwise) and sig = 1.
* ``offoutliers.F:53-77``: two straight-line fits by ``svdfit``
  (``offoutliers.F:165-215``): across shift against across location, down
  shift against down location, basis functions (1, location) (``funcs``,
  ``offoutliers.F:135-163`` with icoef = 1, 2), rows scaled by 1/sig, SVD of
  the design matrix, singular values below tol x the largest set to zero
  (tol = 1e-6, a REAL*4 constant in a real*8 parameter), back-substitution
  skipping zero singular values (``svbksb``, ``offoutliers.F:217-236``).
  LAPACK's SVD stands in for Numerical Recipes' ``svdcmp``: both give the
  singular triplets to working precision.
* ``offoutliers.F:67-68,84-85`` with ``offoutliersState.F``: slope and
  intercept kept as REAL*4.
* ``offoutliers.F:97-118``: perpendicular distances with Fortran's mixed-mode
  rules (REAL*4 x, y, slope, intercept; real*8 locations and shifts; a
  REAL*4 x REAL*4 product stays REAL*4, a REAL*4 with a real*8 operand is
  promoted), each operation rounded on its own (the x86-64 build has no
  fused multiply-add), distances rounded to REAL*4.
* ``offoutliers.F:119-127``: kept where both distances are <= distance
  (REAL*4), 0-based indices in input order.

``decimate`` restates GDAL's nearest-neighbour sampling as prepareGeometry
uses it (``cuDenseOffsets.py:400-460``: ``gdal.Translate`` with a source
window of x_win_num*x_step x y_win_num*y_step pixels onto x_win_num x
y_win_num, noData 0).  GDAL is a third-party dependency absent from the
reference tree; its published rule takes, for output pixel (i, j), the
source pixel under the output pixel's centre, floor(start + (i + 0.5) step),
which for integer steps is start + i*step + step//2.
"""
from __future__ import annotations

import numpy as np

TOL = float(np.float32(1e-6))  # offoutliers.F:167, parameter(tol=1.e-6) in an implicit real*8 unit


def svdfit_line(loc: np.ndarray, z: np.ndarray, sig: np.ndarray) -> np.ndarray:
    """(intercept, slope) of z ~ c0 + c1 loc, svdfit with basis (1, loc)."""
    w = 1.0 / np.asarray(sig, np.float64)
    U = np.stack([w * 1.0, w * np.asarray(loc, np.float64)], axis=1)
    b = np.asarray(z, np.float64) * w
    u, s, vt = np.linalg.svd(U, full_matrices=False)
    wmax = s.max() if s.size else 0.0
    s = np.where(s < TOL * wmax, 0.0, s)
    ub = u.T @ b
    tmp = np.zeros_like(s)
    nz = s != 0.0
    tmp[nz] = ub[nz] / s[nz]
    coef = vt.T @ tmp
    if coef.shape[0] < 2:  # one point: a single singular pair
        coef = np.concatenate([coef, np.zeros(2 - coef.shape[0])])
    return coef


def line_distance(loc: np.ndarray, shift: np.ndarray, slp: np.float32, c: np.float32) -> np.ndarray:
    """offoutliers.F:98-103 in the reference's precisions."""
    f32, f64 = np.float32, np.float64
    slp, c = f32(slp), f32(c)
    loc = np.asarray(loc, f64)
    shift = np.asarray(shift, f64)
    p1 = f32(slp * c)                                   # slpac*cac, REAL*4
    t = (loc - f64(p1)) + f64(slp) * shift              # real*8
    den = f32(f32(1.0) + f32(slp * slp))                # 1+slpac**2, REAL*4
    x = (t / f64(den)).astype(f32)                      # x, REAL*4
    y = (slp * x + c).astype(f32)                       # slpac*x+cac, REAL*4 ops
    dx = x.astype(f64) - loc
    dy = y.astype(f64) - shift
    return np.sqrt(dx * dx + dy * dy).astype(f32)


def offoutliers(loc_across, off_across, loc_down, off_down, distance, sig=None, snr=None, snr_threshold=None,
                fit32=None):
    """Cull an offset field.  Returns a dict: ``index`` (0-based, into the
    input arrays), ``average_across`` / ``average_down`` (REAL*4 intercepts),
    ``fit`` (FP64 across intercept, slope, down intercept, slope), ``fit32``
    (the same as REAL*4), ``distance_across`` / ``distance_down`` (REAL*4, of
    the SNR-kept points, NaN elsewhere).  ``fit32`` given: the distances and
    the selection use those REAL*4 coefficients instead of the fit's (a
    checker's hook for coefficients that round to neighbouring floats)."""
    xa = np.asarray(loc_across, np.float64)
    za = np.asarray(off_across, np.float64)
    xd = np.asarray(loc_down, np.float64)
    zd = np.asarray(off_down, np.float64)
    n = xa.shape[0]
    if n == 0:
        raise ValueError("no offsets to cull")
    sg = np.ones(n) if sig is None else np.asarray(sig, np.float64)
    keep_snr = np.ones(n, bool)
    if snr is not None and snr_threshold is not None:
        keep_snr = ~(np.asarray(snr, np.float64) < float(snr_threshold))
    sel = np.nonzero(keep_snr)[0]
    ca = svdfit_line(xa[sel], za[sel], sg[sel]) if sel.size else np.zeros(2)
    cd = svdfit_line(xd[sel], zd[sel], sg[sel]) if sel.size else np.zeros(2)
    cac, slpac, cdn, slpdn = np.float32(ca[0]), np.float32(ca[1]), np.float32(cd[0]), np.float32(cd[1])
    if fit32 is not None:
        cac, slpac, cdn, slpdn = (np.float32(v) for v in fit32)
    dac = np.full(n, np.nan, np.float32)
    ddn = np.full(n, np.nan, np.float32)
    dac[sel] = line_distance(xa[sel], za[sel], slpac, cac)
    ddn[sel] = line_distance(xd[sel], zd[sel], slpdn, cdn)
    dist = np.float32(distance)
    with np.errstate(invalid="ignore"):
        kept = keep_snr & (dac <= dist) & (ddn <= dist)
    return {"index": np.nonzero(kept)[0].astype(np.int32), "average_across": cac, "average_down": cdn,
            "fit": np.array([ca[0], ca[1], cd[0], cd[1]]), "fit32": np.array([cac, slpac, cdn, slpdn], np.float32),
            "distance_across": dac, "distance_down": ddn}


def decimate(src: np.ndarray, y0: int, x0: int, ystep: int, xstep: int, rows: int, cols: int) -> np.ndarray:
    """Nearest-neighbour decimation onto rows x cols, zero outside ``src``."""
    sy = y0 + np.arange(rows) * ystep + ystep // 2
    sx = x0 + np.arange(cols) * xstep + xstep // 2
    out = np.zeros((rows, cols), src.dtype)
    vy = (sy >= 0) & (sy < src.shape[0])
    vx = (sx >= 0) & (sx < src.shape[1])
    out[np.ix_(vy, vx)] = src[np.ix_(sy[vy], sx[vx])]
    return out
