"""CPU restatement of ISCE2's offset-polynomial fit (stdproc/offsetpoly).

TEST INFRASTRUCTURE ONLY: the tests and bench's CPU baseline use this module
as the checker; the product path never imports it.

Follows ``offsetpoly.f90:53-84`` and the ``svdfit`` / ``poly_funcs`` it links
(``stdproc/resampLib/src/svd.f:1-40``, ``poly_funcs.f90``):

* weights: sig = 1 + 1/snr (``offsetpoly.f90:58``), rows scaled by 1/sig;
* basis functions of (x = across / range location, y = down / azimuth
  location), the first ``ma`` of: 1, x, y, x y, x^2, y^2, x y^2, x^2 y, x^3,
  y^3 (``poly_funcs.f90``, i_coef(i) = i);
* SVD of the N x ma design matrix, singular values below tol x the largest
  set to zero (tol = 1e-12 as a REAL*4 constant in a real*8 parameter,
  ``svd.f:3``), back-substitution skipping zero singular values.  LAPACK's
  SVD stands in for Numerical Recipes' ``svdcmp``.

The coefficients are those of the unscaled locations, as ``getOffsetPoly``
returns them.
"""
from __future__ import annotations

import numpy as np

TOL = float(np.float32(1e-12))
TERMS = ["1", "x", "y", "xy", "x2", "y2", "xy2", "x2y", "x3", "y3"]


def basis(x: np.ndarray, y: np.ndarray, ma: int) -> np.ndarray:
    """The first ``ma`` basis functions, evaluated as poly_funcs does."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    xy = x * y
    cols = [np.ones_like(x), x, y, xy, x * x, y * y, xy * y, xy * x, x * (x * x), y * (y * y)]
    return np.stack(cols[:ma], axis=1)


def offsetpoly(x, y, off, snr, ma: int = 6) -> np.ndarray:
    if not 1 <= ma <= 10:
        raise ValueError("1 to 10 coefficients")
    sig = 1.0 + 1.0 / np.asarray(snr, np.float64)
    w = 1.0 / sig
    U = basis(x, y, ma) * w[:, None]
    b = np.asarray(off, np.float64) * w
    u, s, vt = np.linalg.svd(U, full_matrices=False)
    s = np.where(s < TOL * s.max(), 0.0, s)
    ub = u.T @ b
    tmp = np.zeros_like(s)
    nz = s != 0.0
    tmp[nz] = ub[nz] / s[nz]
    coef = vt.T @ tmp
    return np.concatenate([coef, np.zeros(ma - coef.shape[0])]) if coef.shape[0] < ma else coef


def evaluate(coef: np.ndarray, x, y) -> np.ndarray:
    """The fitted offsets at (x, y)."""
    return basis(x, y, len(coef)) @ np.asarray(coef, np.float64)
