"""The offset polynomial (``ampcor_offsetpoly``) on the GPU against the oracle.

The device fits in centred, scaled locations and maps back exactly, so its
coefficients are those of the reference's unscaled design matrix; what is
compared: the singular values kept (the reference's 1e-12 truncation, which
large coordinates reach for seven or more terms) exactly, the fitted offsets
at the points to 1e-6 px, and the coefficients to 1e-6 relative where the
fit keeps every singular value of a well-conditioned (at most 6-term) basis.
"""
import numpy as np
import pytest

from isce2_gb300.offsets import Offsetpoly, offsetpoly_device
from oracle import offsetpoly_oracle as orc

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def case(n, seed, spread=(8000, 12000), same_y=False):
    rng = np.random.default_rng(seed)
    x = rng.uniform(0, spread[0], n).round()
    y = rng.uniform(0, spread[1], n).round()
    if same_y:
        y[:] = 5000.0
    z = 0.4 + 2e-4 * x - 1e-4 * y + 1e-8 * x * y + rng.normal(0, 0.05, n)
    snr = rng.gamma(2.0, 4.0, n)
    return x, y, z, snr


def oracle_rank(x, y, snr, ma):
    U = orc.basis(x, y, ma) / (1 + 1 / np.asarray(snr))[:, None]
    s = np.linalg.svd(U, compute_uv=False)
    return int((s >= orc.TOL * s.max()).sum())


def fit(x, y, z, snr, ma):
    d = [torch.as_tensor(np.asarray(a, np.float64), device="cuda") for a in (x, y, z, snr)]
    r = offsetpoly_device(*d, ncoef=ma)
    return r["coef"].cpu().numpy()[:ma], int(r["rank"].item())


LAYOUTS = {"wide": dict(), "narrow": dict(spread=(100, 50)), "one_row": dict(same_y=True)}


@pytest.mark.parametrize("ma", list(range(1, 11)))
@pytest.mark.parametrize("layout", list(LAYOUTS))
def test_offsetpoly_matches_oracle(built_lib, ma, layout):
    x, y, z, snr = case(3000, ma, **LAYOUTS[layout])
    ref = orc.offsetpoly(x, y, z, snr, ma)
    got, rank = fit(x, y, z, snr, ma)
    assert rank == oracle_rank(x, y, snr, ma)
    assert np.abs(orc.evaluate(got, x, y) - orc.evaluate(ref, x, y)).max() <= 1e-6
    if rank == ma and ma <= 6:
        assert np.allclose(got, ref, rtol=1e-6, atol=1e-14)


def test_offsetpoly_large_field_and_zero_snr(built_lib):
    # 2 M offsets; SNR 0 gives weight 0 (sig = +inf), as the reference's
    # division does
    x, y, z, snr = case(2_000_000, 40)
    snr[::97] = 0.0
    ref = orc.offsetpoly(x, y, z, snr, 6)
    got, rank = fit(x, y, z, snr, 6)
    assert rank == 6
    assert np.abs(orc.evaluate(got, x, y) - orc.evaluate(ref, x, y)).max() <= 1e-6
    assert np.allclose(got, ref, rtol=1e-6, atol=1e-14)


def test_fewer_points_than_terms(built_lib):
    x, y, z, snr = case(4, 41)
    ref = orc.offsetpoly(x, y, z, snr, 6)
    got, rank = fit(x, y, z, snr, 6)
    assert rank == oracle_rank(x, y, snr, 6) == 4
    assert np.abs(orc.evaluate(got, x, y) - orc.evaluate(ref, x, y)).max() <= 1e-6


def test_offsetpoly_interface(built_lib):
    x, y, z, snr = case(1000, 42)
    o = Offsetpoly()
    o.setLocationAcross(x.tolist())
    o.setLocationDown(y.tolist())
    o.setOffset(z.tolist())
    o.setSNR(snr.tolist())
    o.setNumberFitCoefficients(4)
    o.offsetpoly()
    assert len(o.offsetPoly) == 4
    assert np.allclose(o.offsetPoly, orc.offsetpoly(x, y, z, snr, 4), rtol=1e-6, atol=1e-14)


def test_offsetpoly_rejects_bad_counts(built_lib):
    d = torch.ones(10, dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError):
        offsetpoly_device(d, d, d, d, ncoef=11)
    e = torch.empty(0, dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError):
        offsetpoly_device(e, e, e, e, ncoef=3)
