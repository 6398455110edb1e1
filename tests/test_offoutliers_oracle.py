"""The culling and decimation oracle against known answers, and the host
logic without a GPU: Offoutliers' SNR pre-cull and argument checks, the
geometry raster writer and reader."""
import numpy as np
import pytest

from isce2_gb300.offsets import Offoutliers, RefinedOffset
from oracle.offoutliers_oracle import decimate, line_distance, offoutliers, svdfit_line


def line_field(n_side=40, seed=0):
    """Points exactly on two lines (across shift = 0.5 + 1e-4 x, down shift =
    -0.3 + 2e-4 y) plus outlier pairs at +-500 px above / below the same
    point, which leave the least-squares lines where they are."""
    rng = np.random.default_rng(seed)
    ya, xa = np.meshgrid(np.arange(n_side) * 64.0 + 100, np.arange(n_side) * 48.0 + 80, indexing="ij")
    xa, ya = xa.ravel(), ya.ravel()
    za = 0.5 + 1e-4 * xa
    zd = -0.3 + 2e-4 * ya
    out = rng.choice(xa.size, 30, replace=False)
    X = np.concatenate([xa, xa[out], xa[out]])
    Y = np.concatenate([ya, ya[out], ya[out]])
    ZA = np.concatenate([za, za[out] + 500, za[out] - 500])
    ZD = np.concatenate([zd, zd[out] - 500, zd[out] + 500])
    return X, ZA, Y, ZD, xa.size


def test_line_fit_known_answer():
    X, ZA, Y, ZD, n_in = line_field()
    ca = svdfit_line(X, ZA, np.ones_like(X))
    cd = svdfit_line(Y, ZD, np.ones_like(Y))
    assert abs(ca[0] - 0.5) < 1e-9 and abs(ca[1] - 1e-4) < 1e-12
    assert abs(cd[0] + 0.3) < 1e-9 and abs(cd[1] - 2e-4) < 1e-12


def test_outlier_pairs_are_culled_and_inliers_kept():
    X, ZA, Y, ZD, n_in = line_field()
    r = offoutliers(X, ZA, Y, ZD, distance=10.0)
    assert np.array_equal(r["index"], np.arange(n_in))  # offoutliers.F:119-127: input order, 0-based
    assert r["average_across"] == np.float32(r["fit"][0]) and r["average_down"] == np.float32(r["fit"][2])
    assert np.nanmax(r["distance_across"][:n_in]) < 1e-3
    assert np.nanmin(r["distance_across"][n_in:]) > 400


def test_single_location_gives_minimum_norm_line():
    # every point at across location X: the design matrix has rank one, its
    # small singular value falls below 1e-6 of the large one and svbksb
    # keeps the minimum-norm solution (1, X) zbar / (1 + X^2)
    X = np.full(50, 1234.0)
    z = np.linspace(-1, 1, 50) + 0.7
    c = svdfit_line(X, z, np.ones_like(X))
    zbar = z.mean()
    assert np.allclose(c, [zbar / (1 + X[0] ** 2), zbar * X[0] / (1 + X[0] ** 2)], rtol=1e-12)


def test_weights_are_inverse_sigmas():
    rng = np.random.default_rng(3)
    x = rng.uniform(0, 5000, 400)
    z = 1.5 - 3e-4 * x + rng.normal(0, 0.05, 400)
    sig = rng.uniform(0.5, 2.0, 400)
    c = svdfit_line(x, z, sig)
    w = 1 / sig
    A = np.stack([w, w * x], 1)
    ref = np.linalg.solve(A.T @ A, A.T @ (w * z))
    assert np.allclose(c, ref, rtol=1e-10, atol=1e-13)


def test_distance_is_the_perpendicular_distance_to_float_precision():
    rng = np.random.default_rng(4)
    x = rng.uniform(0, 8000, 1000)
    z = rng.uniform(-20, 20, 1000)
    slp, c = np.float32(2.5e-4), np.float32(-0.75)
    d = line_distance(x, z, slp, c)
    exact = np.abs(z - (float(slp) * x + float(c))) / np.sqrt(1 + float(slp) ** 2)
    # REAL*4 foot points of locations up to 8000 are good to ~5e-4
    assert np.allclose(d, exact, atol=2e-3)


def test_snr_precull_drops_below_threshold_only():
    X, ZA, Y, ZD, n_in = line_field(10)
    snr = np.full(X.size, 5.0)
    snr[[3, 7]] = 1.0
    snr[5] = 2.0  # equal to the threshold: kept (OffsetField.cull drops snr < threshold)
    r = offoutliers(X, ZA, Y, ZD, distance=10.0, snr=snr, snr_threshold=2.0)
    assert 3 not in r["index"] and 7 not in r["index"] and 5 in r["index"]


def test_decimate_known_answer():
    src = np.arange(20 * 30, dtype=np.float32).reshape(20, 30)
    out = decimate(src, 2, 3, 4, 5, 6, 7)
    for i in range(6):
        for j in range(7):
            sy, sx = 2 + 4 * i + 2, 3 + 5 * j + 2
            want = src[sy, sx] if sy < 20 and sx < 30 else 0
            assert out[i, j] == want


def test_offoutliers_port_applies_the_snr_threshold():
    offs = [RefinedOffset(10.0 * k, 5.0 * k, 0.1, -0.2, snr) for k, snr in enumerate([5, 1, 2, 0.5, 3])]
    o = Offoutliers()
    o.wireInputPort(name="offsets", object=offs)
    o.setSNRThreshold(2.0)
    o.addOffsets()
    assert o.locationAcross == [0.0, 20.0, 40.0] and o.snr == [5, 2, 3] and o.sig == [1.0] * 3


def test_offoutliers_rejects_an_empty_field():
    o = Offoutliers()
    o.setDistance(10)
    with pytest.raises(Exception, match="zero size"):
        o.offoutliers()


@pytest.mark.parametrize("dtype", [np.uint8, np.int16, np.float32, np.float64])
def test_raster_writer_and_reader_round_trip(tmp_path, dtype):
    from isce2_gb300.offsets import read_vrt_bands, write_raster

    rng = np.random.default_rng(5)
    bands = [(rng.random((13, 17)) * 100).astype(dtype) for _ in range(3)]
    path = str(tmp_path / "geom.rdr")
    write_raster(path, bands)
    got = read_vrt_bands(path + ".vrt")
    assert len(got) == 3 and all(g.dtype == b.dtype and np.array_equal(g, b) for g, b in zip(got, bands))
    hdr = open(path + ".hdr").read()
    assert "interleave = bsq" in hdr and "bands = 3" in hdr and "samples = 17" in hdr and "lines = 13" in hdr


def test_raster_reader_rejects_a_short_file(tmp_path):
    from isce2_gb300.offsets import read_vrt_bands, write_raster

    path = str(tmp_path / "lat.rdr")
    write_raster(path, [np.zeros((8, 8), np.float64)])
    with open(path, "r+b") as f:
        f.truncate(100)
    with pytest.raises(ValueError, match="too short"):
        read_vrt_bands(path + ".vrt")
