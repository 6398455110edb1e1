"""Offset-field culling and geometry decimation on the GPU against the oracle.

Culling (``ampcor_offoutliers``): the kept indices equal the oracle's
exactly and the REAL*4 averages are equal.  The FP64 line fits agree to
1e-9 relative (normal equations on the GPU, an SVD in the oracle).  If a
coefficient rounds to the neighbouring float (the two fits straddle a
rounding boundary), the selection is checked against the oracle evaluated
with the GPU's REAL*4 coefficients.  Decimation (``ampcor_decimate``) is a
copy, so it is bit-exact for every element size.
"""
import os

import numpy as np
import pytest

from isce2_gb300 import PyCuAmpcor, synth
from isce2_gb300.offsets import (Offoutliers, RefinedOffset, cull_offset_field, decimate, offoutliers_device,
                                 prepare_geometry, read_vrt_bands)
from oracle import offoutliers_oracle as orc

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def field(n, seed, outlier_frac=0.05, spread=8000.0):
    rng = np.random.default_rng(seed)
    xa = rng.uniform(0, spread, n).round()
    xd = rng.uniform(0, spread * 1.5, n).round()
    za = 1.25 + 3e-4 * xa + rng.normal(0, 0.2, n)
    zd = -0.6 - 1e-4 * xd + rng.normal(0, 0.2, n)
    bad = rng.random(n) < outlier_frac
    za[bad] += rng.uniform(-40, 40, bad.sum())
    zd[bad] += rng.uniform(-40, 40, bad.sum())
    snr = rng.gamma(2.0, 3.0, n).astype(np.float32)
    return xa, za, xd, zd, snr


def on_gpu(*arrs):
    return [None if a is None else torch.as_tensor(a, device="cuda") for a in arrs]


def check(got, xa, za, xd, zd, distance, sig=None, snr=None, thr=None):
    ref = orc.offoutliers(xa, za, xd, zd, distance, sig=sig, snr=snr, snr_threshold=thr)
    fit = got["fit"].cpu().numpy()
    assert np.allclose(fit, ref["fit"], rtol=1e-9, atol=1e-12), (fit, ref["fit"])
    g32 = fit.astype(np.float32)
    if not np.array_equal(g32, ref["fit32"]):
        # neighbouring floats only; the selection then follows the GPU's REAL*4 coefficients
        ulps = np.abs(g32.view(np.int32).astype(np.int64) - ref["fit32"].view(np.int32).astype(np.int64))
        assert ulps.max() <= 1, (g32, ref["fit32"])
        ref = orc.offoutliers(xa, za, xd, zd, distance, sig=sig, snr=snr, snr_threshold=thr, fit32=g32)
    cnt = int(got["count"].item())
    idx = got["index"][:cnt].cpu().numpy()
    assert np.array_equal(idx, ref["index"]), (cnt, ref["index"].size)
    assert got["average_across"].item() == ref["average_across"]
    assert got["average_down"].item() == ref["average_down"]
    return ref


@pytest.mark.parametrize("n,seed", [(1, 0), (2, 1), (37, 2), (1000, 3), (22632, 4), (1_000_003, 5)])
def test_cull_matches_oracle(built_lib, n, seed):
    xa, za, xd, zd, _ = field(n, seed)
    g = offoutliers_device(*on_gpu(xa, za, xd, zd), distance=3.0)
    ref = check(g, xa, za, xd, zd, 3.0)
    if n >= 1000:
        assert 0 < ref["index"].size < n  # the case culls something and keeps something


def test_cull_with_sigmas_and_snr_threshold(built_lib):
    xa, za, xd, zd, snr = field(50_000, 11)
    sig = np.random.default_rng(12).uniform(0.5, 3.0, xa.size)
    xa_d, za_d, xd_d, zd_d, sig_d, snr_d = on_gpu(xa, za, xd, zd, sig, snr)
    g = offoutliers_device(xa_d, za_d, xd_d, zd_d, distance=2.5, sig=sig_d, snr=snr_d, snr_threshold=2.0)
    check(g, xa, za, xd, zd, 2.5, sig=sig, snr=snr, thr=2.0)


def test_cull_single_column_is_rank_deficient(built_lib):
    # every offset at one across location: the across fit keeps one singular
    # value (the minimum-norm line), as svdfit's threshold does
    xa, za, xd, zd, _ = field(3000, 13)
    xa[:] = 4321.0
    g = offoutliers_device(*on_gpu(xa, za, xd, zd), distance=4.0)
    check(g, xa, za, xd, zd, 4.0)


def test_cull_is_reproducible(built_lib):
    xa, za, xd, zd, snr = field(200_000, 14)
    args = on_gpu(xa, za, xd, zd)
    a = offoutliers_device(*args, distance=3.0)
    b = offoutliers_device(*args, distance=3.0)
    assert torch.equal(a["fit"], b["fit"]) and torch.equal(a["index"][:int(a["count"].item())],
                                                           b["index"][:int(b["count"].item())])


def test_cull_rejects_empty_field(built_lib):
    e = torch.empty(0, dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError):
        offoutliers_device(e, e, e, e, distance=1.0)


def test_offoutliers_interface_matches_oracle(built_lib):
    xa, za, xd, zd, snr = field(5000, 15)
    offs = [RefinedOffset(float(xa[k]), float(xd[k]), float(za[k]), float(zd[k]), float(snr[k]))
            for k in range(xa.size)]
    o = Offoutliers()
    o.wireInputPort(name="offsets", object=offs)
    o.setSNRThreshold(2.0)
    o.setDistance(3)
    o.offoutliers()
    keep = ~(snr.astype(np.float64) < 2.0)
    ref = orc.offoutliers(xa[keep], za[keep], xd[keep], zd[keep], 3.0)
    assert o.getIndexArray() == ref["index"].tolist()  # indices into the SNR-kept list, as the reference's
    assert o.getAverageOffsetAcross() == float(ref["average_across"])
    assert o.getAverageOffsetDown() == float(ref["average_down"])
    loc = o.getRefinedLocations()
    assert loc[0] == xa[keep][ref["index"]].tolist() and loc[4] == [float(s) for s in snr[keep][ref["index"]]]
    assert len(o.getRefinedOffsetField()) == ref["index"].size


def test_dense_field_from_pycuampcor(built_lib):
    # a PyCuAmpcor run's offset field culled where it lies, against the
    # oracle culling the same field copied to the host
    n = 1024
    sc = synth.make_pair((n, n), d_down=lambda c: -0.7 + 2e-4 * c, d_across=lambda r: 1.3 - 1e-4 * r,
                         snr_db=5.0, seed_ref=21, seed_noise=22)
    obj = PyCuAmpcor()
    kw = dict(referenceImageHeight=n, referenceImageWidth=n, secondaryImageHeight=n, secondaryImageWidth=n,
              windowSizeHeight=64, windowSizeWidth=64, halfSearchRangeDown=20, halfSearchRangeAcross=20,
              skipSampleDown=32, skipSampleAcross=32, rawDataOversamplingFactor=2,
              corrSurfaceOverSamplingFactor=16, corrSurfaceZoomInWindow=8, derampMethod=0,
              referenceStartPixelDownStatic=20, referenceStartPixelAcrossStatic=20,
              numberWindowDown=28, numberWindowAcross=28)
    for k, v in kw.items():
        setattr(obj, k, v)
    obj.setupParams()
    obj.setConstantGrossOffset(0, 0)
    obj.checkPixelInImageRange()
    ref_d = torch.from_numpy(sc.reference).cuda()
    sec_d = torch.from_numpy(sc.secondary).cuda()
    out = obj.run_device(ref_d, sec_d)
    loc_d = 20 + 32 * np.arange(28) + 32.0
    loc_a = 20 + 32 * np.arange(28) + 32.0
    g = cull_offset_field(out["offset"], out["snr"], loc_d, loc_a, distance=0.5, snr_threshold=2.0)
    off = out["offset"].cpu().numpy().reshape(-1, 2).astype(np.float64)
    snr = out["snr"].cpu().numpy().reshape(-1)
    LD, LA = np.meshgrid(loc_d, loc_a, indexing="ij")
    check(g, LA.ravel(), off[:, 1], LD.ravel(), off[:, 0], 0.5, snr=snr, thr=2.0)


@pytest.mark.parametrize("dtype", [np.uint8, np.int16, np.float32, np.float64])
def test_decimate_matches_oracle(built_lib, dtype):
    rng = np.random.default_rng(30)
    src = (rng.random((517, 389)) * 200).astype(dtype)
    full = torch.as_tensor(src, device="cuda")
    for (y0, x0, ys, xs, rows, cols) in [(0, 0, 8, 4, 64, 97), (13, 7, 16, 16, 33, 25), (5, 3, 3, 5, 200, 90)]:
        got = decimate(full, y0, x0, ys, xs, rows, cols).cpu().numpy()
        assert np.array_equal(got, orc.decimate(src, y0, x0, ys, xs, rows, cols))
    # a column window of a wider raster (row stride above the width)
    view = full[:, 50:300]
    got = decimate(view, 2, 1, 6, 6, 90, 45).cpu().numpy()
    assert np.array_equal(got, orc.decimate(src[:, 50:300], 2, 1, 6, 6, 90, 45))


def write_band_vrt(path, dtype_name, arrs):
    """raw BIL file of the bands + a VRTRawRasterBand header"""
    H, W = arrs[0].shape
    isz = arrs[0].dtype.itemsize
    np.stack(arrs, axis=1).tofile(path)
    with open(path + ".vrt", "w") as f:
        f.write(f'<VRTDataset rasterXSize="{W}" rasterYSize="{H}">\n')
        for k in range(len(arrs)):
            f.write(f'  <VRTRasterBand dataType="{dtype_name}" band="{k + 1}" subClass="VRTRawRasterBand">\n'
                    f'    <SourceFilename relativeToVRT="1">{os.path.basename(path)}</SourceFilename>\n'
                    f'    <ImageOffset>{k * W * isz}</ImageOffset>\n    <PixelOffset>{isz}</PixelOffset>\n'
                    f'    <LineOffset>{len(arrs) * W * isz}</LineOffset>\n    <ByteOrder>LSB</ByteOrder>\n'
                    f'  </VRTRasterBand>\n')
        f.write("</VRTDataset>\n")


def test_prepare_geometry_files(built_lib, tmp_path):
    rng = np.random.default_rng(31)
    full = tmp_path / "full"
    full.mkdir()
    H, W = 700, 450
    lat = rng.uniform(30, 31, (H, W))
    los = [rng.uniform(20, 45, (H, W)).astype(np.float32), rng.uniform(-180, 180, (H, W)).astype(np.float32)]
    water = (rng.random((H, W)) > 0.8).astype(np.uint8)
    write_band_vrt(str(full / "lat.rdr.full"), "Float64", [lat])
    write_band_vrt(str(full / "los.rdr.full"), "Float32", los)
    write_band_vrt(str(full / "waterMask.rdr.full"), "Byte", [water])
    out = tmp_path / "geom"
    args = dict(x_start=20, y_start=33, x_step=16, y_step=32, x_win_num=27, y_win_num=21)
    written = prepare_geometry(str(full), str(out), fbases=["lat", "lon", "los", "waterMask"], **args)
    assert [os.path.basename(p) for p in written] == ["lat.rdr", "los.rdr", "waterMask.rdr"]
    for name, bands in (("lat", [lat]), ("los", los), ("waterMask", [water])):
        got = read_vrt_bands(str(out / f"{name}.rdr.vrt"))
        assert len(got) == len(bands)
        for g, b in zip(got, bands):
            want = orc.decimate(b, args["y_start"], args["x_start"], args["y_step"], args["x_step"],
                                args["y_win_num"], args["x_win_num"])
            assert g.dtype == b.dtype and np.array_equal(g, want)
