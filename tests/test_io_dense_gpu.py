"""File mode, VRT input and the DenseAmpcor front end against the pins.

* ``runAmpcor`` in file-name mode, reading the images through GDAL-style VRT
  raw-band headers (the form cuDenseOffsets.py passes) and writing the raw
  BIP fields, compared with what the reference PyCuAmpcor wrote for the same
  case (``tests/golden/ref_<case>.npz``).
* ``DenseAmpcor`` compared with the FP64 oracle on the same windows, start
  pixels and gross offsets (its fields are the merged offsets of those
  windows, with DenseAmpcor's sentinels on rejected windows).

Tolerances are those of the parity tests: integer peaks equal outside float32
near-ties, sub-pixel RMS <= 0.01 px, SNR 1e-3 and covariance 2e-3 relative.
"""
import os
import sys

import numpy as np
import pytest

from isce2_gb300 import DenseAmpcor, PyCuAmpcor, synth
from isce2_gb300.denseampcor import SlcImage
from oracle.ampcor_oracle import OracleParams, run_windows

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import ref_cases  # noqa: E402

pytestmark = pytest.mark.gpu


def write_vrt(path_vrt, raw_name, H, W):
    with open(path_vrt, "w") as f:
        f.write(f'<VRTDataset rasterXSize="{W}" rasterYSize="{H}">\n'
                f'  <VRTRasterBand dataType="CFloat32" band="1" subClass="VRTRawRasterBand">\n'
                f'    <SourceFilename relativeToVRT="1">{raw_name}</SourceFilename>\n'
                f'    <ImageOffset>0</ImageOffset>\n    <PixelOffset>8</PixelOffset>\n'
                f'    <LineOffset>{8 * W}</LineOffset>\n    <ByteOrder>LSB</ByteOrder>\n'
                f'  </VRTRasterBand>\n</VRTDataset>\n')


@pytest.mark.parametrize("name", ["rect_deramp1", "small_sinc"])
def test_run_ampcor_file_mode_vrt_matches_reference(built_lib, tmp_path, name):
    fx = ref_cases.load_fixture(name)
    q, gross = ref_cases.case_params(name)
    ref, sec = ref_cases.case_images(name)
    H, W = ref.shape
    for tag, img in (("ref", ref), ("sec", sec)):
        img.astype(np.complex64).tofile(tmp_path / f"{tag}.slc")
        write_vrt(tmp_path / f"{tag}.slc.vrt", f"{tag}.slc", H, W)
    obj = PyCuAmpcor()
    for k, v in q.items():
        setattr(obj, k, v)
    obj.referenceImageName = str(tmp_path / "ref.slc.vrt")
    obj.secondaryImageName = str(tmp_path / "sec.slc.vrt")
    for attr, fn in (("offsetImageName", "dense.off"), ("grossOffsetImageName", "gross.off"),
                     ("snrImageName", "snr.snr"), ("covImageName", "cov.cov")):
        setattr(obj, attr, str(tmp_path / fn))
    obj.setupParams()
    obj.setConstantGrossOffset(0, 0)
    obj.checkPixelInImageRange()
    obj.runAmpcor()
    n = fx["offset"].shape[0]
    off = np.fromfile(tmp_path / "dense.off", np.float32).reshape(n, 2)
    snr = np.fromfile(tmp_path / "snr.snr", np.float32)
    cov = np.fromfile(tmp_path / "cov.cov", np.float32).reshape(n, 3)
    gro = np.fromfile(tmp_path / "gross.off", np.float32).reshape(n, 2)
    np.testing.assert_array_equal(gro, fx["gross_out"])
    e = off - fx["offset"]
    assert float(np.sqrt(np.mean(e ** 2))) <= 0.01
    np.testing.assert_allclose(snr, fx["snr"], rtol=1e-3)
    sent = fx["cov"][:, 0] == 99.0
    np.testing.assert_array_equal(cov[sent], fx["cov"][sent])
    np.testing.assert_allclose(cov[~sent], fx["cov"][~sent], rtol=2e-3, atol=1e-6)


def test_denseampcor_matches_oracle(built_lib, tmp_path):
    n = 640
    sc = synth.make_pair((n, n), d_down=lambda c: -1.3 + 0.4 * c / n, d_across=lambda r: 0.6 - 0.3 * r / n,
                         snr_db=12.0, seed_ref=83, seed_noise=84)
    d = DenseAmpcor(windowSizeWidth=64, windowSizeHeight=64, searchWindowSizeWidth=16, searchWindowSizeHeight=16,
                    skipSampleAcross=48, skipSampleDown=48, acrossGrossOffset=1, downGrossOffset=-1,
                    oversamplingFactor=16, zoomWindowSize=8,
                    offsetImageName=str(tmp_path / "off.bil"), snrImageName=str(tmp_path / "snr.bil"),
                    covImageName=str(tmp_path / "cov.bil"))
    d.denseampcor(SlcImage(data=sc.reference), sc.secondary)
    L, C = d.offsetLines, d.offsetCols
    k = L * C
    # the same windows through the oracle: DenseAmpcor's centres, half-window
    # 31 up/left of the centre, constant gross offset (-1, +1), merged
    p = OracleParams(referenceImageHeight=n, referenceImageWidth=n, secondaryImageHeight=n, secondaryImageWidth=n,
                     numberWindowDown=L, numberWindowAcross=C, windowSizeHeight=64, windowSizeWidth=64,
                     halfSearchRangeDown=16, halfSearchRangeAcross=16, rawDataOversamplingFactor=2,
                     corrSurfaceOverSamplingFactor=16, corrSurfaceZoomInWindow=8, derampMethod=1,
                     mergeGrossOffset=1)
    st = p.starts_from(d.locationDown.ravel() - 31, d.locationAcross.ravel() - 31, np.full(k, -1), np.full(k, 1))
    o = run_windows(sc.reference, sc.secondary, p, st)
    want = o["offset"] + np.stack([st["grossD"], st["grossA"]], 1).astype(np.float32)
    good = (d.snr > 0).ravel()
    assert good.mean() > 0.9
    ok = good & (o["raw_gap"] >= 2e-5)
    got = np.stack([d.locationDownOffset.ravel(), d.locationAcrossOffset.ravel()], 1)
    e = got[ok] - want[ok]
    assert float(np.sqrt(np.mean(e ** 2))) <= 0.01
    np.testing.assert_allclose(d.snr.ravel()[ok], o["snr"][ok], rtol=1e-3)
