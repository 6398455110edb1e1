"""DenseAmpcor-compatible front end: parameter surface, window checks and
window-centre grid (CPU), and a GPU run checked against PyCuAmpcor on the
same windows and against the known offset field."""
import os

import numpy as np
import pytest

from isce2_gb300 import DenseAmpcor, PyCuAmpcor, synth
from isce2_gb300.denseampcor import SlcImage


def test_defaults_follow_reference():
    d = DenseAmpcor()
    # DenseAmpcor.py:81-280
    assert (d.windowSizeWidth, d.windowSizeHeight) == (64, 64)
    assert (d.searchWindowSizeWidth, d.searchWindowSizeHeight) == (100, 100)
    assert d.zoomWindowSize == 16 and d.oversamplingFactor == 16 and d.margin == 50
    assert d.thresholdCov == 1000.0 and d.scaling_factor == 1.0
    assert d.offsetImageName == "dense_ampcor.bil" and d.covImageName == "dense_ampcor_cov.bil"


@pytest.mark.parametrize("bad, msg", [
    (dict(windowSizeWidth=63), "even"),
    (dict(zoomWindowSize=12), "power of 2"),
    (dict(oversamplingFactor=24), "power of 2"),
    (dict(searchWindowSizeWidth=128), "< 2 \\* Window Size Width"),
    (dict(searchWindowSizeWidth=4, searchWindowSizeHeight=4, zoomWindowSize=16), "Zoom window size"),
])
def test_check_windows(bad, msg):
    d = DenseAmpcor(**{**dict(searchWindowSizeWidth=20, searchWindowSizeHeight=20), **bad})
    with pytest.raises(ValueError, match=msg):
        d.checkWindows()


def test_grid_matches_reference_arithmetic():
    # worked by hand from DenseAmpcor.py:368-400: 1000 x 1000, W 64, search 20,
    # skip 32, margin 50, no gross offset -> offAc 173, lastAc 845, centres
    # 224, 256, ..., 768 (18 across)
    d = DenseAmpcor(searchWindowSizeWidth=20, searchWindowSizeHeight=20, skipSampleAcross=32, skipSampleDown=32)
    d.fileLength1 = d.fileLength2 = d.lineLength1 = d.lineLength2 = 1000
    d.checkWindows()
    gD, gA = d.grid()
    assert list(gA) == list(range(224, 794, 32)) and d.numLocationAcross == 18
    assert d.numLocationDown == len(gD) == 18 and gD[0] == 224
    # a negative gross offset widens the left margin
    d2 = DenseAmpcor(searchWindowSizeWidth=20, searchWindowSizeHeight=20, skipSampleAcross=32, skipSampleDown=32,
                     acrossGrossOffset=-80)
    d2.fileLength1 = d2.fileLength2 = d2.lineLength1 = d2.lineLength2 = 1000
    d2.checkWindows()
    _, gA2 = d2.grid()
    assert gA2[0] >= 80 + 104 + d2.pixLocOffAc


@pytest.mark.gpu
def test_gpu_run_matches_pycuampcor(built_lib, tmp_path):
    n = 640
    sc = synth.make_pair((n, n), d_down=lambda c: -1.3 + 0 * c, d_across=lambda r: 0.6 + 0 * r,
                         snr_db=15.0, seed_ref=81, seed_noise=82)
    d = DenseAmpcor(windowSizeWidth=64, windowSizeHeight=64, searchWindowSizeWidth=16, searchWindowSizeHeight=16,
                    skipSampleAcross=48, skipSampleDown=48, acrossGrossOffset=1, downGrossOffset=-1,
                    oversamplingFactor=16, zoomWindowSize=8,
                    offsetImageName=str(tmp_path / "off.bil"), snrImageName=str(tmp_path / "snr.bil"),
                    covImageName=str(tmp_path / "cov.bil"))
    sc.reference.tofile(tmp_path / "ref.slc")
    d.denseampcor(SlcImage(str(tmp_path / "ref.slc"), n, n), sc.secondary)
    L, C = d.offsetLines, d.offsetCols
    off = np.fromfile(tmp_path / "off.bil", np.float32).reshape(2 * L, C)
    assert os.path.exists(str(tmp_path / "off.bil") + ".xml")
    np.testing.assert_array_equal(off[::2], d.locationDownOffset)
    good = d.snr > 0
    assert good.mean() > 0.9
    assert np.abs(d.locationDownOffset[good] + 1.3).max() < 0.1
    assert np.abs(d.locationAcrossOffset[good] - 0.6).max() < 0.1
    # the same windows straight through PyCuAmpcor (total offsets)
    obj = PyCuAmpcor()
    for k, v in dict(referenceImageHeight=n, referenceImageWidth=n, secondaryImageHeight=n, secondaryImageWidth=n,
                     windowSizeHeight=64, windowSizeWidth=64, halfSearchRangeDown=16, halfSearchRangeAcross=16,
                     numberWindowDown=L, numberWindowAcross=C, corrSurfaceOverSamplingFactor=16,
                     corrSurfaceZoomInWindow=8, derampMethod=1, mergeGrossOffset=1).items():
        setattr(obj, k, v)
    obj.setupParams()
    k = L * C
    obj.setStartPixels(d.locationDown.ravel() - 31, d.locationAcross.ravel() - 31, np.full(k, -1), np.full(k, 1))
    r = obj.run_arrays(sc.reference, sc.secondary)
    np.testing.assert_array_equal(r["offset"].reshape(-1, 2)[good.ravel(), 0], d.locationDownOffset[good])
