"""Row-band sharding through the engine: every band of window rows, run on
the image rows it reads (``shard.band_job``), gives exactly the fields the
whole job gives for those windows, so one scene can be split over GPUs or
processes with a host-side join and no collective."""
import numpy as np
import pytest

from isce2_gb300 import PyCuAmpcor, shard, synth

pytestmark = pytest.mark.gpu


def _run(p, ref, sec, gD, gA):
    obj = PyCuAmpcor()
    for k, v in p.items():
        setattr(obj, k, v)
    obj.setupParams()
    obj.setConstantGrossOffset(gD, gA)
    obj.checkPixelInImageRange()
    return obj.run_arrays(ref, sec)


@pytest.mark.parametrize("world", [2, 3])
def test_engine_bands_join_to_the_whole_job(built_lib, world):
    n, gD, gA = 900, -2, 3
    sc = synth.make_pair((n, n), d_down=lambda c: -1.0 + 0.4 * c / n, d_across=lambda r: 0.7 + 0 * r,
                         snr_db=10.0, seed_ref=93, seed_noise=94)
    p = dict(referenceImageHeight=n, referenceImageWidth=n, secondaryImageHeight=n, secondaryImageWidth=n,
             windowSizeHeight=96, windowSizeWidth=64, halfSearchRangeDown=24, halfSearchRangeAcross=24,
             skipSampleDown=40, skipSampleAcross=48, rawDataOversamplingFactor=2,
             corrSurfaceOverSamplingFactor=32, corrSurfaceZoomInWindow=16, derampMethod=1,
             referenceStartPixelDownStatic=30, referenceStartPixelAcrossStatic=30,
             numberWindowDown=17, numberWindowAcross=14)
    whole = _run(p, sc.reference, sc.secondary, gD, gA)
    parts = []
    for band in shard.row_bands(p["numberWindowDown"], world):
        bp, r0, r1 = shard.band_job(p, band, gross_down=gD)
        parts.append(_run(bp, sc.reference[r0:r1], sc.secondary[r0:r1], gD, gA))
    joined = shard.join_bands(parts)
    for k in ("offset", "snr", "cov"):
        np.testing.assert_array_equal(joined[k], whole[k])
