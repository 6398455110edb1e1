"""C ABI and host logic, without a GPU: the library loads, exports every
function include/ampcor_gb.h declares, and its geometry, start-pixel and
range logic match the oracle's restatement of cuAmpcorParameter."""
import ctypes
import os
import re

import numpy as np
import pytest

from isce2_gb300 import PyCuAmpcor, _lib
from oracle.ampcor_oracle import OracleParams

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "ampcor_gb.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ampcor_[a-z_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(built_lib):
    names = declared_functions()
    assert len(names) >= 18
    for n in names:
        assert hasattr(built_lib, n), n
    assert set(names) == set(_lib.exported_symbols())
    assert b"sm_103a" in built_lib.ampcor_version()


def test_defaults_match_reference(built_lib):
    obj = PyCuAmpcor()
    # cuAmpcorParameter.cpp:18-64
    assert obj.algorithm == 0 and obj.deviceID == 0 and obj.nStreams == 1 and obj.derampMethod == 1
    assert (obj.windowSizeHeight, obj.windowSizeWidth) == (64, 64)
    assert (obj.halfSearchRangeDown, obj.halfSearchRangeAcross) == (20, 20)
    assert (obj.skipSampleDown, obj.skipSampleAcross) == (64, 64)
    assert obj.rawDataOversamplingFactor == 2 and obj.corrSurfaceZoomInWindow == 16
    assert obj.corrSurfaceOverSamplingFactor == 16 and obj.corrSurfaceOverSamplingMethod == 0
    assert obj.corrStatWindowSize == 21 and obj.mergeGrossOffset == 0
    assert obj.referenceImageName == "reference.slc" and obj.offsetImageName == "DenseOffset.off"
    p = _lib.AmpcorParams()
    built_lib.ampcor_params_default(ctypes.byref(p))
    for f in _lib.PARAM_FIELDS:
        assert getattr(p, f) == getattr(obj, f), f


CONFIGS = [
    dict(windowSizeHeight=64, windowSizeWidth=64, halfSearchRangeDown=20, halfSearchRangeAcross=20,
         rawDataOversamplingFactor=2, corrSurfaceZoomInWindow=8, corrSurfaceOverSamplingFactor=16),
    dict(windowSizeHeight=128, windowSizeWidth=64, halfSearchRangeDown=32, halfSearchRangeAcross=32,
         rawDataOversamplingFactor=2, corrSurfaceZoomInWindow=16, corrSurfaceOverSamplingFactor=32),
    dict(windowSizeHeight=32, windowSizeWidth=48, halfSearchRangeDown=3, halfSearchRangeAcross=5,
         rawDataOversamplingFactor=2, corrSurfaceZoomInWindow=16, corrSurfaceOverSamplingFactor=16),
]


@pytest.mark.parametrize("cfg", CONFIGS)
def test_geometry_matches_oracle(built_lib, cfg):
    obj = PyCuAmpcor()
    base = dict(referenceImageHeight=1000, referenceImageWidth=900, secondaryImageHeight=1000,
                secondaryImageWidth=900, numberWindowDown=5, numberWindowAcross=7, skipSampleDown=40,
                skipSampleAcross=50, referenceStartPixelDownStatic=60, referenceStartPixelAcrossStatic=70)
    for k, v in {**base, **cfg}.items():
        setattr(obj, k, v)
    obj.setupParams()
    g = obj.geometry()
    d = OracleParams(**{**base, **cfg}).derived()
    assert g["searchWindowSizeHeightRaw"] == d["searchHeightRaw"]
    assert g["searchWindowSizeWidthRaw"] == d["searchWidthRaw"]
    assert g["zoomWindowSize"] == d["zoom"] and g["halfZoomWindowSizeRaw"] == d["hz"]
    assert g["corrRawZoomInHeight"] == d["corrRawZoomInHeight"]
    assert g["corrRawZoomInWidth"] == d["corrRawZoomInWidth"]
    assert g["numberWindows"] == 35


def test_start_pixels_and_gross_offsets(built_lib):
    obj = PyCuAmpcor()
    kw = dict(referenceImageHeight=800, referenceImageWidth=800, secondaryImageHeight=800, secondaryImageWidth=800,
              numberWindowDown=4, numberWindowAcross=3, skipSampleDown=33, skipSampleAcross=44,
              referenceStartPixelDownStatic=50, referenceStartPixelAcrossStatic=60)
    for k, v in kw.items():
        setattr(obj, k, v)
    obj.setupParams()
    p = OracleParams(**kw)
    obj.setConstantGrossOffset(3, -2)
    st = obj.startPixels()
    o = p.constant_gross_starts(3, -2)
    np.testing.assert_array_equal(st["refD"], o["refD"])
    np.testing.assert_array_equal(st["refA"], o["refA"])
    np.testing.assert_array_equal(st["grossA"], o["grossA"])
    vD = np.arange(12, dtype=np.int32) - 5
    vA = -np.arange(12, dtype=np.int32)
    obj.setVaryingGrossOffset(vD, vA)
    st = obj.startPixels()
    o = p.varying_gross_starts(vD, vA)
    np.testing.assert_array_equal(st["grossD"], o["grossD"])
    np.testing.assert_array_equal(st["refA"], o["refA"])
    with pytest.raises(ValueError):
        obj.setVaryingGrossOffset(vD[:5], vA[:5])


def test_range_check_errors_instead_of_exit(built_lib):
    obj = PyCuAmpcor()
    for k, v in dict(referenceImageHeight=300, referenceImageWidth=300, secondaryImageHeight=300,
                     secondaryImageWidth=300, numberWindowDown=2, numberWindowAcross=2,
                     referenceStartPixelDownStatic=20, referenceStartPixelAcrossStatic=20).items():
        setattr(obj, k, v)
    obj.setupParams()
    obj.setConstantGrossOffset(0, 0)
    obj.checkPixelInImageRange()
    obj.setConstantGrossOffset(-5, 0)  # secondary start below 0
    with pytest.raises(ValueError, match="Secondary Window start pixel out ot range in Down"):
        obj.checkPixelInImageRange()
    obj.setConstantGrossOffset(0, 200)
    with pytest.raises(ValueError, match="end pixel"):
        obj.checkPixelInImageRange()


def test_call_order_and_bad_parameters(built_lib):
    obj = PyCuAmpcor()
    with pytest.raises(_lib.AmpcorError):
        obj.setConstantGrossOffset(0, 0)  # before setupParams
    obj.numberWindowDown = 0
    with pytest.raises(ValueError, match="Incorrect number of windows"):
        obj.setupParams()
    obj.numberWindowDown = 1
    obj.corrSurfaceOverSamplingMethod = 2
    with pytest.raises(Exception, match="0 \\(FFT\\) or 1 \\(sinc\\)"):
        obj.setupParams()
    obj.corrSurfaceOverSamplingMethod = 1
    obj.corrSurfaceZoomInWindow = 6  # not a multiple of 2 * raw: the sinc taps would leave the surface
    with pytest.raises(_lib.AmpcorError, match="sinc"):
        obj.setupParams()
    obj.corrSurfaceZoomInWindow = 16
    obj.setupParams()


def test_unsupported_prime_window_is_reported(built_lib):
    obj = PyCuAmpcor()
    obj.windowSizeHeight = 139 * 2  # 278 = 2 * 139, prime 139 > 131
    obj.windowSizeWidth = 64
    with pytest.raises(_lib.AmpcorError, match="prime factor"):
        obj.setupParams()


def test_raw_tile_placement(built_lib):
    # a 128 x 128 window searched +-48: a 224 x 224 raw tile (~400 KB)
    def setup(mode):
        obj = PyCuAmpcor()
        obj.referenceImageHeight = obj.referenceImageWidth = 4096
        obj.secondaryImageHeight = obj.secondaryImageWidth = 4096
        obj.windowSizeHeight = obj.windowSizeWidth = 128
        obj.halfSearchRangeDown = obj.halfSearchRangeAcross = 48
        obj.rawTile = mode
        obj.setupParams()
        return obj
    with pytest.raises(_lib.AmpcorError, match="does not fit in shared memory"):
        setup("shared")
    assert setup("auto").geometry()["fftHeight"] == 224
    setup("l2")
    bad = PyCuAmpcor()
    with pytest.raises(ValueError):
        _lib.check(bad._h, _lib.lib().ampcor_set_raw_mode(bad._h, 4))


def test_run_without_gpu_fails_loudly(built_lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    obj = PyCuAmpcor()
    for k, v in dict(referenceImageHeight=300, referenceImageWidth=300, secondaryImageHeight=300,
                     secondaryImageWidth=300, referenceStartPixelDownStatic=20,
                     referenceStartPixelAcrossStatic=20).items():
        setattr(obj, k, v)
    obj.setupParams()
    obj.setConstantGrossOffset(0, 0)
    z = np.zeros((300, 300), np.complex64)
    with pytest.raises(_lib.AmpcorError) as e:
        obj.run_arrays(z, z)
    assert e.value.code == _lib.AMPCOR_ERR_CUDA


def test_server_without_gpu_fails_loudly(built_lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    assert built_lib.ampcor_server_create(ctypes.byref(h), 0, 1 << 30, 1024) == _lib.AMPCOR_ERR_CUDA
    assert built_lib.ampcor_server_create(ctypes.byref(h), 0, 0, 1024) == _lib.AMPCOR_ERR_ARG


def test_precision_mode_validation(built_lib):
    obj = PyCuAmpcor()
    obj.precision = "split-bf16"
    obj.setupParams()  # 64 x 64 windows: the tensor-core oversampler applies
    big = PyCuAmpcor()
    big.windowSizeHeight = big.windowSizeWidth = 128
    big.referenceImageHeight = big.referenceImageWidth = 4096
    big.secondaryImageHeight = big.secondaryImageWidth = 4096
    big.precision = "bf16"
    with pytest.raises(_lib.AmpcorError, match="tensor-core oversampling"):
        big.setupParams()
    with pytest.raises(ValueError):
        _lib.check(obj._h, _lib.lib().ampcor_set_precision(obj._h, 3))
