"""Device error reporting of asynchronous runs.

Every kernel wait on a copy is bounded; a wait that gives up sets a device
error word that ``ampcor_run_status`` reads.  The timeout is made to happen
the allowed way: a self-test block waits on an mbarrier that nothing ever
completes (no copy is in flight), gives up after a few polls and returns.
The context stays usable: a normal run afterwards is correct and reports no
error.
"""
import ctypes

import numpy as np
import pytest

from isce2_gb300 import PyCuAmpcor, _lib, synth
from oracle.ampcor_oracle import OracleParams, run_windows

pytestmark = pytest.mark.gpu

KW = dict(referenceImageHeight=256, referenceImageWidth=256, secondaryImageHeight=256, secondaryImageWidth=256,
          windowSizeHeight=48, windowSizeWidth=48, halfSearchRangeDown=12, halfSearchRangeAcross=12,
          skipSampleDown=48, skipSampleAcross=48, rawDataOversamplingFactor=2, corrSurfaceOverSamplingFactor=16,
          corrSurfaceZoomInWindow=8, derampMethod=0, referenceStartPixelDownStatic=12,
          referenceStartPixelAcrossStatic=12, numberWindowDown=3, numberWindowAcross=3)


def make():
    obj = PyCuAmpcor()
    for k, v in KW.items():
        setattr(obj, k, v)
    obj.setupParams()
    obj.setConstantGrossOffset(0, 0)
    obj.checkPixelInImageRange()
    return obj


def test_timed_out_wait_is_reported_and_context_survives(built_lib):
    import torch

    obj = make()
    L = _lib.lib()
    st = torch.cuda.Stream()
    assert L.ampcor_selftest_wait_timeout(obj._h, 64, ctypes.c_void_p(st.cuda_stream)) == _lib.AMPCOR_OK
    with pytest.raises(_lib.AmpcorError, match="gave up"):
        obj.run_status(st)
    assert obj.run_status(st) == 0  # the status call cleared the word

    sc = synth.make_pair((256, 256), d_down=lambda c: 0.4 + 0 * c, d_across=lambda r: -1.2 + 0 * r,
                         snr_db=20.0, seed_ref=3, seed_noise=4)
    ref_d = torch.from_numpy(sc.reference).cuda()
    sec_d = torch.from_numpy(sc.secondary).cuda()
    with torch.cuda.stream(st):
        out = obj.run_device(ref_d, sec_d, stream=st)
    assert obj.run_status(st) == 0
    p = OracleParams(**KW)
    want = run_windows(sc.reference, sc.secondary, p, p.constant_gross_starts(0, 0))["offset"]
    got = out["offset"].reshape(-1, 2).cpu().numpy()
    assert np.abs(got - want).max() <= 0.01


def test_status_before_any_run_is_ok(built_lib):
    assert make().run_status() == 0


def test_selftest_rejects_bad_limits(built_lib):
    obj = make()
    L = _lib.lib()
    assert L.ampcor_selftest_wait_timeout(obj._h, 0, None) == _lib.AMPCOR_ERR_ARG
    assert L.ampcor_selftest_wait_timeout(obj._h, (1 << 20) + 1, None) == _lib.AMPCOR_ERR_ARG
