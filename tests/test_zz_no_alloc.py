"""Allocation-free entry point (ampcor_run_device_noalloc), called through the
C ABI and compared with the allocating entry point on the same inputs.

Callers that cannot call cudaMalloc (their own pool owns the device memory, or
a driver allocation on their hot path could synchronise the device or fail)
use this entry point; its working memory is a static device array of
AMPCOR_NOALLOC_SCRATCH_BYTES.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from isce2_gb300 import PyCuAmpcor, _lib, synth

pytestmark = pytest.mark.gpu

SCRATCH_BYTES = 32 << 20


def _setup(H, W, **kw):
    obj = PyCuAmpcor()
    hs = kw.get("halfSearchRangeDown", 20)
    base = dict(referenceImageHeight=H, referenceImageWidth=W, secondaryImageHeight=H, secondaryImageWidth=W,
                referenceStartPixelDownStatic=hs, referenceStartPixelAcrossStatic=hs)
    for k, v in {**base, **kw}.items():
        setattr(obj, k, v)
    obj.setupParams()
    obj.setConstantGrossOffset(0, 0)
    return obj


def _run(L, obj, r, s, entry):
    import torch

    n = obj.numberWindowDown * obj.numberWindowAcross
    off = torch.full((n, 2), float("nan"), device="cuda")
    snr = torch.full((n,), float("nan"), device="cuda")
    cov = torch.full((n, 3), float("nan"), device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    if entry == "noalloc":
        rc = L.ampcor_run_device_noalloc(obj._h, r.data_ptr(), r.stride(0), s.data_ptr(), s.stride(0),
                                         off.data_ptr(), snr.data_ptr(), cov.data_ptr(), st)
    else:
        rc = L.ampcor_run_device(obj._h, r.data_ptr(), r.stride(0), s.data_ptr(), s.stride(0),
                                 off.data_ptr(), snr.data_ptr(), cov.data_ptr(), None, st)
    _lib.check(obj._h, rc)
    # no bounded device wait of the run gave up (the no-alloc run keeps its
    # error word in the static scratch; the status call reads and clears it)
    e = ctypes.c_int32(-1)
    _lib.check(obj._h, L.ampcor_run_status(obj._h, st, ctypes.byref(e)))
    assert e.value == 0
    torch.cuda.synchronize()
    return off.cpu().numpy(), snr.cpu().numpy(), cov.cpu().numpy()


@pytest.mark.parametrize("case", ["small", "batched"])
def test_noalloc_matches_allocating_entry_point_twice(case):
    import torch

    L = _lib.lib()
    if case == "small":
        H, W = 512, 480
        kw = dict(windowSizeHeight=64, windowSizeWidth=64, halfSearchRangeDown=20, halfSearchRangeAcross=20,
                  skipSampleDown=48, skipSampleAcross=48, numberWindowDown=8, numberWindowAcross=7,
                  corrSurfaceZoomInWindow=8, corrSurfaceOverSamplingFactor=16, derampMethod=0)
    else:  # burst geometry: several batches through the 32 MiB scratch
        H, W = 1400, 1100
        kw = dict(windowSizeHeight=128, windowSizeWidth=64, halfSearchRangeDown=32, halfSearchRangeAcross=32,
                  skipSampleDown=64, skipSampleAcross=64, numberWindowDown=19, numberWindowAcross=15,
                  corrSurfaceZoomInWindow=16, corrSurfaceOverSamplingFactor=32, derampMethod=1)
    sc = synth.make_pair((H, W), d_down=lambda c: -0.6 + 0.3 * c / W, d_across=lambda r: 1.1 + 0.2 * r / H,
                         snr_db=10.0, seed_ref=31, seed_noise=32)
    obj = _setup(H, W, **kw)
    r = torch.from_numpy(sc.reference).cuda()
    s = torch.from_numpy(sc.secondary).cuda()
    ref_off, ref_snr, ref_cov = _run(L, obj, r, s, "alloc")
    for _ in range(2):  # the second call sees what the first left in the shared array
        off, snr, cov = _run(L, obj, r, s, "noalloc")
        np.testing.assert_allclose(off, ref_off, rtol=0, atol=1e-6)
        np.testing.assert_allclose(snr, ref_snr, rtol=1e-6)
        np.testing.assert_allclose(cov, ref_cov, rtol=1e-6, atol=1e-9)


def test_noalloc_rejects_geometry_beyond_scratch():
    import torch

    L = _lib.lib()
    H, W = 9000, 9000
    obj = _setup(H, W, windowSizeHeight=64, windowSizeWidth=64, halfSearchRangeDown=20, halfSearchRangeAcross=20,
                 skipSampleDown=11, skipSampleAcross=11, numberWindowDown=800, numberWindowAcross=800)
    # 640 000 windows need 640 000 x 68 B of coordinates and results: more than the scratch
    assert 640000 * 68 > SCRATCH_BYTES
    r = torch.zeros((H, W), dtype=torch.complex64, device="cuda")
    out = torch.zeros((640000, 6), device="cuda")
    rc = L.ampcor_run_device_noalloc(obj._h, r.data_ptr(), W, r.data_ptr(), W, out.data_ptr(),
                                     out.data_ptr(), out.data_ptr(), None)
    assert rc == _lib.AMPCOR_ERR_UNSUPPORTED
    assert "static scratch holds" in _lib.last_error(obj._h)
