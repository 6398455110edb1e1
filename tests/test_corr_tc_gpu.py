"""Tensor-core oversampled correlation (tcgen05 contractions whose template
operand is read MN-major with the 16 lag shifts as descriptor steps):
split-BF16 and BF16 against the FP32 path, the FP64 oracle and outputs of
the reference PyCuAmpcor itself.

Tolerances: split-BF16 as the FP32 path (sub-pixel RMS <= 0.01 px against
the oracle or the reference, at most 2 % of windows more than one zoom-grid
step away); BF16 (about 8 significant bits) RMS <= 0.05 px.  The raw stage is
untouched, so integer peaks and zoom starts equal the FP32 path's exactly."""
import os
import sys

import numpy as np
import pytest

from isce2_gb300 import AmpcorBatch, PyCuAmpcor, synth
from oracle.ampcor_oracle import OracleParams, run_windows

from test_parity_gpu import RAW_TIE, grid_params, make_obj

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import ref_cases  # noqa: E402

pytestmark = pytest.mark.gpu


def _run(kw, sc, corr, **extra):
    obj = make_obj(**kw)
    obj.corrPrecision = corr
    for k, v in extra.items():
        setattr(obj, k, v)
    obj.setupParams()
    obj.setConstantGrossOffset(0, 0)
    return obj.run_arrays(sc.reference, sc.secondary, diag=True)


def _err_stats(off, ref_off, near, step):
    e = off.reshape(-1, 2)[~near] - ref_off[~near]
    return float(np.sqrt(np.mean(e ** 2))), float((np.abs(e).max(axis=1) > 1.01 * step).mean())


@pytest.mark.parametrize("deramp", [0, 1])
def test_tensor_core_correlation_against_oracle(built_lib, deramp):
    n = 640
    sc = synth.make_pair((n, n), d_down=lambda c: -0.7 + 0.5 * c / n, d_across=lambda r: 1.3 + 0.5 * r / n,
                         snr_db=10.0, seed_ref=61, seed_noise=62)
    kw = grid_params(n, n, 64, 64, 16, 40, ovs=32, zoom=16, deramp=deramp)
    op = OracleParams(**{k: v for k, v in kw.items() if k in OracleParams.__dataclass_fields__})
    ref = run_windows(sc.reference, sc.secondary, op, op.constant_gross_starts(0, 0))
    near = ref["raw_gap"] < RAW_TIE
    step = 1.0 / (2 * 32)
    res = {m: _run(kw, sc, m) for m in ("fp32", "split-bf16", "bf16")}
    for mode, tol in (("split-bf16", 0.01), ("bf16", 0.05)):
        rms, big = _err_stats(res[mode]["offset"], ref["offset"], near, step)
        assert rms <= tol, (mode, rms)
        np.testing.assert_array_equal(res[mode]["diag"][..., :4], res["fp32"]["diag"][..., :4])
        np.testing.assert_array_equal(res[mode]["snr"], res["fp32"]["snr"])
    rms, big = _err_stats(res["split-bf16"]["offset"], ref["offset"], near, step)
    assert big <= 0.02, big


def test_tensor_core_correlation_burst_geometry(built_lib):
    """Window 128 x 64, half search 32, ovs 32, zoom 16: 256 x 128 templates
    against 272 x 144 search chips, streamed in eight bands, with both
    tensor-core stages (split-BF16 oversampler off: chips above its 80 limit)."""
    H, W = 900, 700
    sc = synth.make_pair((H, W), d_down=lambda c: -2.0 + 1.5 * (c / W) ** 2,
                         d_across=lambda r: 1.0 + 2.0 * (r / H) ** 2, snr_db=5.0, seed_ref=63, seed_noise=64)
    kw = grid_params(H, W, 128, 64, 32, 64, ovs=32, zoom=16, deramp=1)
    op = OracleParams(**{k: v for k, v in kw.items() if k in OracleParams.__dataclass_fields__})
    ref = run_windows(sc.reference, sc.secondary, op, op.constant_gross_starts(0, 0))
    near = ref["raw_gap"] < RAW_TIE
    got = _run(kw, sc, "split-bf16")
    d = got["diag"].reshape(-1, 8)
    np.testing.assert_array_equal(d[~near, 0:2], ref["offset_init"][~near])
    rms, big = _err_stats(got["offset"], ref["offset"], near, 1.0 / 64)
    assert rms <= 0.01 and big <= 0.02, (rms, big)


def _ref_case_zp(q):
    raw = q["rawDataOversamplingFactor"]
    hs = min(q["halfSearchRangeDown"], q["halfSearchRangeAcross"])
    zoom = min(q["corrSurfaceZoomInWindow"], 2 * raw * hs)
    return 2 * (zoom // (2 * raw)) * raw


@pytest.mark.parametrize("name", list(ref_cases.CASES))
def test_tensor_core_correlation_against_reference(built_lib, name):
    fx = ref_cases.load_fixture(name)
    q, gross = ref_cases.case_params(name)
    if _ref_case_zp(q) > 16:
        pytest.skip("kept surface above 16 x 16 lags")
    r, s = ref_cases.case_images(name)
    obj = PyCuAmpcor()
    for k, v in q.items():
        setattr(obj, k, v)
    obj.corrPrecision = "split-bf16"
    obj.setupParams()
    if gross is None:
        obj.setConstantGrossOffset(0, 0)
    else:
        obj.setVaryingGrossOffset(gross[0], gross[1])
    obj.checkPixelInImageRange()
    got = obj.run_arrays(r, s, diag=True)
    near = fx["raw_gap"] < RAW_TIE
    d = got["diag"].reshape(-1, 8)
    np.testing.assert_array_equal(d[~near, 0:2], fx["offset_init"][~near])
    np.testing.assert_array_equal(d[~near, 2:4], fx["zoom_start"][~near])
    step = 1.0 / (q["rawDataOversamplingFactor"] * q["corrSurfaceOverSamplingFactor"])
    rms, big = _err_stats(got["offset"], fx["offset"], near, step)
    assert rms <= 0.01 and big <= 0.02, (rms, big)


def test_tensor_core_correlation_batched_equals_plain(built_lib):
    """The batched chain runs the same tensor-core kernel over its wave
    workspace (one wave of two geometries, more windows than CTAs, so CTAs
    of the persistent wave kernel take several windows each): fields
    bit-identical to the plain run's."""
    import torch

    jobs = []
    for seed, (H, W, kw) in enumerate([(1040, 960, dict(Wh=64, Ww=64, hs=20, skip=48, ovs=16, zoom=16)),
                                       (700, 400, dict(Wh=128, Ww=64, hs=32, skip=64, ovs=32, zoom=16,
                                                       deramp=1))]):
        sc = synth.make_pair((H, W), d_down=lambda c: -1.1 + 0.4 * c / W, d_across=lambda r: 0.7 + 0.3 * r / H,
                             snr_db=12.0, seed_ref=70 + 2 * seed, seed_noise=71 + 2 * seed)
        p = grid_params(H, W, **kw)
        obj = make_obj(**p)
        obj.corrPrecision = "split-bf16"
        obj.setupParams()
        obj.setConstantGrossOffset(0, 0)
        jobs.append((sc, p, obj))
    b = AmpcorBatch(0)
    b.set_shape("chain")
    outs = [b.add(obj, torch.from_numpy(sc.reference).cuda(), torch.from_numpy(sc.secondary).cuda())
            for sc, p, obj in jobs]
    st = torch.cuda.Stream()
    with torch.cuda.stream(st):
        b.run(stream=st)
    b.synchronize(stream=st)
    for (sc, p, obj), out in zip(jobs, outs):
        plain = obj.run_arrays(sc.reference, sc.secondary)
        np.testing.assert_array_equal(out["offset"].cpu().numpy().reshape(-1, 2), plain["offset"].reshape(-1, 2))
        np.testing.assert_array_equal(out["snr"].cpu().numpy().ravel(), plain["snr"].ravel())


def test_tensor_core_correlation_rejects_large_surfaces(built_lib):
    kw = grid_params(640, 640, 64, 64, 16, 40, ovs=16, zoom=32)
    obj = make_obj(**kw)
    obj.corrPrecision = "split-bf16"
    with pytest.raises(Exception, match="16 x 16"):
        obj.setupParams()


def test_tensor_core_correlation_batch_shapes(built_lib):
    """A batch holding a tensor-core-correlation job runs the chain by
    default, refuses a fused shape, and its tuner keeps the chain."""
    import torch

    from isce2_gb300._lib import AmpcorError

    H, W = 520, 480
    sc = synth.make_pair((H, W), d_down=lambda c: -1.1 + 0.4 * c / W, d_across=lambda r: 0.7 + 0.3 * r / H,
                         snr_db=12.0, seed_ref=80, seed_noise=81)
    p = grid_params(H, W, Wh=64, Ww=64, hs=20, skip=48, ovs=16, zoom=16)
    obj = make_obj(**p)
    obj.corrPrecision = "split-bf16"
    obj.setupParams()
    obj.setConstantGrossOffset(0, 0)
    r, s = torch.from_numpy(sc.reference).cuda(), torch.from_numpy(sc.secondary).cuda()
    plain = obj.run_arrays(sc.reference, sc.secondary)
    st = torch.cuda.Stream()
    b = AmpcorBatch(0)
    out = b.add(obj, r, s)
    assert b.config()["mode"] == "chain"
    with torch.cuda.stream(st):
        b.run(stream=st)
    b.synchronize(stream=st)
    np.testing.assert_array_equal(out["offset"].cpu().numpy().reshape(-1, 2), plain["offset"].reshape(-1, 2))
    b.set_shape("512x1")
    with pytest.raises(AmpcorError, match="fused"):
        b.run(stream=st)
    b.tune(stream=st)
    assert b.config()["mode"] == "chain"
