"""Tensor-core oversampler (tcgen05 contractions of the half-sample shift
matrices): split-BF16 and BF16 against the FP32 FFT path and the FP64
oracle.  Tolerances: split-BF16 RMS <= 0.01 px against the oracle (as the
FP32 path) with at most 2 % of windows more than one zoom step away; BF16
(about 8 significant bits) RMS <= 0.05 px."""
import numpy as np
import pytest

from isce2_gb300 import synth
from oracle.ampcor_oracle import OracleParams, run_windows

from test_parity_gpu import RAW_TIE, grid_params, make_obj

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("deramp", [0, 1])
def test_tensor_core_oversampler(built_lib, deramp):
    n = 640
    sc = synth.make_pair((n, n), d_down=lambda c: -0.7 + 0.5 * c / n, d_across=lambda r: 1.3 + 0.5 * r / n,
                         snr_db=10.0, seed_ref=51, seed_noise=52)
    kw = grid_params(n, n, 64, 64, 16, 40, ovs=32, zoom=16, deramp=deramp)
    op = OracleParams(**{k: v for k, v in kw.items() if k in OracleParams.__dataclass_fields__})
    ref = run_windows(sc.reference, sc.secondary, op, op.constant_gross_starts(0, 0))
    near = ref["raw_gap"] < RAW_TIE
    step = 1.0 / (2 * 32)
    res = {}
    for mode in ("fp32", "split-bf16", "bf16"):
        obj = make_obj(**kw)
        obj.precision = mode
        obj.setupParams()
        obj.setConstantGrossOffset(0, 0)
        res[mode] = obj.run_arrays(sc.reference, sc.secondary, diag=True)
    for mode, tol in (("split-bf16", 0.01), ("bf16", 0.05)):
        e = res[mode]["offset"].reshape(-1, 2) - ref["offset"]
        rms = float(np.sqrt(np.mean(e[~near] ** 2)))
        assert rms <= tol, (mode, rms)
        # the raw stage is shared: integer peaks equal the FP32 path's
        np.testing.assert_array_equal(res[mode]["diag"][..., :4], res["fp32"]["diag"][..., :4])
    e = res["split-bf16"]["offset"].reshape(-1, 2) - ref["offset"]
    assert (np.abs(e[~near]).max(axis=1) > step * 1.01).mean() <= 0.02


def test_sixty_db_scene_reduced_size(built_lib):
    """The 60 dB precision scene at 1024^2 (speckle, 20 point targets at 1e3 x
    the mean amplitude, a water rectangle at 1e-3 x), window 64, half search
    16, skip 16, ovs 64: windows with a target, with water and plain speckle
    against the FP64 oracle.  Integer peaks equal outside float32 near-ties;
    sub-pixel RMS <= 0.01 px per class, at most 2 % of windows more than one
    zoom step (1/128 px) away."""
    n = 1024
    sc = synth.scene_precision(n, n_targets=20)
    kw = grid_params(n, n, 64, 64, 16, 16, ovs=64, zoom=16, deramp=1)
    obj = make_obj(**kw)
    obj.setupParams()
    obj.setConstantGrossOffset(0, 0)
    got = obj.run_arrays(sc.reference, sc.secondary, diag=True)
    nA = kw["numberWindowAcross"]
    nwin = kw["numberWindowDown"] * nA
    # window classes, from the scene recipe's seeds (synth.scene_precision)
    rng = np.random.default_rng(42)
    tr, tc = rng.integers(0, n, 20), rng.integers(0, n, 20)
    rng = np.random.default_rng(43)
    side = int(np.sqrt(0.1) * n)
    r0, c0 = rng.integers(0, n - side, 2)
    refD = 16 + 16 * (np.arange(nwin) // nA)
    refA = 16 + 16 * (np.arange(nwin) % nA)
    has_t = np.zeros(nwin, bool)
    for a, b in zip(tr, tc):
        has_t |= (a >= refD) & (a < refD + 64) & (b >= refA) & (b < refA + 64)
    has_w = (refD < r0 + side) & (refD + 64 > r0) & (refA < c0 + side) & (refA + 64 > c0)
    cls = np.where(has_t, 0, np.where(has_w, 1, 2))
    pick = [np.random.default_rng(7 + c).choice(np.flatnonzero(cls == c), 16, replace=False) for c in range(3)]
    sel = np.sort(np.concatenate(pick))
    op = OracleParams(**{k: v for k, v in kw.items() if k in OracleParams.__dataclass_fields__})
    ref = run_windows(sc.reference, sc.secondary, op, op.constant_gross_starts(0, 0), sel=sel)
    near = ref["raw_gap"] < RAW_TIE
    d = got["diag"].reshape(-1, 8)[sel]
    np.testing.assert_array_equal(d[~near, 0:2], ref["offset_init"][~near])
    e = got["offset"].reshape(-1, 2)[sel] - ref["offset"]
    step = 1.0 / (2 * 64)
    for c in range(3):
        m = (cls[sel] == c) & ~near
        assert m.sum() >= 12
        assert float(np.sqrt(np.mean(e[m] ** 2))) <= 0.01, (c, e[m])
    assert (np.abs(e[~near]).max(axis=1) > step * 1.01).mean() <= 0.02
