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
