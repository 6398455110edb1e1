"""The FP64 oracle against outputs of the reference PyCuAmpcor itself.

The fixtures ``tests/golden/ref_<case>.npz`` hold what ISCE2's PyCuAmpcor,
built from its own sources for sm_103a with cuFFT (``oracle/build_ref.py``),
computed on the cases of ``tests/golden/ref_cases.py`` (generator:
``tests/golden/make_ref_fixtures.py``).  These tests pin the oracle to the
reference, so the GPU parity tests that compare against the oracle inherit
the pin.

The reference computes in float32 (cuFFT, FP32 kernels, ``rsqrtf``) and the
oracle in float64, so equality is required only where float32 rounding
cannot decide the outcome:

* integer raw peak, clamped zoom start and shift: equal, except on windows
  whose two best raw NCC values are closer than ``RAW_TIE`` in either
  computation (counted; at most 5 % of a case's windows);
* zoomed arg-max and sub-pixel offset: RMS difference <= 0.01 px over the
  other windows and at most 2 % of them more than one zoom-grid step apart;
* SNR and covariance: 1e-3 and 2e-3 relative; covariance sentinels equal;
* stage surfaces (small cases): normalised raw and oversampled correlation
  within 5e-5 absolute.
"""
import os
import sys
import zlib

import numpy as np
import pytest

from oracle.ampcor_oracle import OracleParams, run_windows

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import ref_cases  # noqa: E402

RAW_TIE = 2e-5
CASES = [c for c in ref_cases.CASES if os.path.exists(os.path.join(GOLDEN, f"ref_{c}.npz"))]
MAX_WINDOWS = 48  # oracle windows per case (seeded sample of the larger cases)


def oracle_run(name, fx, sel=None, surfaces=False):
    q, gross = ref_cases.case_params(name)
    assert q == fx["params"], "case definition changed since the fixture was made"
    ref, sec = ref_cases.case_images(name)
    p = OracleParams(**{k: v for k, v in q.items() if k in OracleParams.__dataclass_fields__})
    st = p.constant_gross_starts(0, 0) if gross is None else p.varying_gross_starts(gross[0], gross[1])
    out = run_windows(ref, sec, p, st, sel=sel, surfaces=surfaces)
    if p.mergeGrossOffset:
        s = np.arange(st["refD"].size) if sel is None else sel
        out["offset"] = out["offset"] + np.stack([st["grossD"][s], st["grossA"][s]], 1).astype(np.float32)
    return q, out


def sample(n, name):
    if n <= MAX_WINDOWS:
        return np.arange(n)
    return np.sort(np.random.default_rng(zlib.crc32(name.encode())).choice(n, MAX_WINDOWS, replace=False))


def test_fixtures_present():
    assert len(CASES) == len(ref_cases.CASES), sorted(set(ref_cases.CASES) - set(CASES))


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(name):
    fx = ref_cases.load_fixture(name)
    n = fx["offset"].shape[0]
    sel = sample(n, name)
    small = "raw_surface" in fx
    q, got = oracle_run(name, fx, sel=sel, surfaces=small)
    near = (fx["raw_gap"][sel] < RAW_TIE) | (got["raw_gap"] < RAW_TIE)
    assert near.mean() <= 0.05, near.mean()
    ok = ~near
    np.testing.assert_array_equal(got["offset_init"][ok], fx["offset_init"][sel][ok])
    np.testing.assert_array_equal(got["zoom_start"][ok], fx["zoom_start"][sel][ok])
    np.testing.assert_array_equal(got["zoom_shift"][ok], fx["zoom_shift"][sel][ok])
    e = got["offset"][ok] - fx["offset"][sel][ok]
    step = 1.0 / (q["rawDataOversamplingFactor"] * q["corrSurfaceOverSamplingFactor"])
    rms = float(np.sqrt(np.mean(e ** 2)))
    assert rms <= 0.01, rms
    assert (np.abs(e).max(axis=1) > 1.01 * step).mean() <= 0.02
    snr_ref = fx["snr"][sel][ok]
    fin = np.isfinite(snr_ref)
    np.testing.assert_allclose(got["snr"][ok][fin], snr_ref[fin], rtol=1e-3)
    cov_ref = fx["cov"][sel][ok]
    sent = cov_ref[:, 0] == 99.0
    np.testing.assert_array_equal(got["cov"][ok][sent], cov_ref[sent])
    np.testing.assert_allclose(got["cov"][ok][~sent], cov_ref[~sent], rtol=2e-3, atol=1e-6)
    if small:
        np.testing.assert_allclose(got["raw_surface"], fx["raw_surface"][sel], atol=5e-5)
        np.testing.assert_allclose(got["os_surface"][ok], fx["os_surface"][sel][ok], atol=5e-5)


def test_reference_gross_offsets_echoed():
    """runAmpcor writes the per-window gross offsets it was given
    (cuAmpcorController.cpp:139-155); the varying case's file equals its input."""
    name = "rect_varying_merge"
    if name not in CASES:
        pytest.skip("fixture missing")
    fx = ref_cases.load_fixture(name)
    np.testing.assert_array_equal(fx["gross_out"], fx["gross"].T.astype(np.float32))
