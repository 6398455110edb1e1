"""Request server: continuous batching with HBM-budget admission.

Each request's fields are bit-identical alone and in a mix of requests of
other geometries that arrive while it runs; the fields match the FP64
oracle within the parity tolerances; admission never exceeds the budget."""
import time

import numpy as np
import pytest

from isce2_gb300 import AmpcorServer, synth
from oracle.ampcor_oracle import OracleParams, run_windows

from test_parity_gpu import RAW_TIE, grid_params, make_obj

pytestmark = pytest.mark.gpu


def _request(seed, H, W, **kw):
    sc = synth.make_pair((H, W), d_down=lambda c: 0.9 - 0.3 * c / W, d_across=lambda r: -1.2 + 0.4 * r / H,
                         snr_db=12.0, seed_ref=seed, seed_noise=seed + 1)
    p = grid_params(H, W, **kw)
    obj = make_obj(**p)
    obj.setupParams()
    obj.setConstantGrossOffset(0, 0)
    return sc, p, obj


def _drain(srv, ids, timeout=120.0):
    out, t0 = {}, time.time()
    pending = set(ids)
    while pending:
        srv.progress()
        for rid in srv.poll():
            out[rid] = srv.take(rid)
            pending.discard(rid)
        assert time.time() - t0 < timeout, "server did not finish"
    return out


def test_alone_equals_mixed(built_lib):
    import torch

    reqs = [
        _request(61, 600, 520, Wh=64, Ww=64, hs=16, skip=40, deramp=0),
        _request(63, 700, 420, Wh=128, Ww=64, hs=32, skip=48, ovs=32, zoom=16, deramp=1),
        _request(65, 360, 400, Wh=48, Ww=32, hs=10, skip=24, ovs=16, zoom=8, deramp=1),
        _request(67, 560, 560, Wh=128, Ww=128, hs=48, skip=100, ovs=16, zoom=16, deramp=0),
    ]
    dev = [(torch.from_numpy(sc.reference).cuda(), torch.from_numpy(sc.secondary).cuda()) for sc, _, _ in reqs]
    # alone: one request at a time, small steps so that it spans several
    srv = AmpcorServer(0, step_windows=37)
    alone = []
    for (sc, p, obj), (r, s) in zip(reqs, dev):
        rid = srv.submit(obj, r, s)
        alone.append(_drain(srv, [rid])[rid])
    # mixed: all submitted together (device and host images), other step size
    srv2 = AmpcorServer(0, step_windows=101)
    ids = []
    for k, ((sc, p, obj), (r, s)) in enumerate(zip(reqs, dev)):
        ids.append(srv2.submit(obj, r, s) if k % 2 == 0 else srv2.submit(obj, sc.reference, sc.secondary))
        srv2.progress()
    mixed = _drain(srv2, ids)
    for a, rid in zip(alone, ids):
        for k in ("offset", "snr", "cov"):
            np.testing.assert_array_equal(a[k], mixed[rid][k], err_msg=k)
    # and against the FP64 oracle
    for (sc, p, _), a in zip(reqs, alone):
        op = OracleParams(**{k: v for k, v in p.items() if k in OracleParams.__dataclass_fields__})
        ref = run_windows(sc.reference, sc.secondary, op, op.constant_gross_starts(0, 0))
        near = ref["raw_gap"] < RAW_TIE
        e = a["offset"].reshape(-1, 2) - ref["offset"]
        assert np.sqrt(np.mean(e[~near] ** 2)) <= 0.01
        step = 1.0 / (p["rawDataOversamplingFactor"] * p["corrSurfaceOverSamplingFactor"])
        assert (np.abs(e[~near]).max(axis=1) > step * 1.01).mean() <= 0.02


def test_budget_bounds_admission(built_lib):
    reqs = [_request(71 + k, 400, 400, Wh=64, Ww=64, hs=12, skip=32, deramp=0) for k in range(4)]
    one = 2 * 400 * 400 * 8 + 200 * 1024  # one request's images plus small fields
    srv = AmpcorServer(0, hbm_budget_bytes=int(1.5 * one), step_windows=64)
    ids = [srv.submit(obj, sc.reference, sc.secondary) for sc, _, obj in reqs]
    srv.progress()
    st = srv.stats()
    assert st["active"] + st["queued"] == 4 and st["active"] <= 1
    out = _drain(srv, ids)
    st = srv.stats()
    assert st["peak_bytes"] <= int(1.5 * one) and st["peak_active"] == 1
    assert st["bytes_used"] == 0 and len(out) == 4
    with pytest.raises(Exception, match="budget"):
        small = AmpcorServer(0, hbm_budget_bytes=1024)
        small.submit(reqs[0][2], reqs[0][0].reference, reqs[0][0].secondary)
