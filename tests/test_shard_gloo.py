"""Row-band sharding over two gloo ranks on the CPU: each rank runs its band
(cropped to the image rows it reads) through the oracle, rank 0 gathers the
fields, and the joined field equals the whole job's."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as tmp

from isce2_gb300 import shard


def _params(n):
    return dict(referenceImageHeight=n, referenceImageWidth=n, secondaryImageHeight=n, secondaryImageWidth=n,
                windowSizeHeight=32, windowSizeWidth=32, halfSearchRangeDown=8, halfSearchRangeAcross=8,
                skipSampleDown=24, skipSampleAcross=24, rawDataOversamplingFactor=2,
                corrSurfaceOverSamplingFactor=16, corrSurfaceZoomInWindow=8, derampMethod=0,
                referenceStartPixelDownStatic=12, referenceStartPixelAcrossStatic=12,
                numberWindowDown=11, numberWindowAcross=11)


def _scene(n):
    from isce2_gb300 import synth
    return synth.make_pair((n, n), d_down=lambda c: 1.4 + 0.2 * c / n, d_across=lambda r: -2.1 + 0 * r,
                           snr_db=12.0, seed_ref=91, seed_noise=92)


def _run(p, ref, sec, gD, gA):
    from oracle.ampcor_oracle import OracleParams, run_windows
    op = OracleParams(**{k: v for k, v in p.items() if k in OracleParams.__dataclass_fields__})
    out = run_windows(ref, sec, op, op.constant_gross_starts(gD, gA))
    return {"offset": out["offset"].reshape(p["numberWindowDown"], p["numberWindowAcross"], 2),
            "snr": out["snr"].reshape(p["numberWindowDown"], p["numberWindowAcross"])}


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    n, gD, gA = 320, 1, -2
    sc = _scene(n)
    p = _params(n)
    band = shard.row_bands(p["numberWindowDown"], world)[rank]
    bp, r0, r1 = shard.band_job(p, band, gross_down=gD)
    local = _run(bp, sc.reference[r0:r1], sc.secondary[r0:r1], gD, gA)
    joined = shard.gather_bands(local, rank, world)
    if rank == 0:
        whole = _run(p, sc.reference, sc.secondary, gD, gA)
        q.put({k: (np.array_equal(joined[k], whole[k]), joined[k].shape) for k in whole})
    dist.barrier()
    dist.destroy_process_group()


def test_row_bands_cover_exactly():
    for n, w in [(11, 2), (7, 3), (184, 8), (3, 4)]:
        b = shard.row_bands(n, w)
        assert b[0][0] == 0 and b[-1][1] == n and all(x[1] == y[0] for x, y in zip(b, b[1:]))
        assert max(x[1] - x[0] for x in b) - min(x[1] - x[0] for x in b) <= 1


def test_two_rank_bands_join_to_the_whole_job():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = q.get(timeout=240)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for k, (same, shape) in res.items():
        assert same, k
    assert res["offset"][1] == (11, 11, 2)
