"""Row-band sharding of one dense offset job over several processes / GPUs.

Windows are independent (no exchange step), so a job splits into contiguous
bands of window rows, one per rank, in the way DenseAmpcor splits its grid
over row-band processes (DenseAmpcor.py:414-436).  Each rank needs only the
image rows its band touches (reference chips plus the search margin and the
gross offsets), runs its band as an ordinary job, and the fields are joined
on the host.  There is no collective on the data path: the join is a gather
of the per-band fields.
"""
from __future__ import annotations

import numpy as np


def row_bands(n_down: int, world: int) -> list[tuple[int, int]]:
    """Contiguous window-row ranges [w0, w1), as even as possible, in rank order."""
    base, extra = divmod(n_down, world)
    out, w0 = [], 0
    for r in range(world):
        w1 = w0 + base + (1 if r < extra else 0)
        out.append((w0, w1))
        w0 = w1
    return out


def band_job(params: dict, band: tuple[int, int], gross_down: int = 0) -> tuple[dict, int, int]:
    """PyCuAmpcor properties of one band of a constant-gross-offset job and the
    image rows [r0, r1) it reads from both images (a superset of the
    reference and search chips).  The band's reference start is expressed in
    the cropped image, whose row 0 is image row r0."""
    w0, w1 = band
    p = dict(params)
    Wh = p["windowSizeHeight"]
    hsD, hsA = p["halfSearchRangeDown"], p["halfSearchRangeAcross"]
    start = p["referenceStartPixelDownStatic"] + w0 * p["skipSampleDown"]
    last = p["referenceStartPixelDownStatic"] + (w1 - 1) * p["skipSampleDown"]
    # search chip rows: ref start + gross - hsD .. + Wh + 2*max(hs) (the
    # swapped-size search chip and the zoom-in chip both stay inside)
    r0 = max(0, min(start, start + gross_down - hsD))
    r1 = max(last + Wh, last + gross_down - hsD + Wh + 2 * max(hsD, hsA)) + 1
    r1 = min(r1, p["referenceImageHeight"], p["secondaryImageHeight"])
    p["numberWindowDown"] = w1 - w0
    p["referenceStartPixelDownStatic"] = start - r0
    p["referenceImageHeight"] = r1 - r0
    p["secondaryImageHeight"] = r1 - r0
    return p, r0, r1


def join_bands(fields: list[dict]) -> dict:
    """Concatenate per-band fields (window rows first) in band order."""
    return {k: np.concatenate([f[k] for f in fields], axis=0) for k in fields[0]}


def gather_bands(local: dict, rank: int, world: int, group=None) -> dict | None:
    """Gather every rank's band fields on rank 0 (host-side, any backend)."""
    import torch.distributed as dist

    got = [None] * world if rank == 0 else None
    dist.gather_object(local, got, dst=0, group=group)
    return join_bands(got) if rank == 0 else None
