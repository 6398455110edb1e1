"""Run the reference PyCuAmpcor on the cases of ``ref_cases.py`` and save its
outputs as fixtures ``ref_<case>.npz``.

Needs a CUDA GPU and the reference build of ``oracle/build_ref.py``
(``python oracle/build_ref.py --gpu``).  Each case runs as one chunk (every
window in one batch), so the reference's debug dumps (it is built without
NDEBUG) hold every window: its raw arg-max ``i_offsetInit``, the clamped zoom
start ``i_offsetInitAdjusted`` and shift ``i_maxLocShift``, the zoomed
arg-max ``i_offsetZoomIn``, the peak values, and the normalised correlation
surfaces from which the FP32 near-tie gaps are taken.  Its final outputs
(offset, SNR, covariance files) are what runAmpcor writes.

Usage:  python tests/golden/make_ref_fixtures.py [--out DIR] [case ...]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import ref_cases  # noqa: E402
from oracle import build_ref  # noqa: E402


def _gap(surf):
    """top-1 minus top-2 value per window (FP32 values as the reference has them)."""
    v = np.where(np.isnan(surf), -np.inf, surf).astype(np.float64)
    s = np.sort(v, axis=1)
    return s[:, -1] - s[:, -2]


def run_case(binary, name, work):
    q, gross = ref_cases.case_params(name)
    ref, sec = ref_cases.case_images(name)
    d = os.path.join(work, name)
    os.makedirs(d, exist_ok=True)
    for tag, img in (("ref", ref), ("sec", sec)):
        fn = os.path.join(d, f"{tag}.c64")
        np.ascontiguousarray(img, np.complex64).tofile(fn)
        with open(fn + ".shape", "w") as f:
            f.write(f"{img.shape[0]} {img.shape[1]} 8\n")
    nD, nA = q["numberWindowDown"], q["numberWindowAcross"]
    n = nD * nA
    args = [f"{k}={v}" for k, v in q.items()]
    args += [f"referenceImageName={os.path.join(d, 'ref.c64')}", f"secondaryImageName={os.path.join(d, 'sec.c64')}",
             f"numberWindowDownInChunk={nD}", f"numberWindowAcrossInChunk={nA}", f"outdir={d}"]
    if gross is not None:
        gfile = os.path.join(d, "gross.i32")
        gross.astype(np.int32).tofile(gfile)
        args.append(f"grossFile={gfile}")
    r = subprocess.run([binary, *args], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{name}: reference run failed ({r.returncode})\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")

    def rd(fn, dt, shape):
        return np.fromfile(os.path.join(d, fn), dt).reshape(shape)

    raw = q["rawDataOversamplingFactor"]
    zoom = min(q["corrSurfaceZoomInWindow"], 2 * raw * min(q["halfSearchRangeDown"], q["halfSearchRangeAcross"]))
    zn = zoom * q["corrSurfaceOverSamplingFactor"]
    rawc = rd("r_corrBatchRaw", np.float32, (n, -1))
    zsurf = rd("r_corrBatchZoomInOverSampled", np.float32, (n, zn * zn))
    out = dict(
        params=np.array(json.dumps(q)), digest=np.array(ref_cases.image_digest(ref, sec)),
        offset=rd("offset.bip", np.float32, (n, 2)), snr=rd("snr.bip", np.float32, (n,)),
        cov=rd("cov.bip", np.float32, (n, 3)), gross_out=rd("gross.bip", np.float32, (n, 2)),
        offset_init=rd("i_offsetInit", np.int32, (n, 2)), zoom_start=rd("i_offsetInitAdjusted", np.int32, (n, 2)),
        zoom_shift=rd("i_maxLocShift", np.int32, (n, 2)), zoom_loc=rd("i_offsetZoomIn", np.int32, (n, 2)),
        maxval=rd("r_maxval", np.float32, (n,)), zoom_maxval=rd("r_maxvalZoomInOversampled", np.float32, (n,)),
        raw_gap=_gap(rawc), zoom_gap=_gap(zsurf),
    )
    if gross is not None:
        out["gross"] = gross
    if n * rawc.shape[1] <= 200_000:  # stage-level pins for the small cases
        out["raw_surface"] = rawc
        out["os_surface"] = rd("r_corrBatchZoomIn", np.float32, (n, -1))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=HERE)
    ap.add_argument("cases", nargs="*")
    a = ap.parse_args()
    binary = build_ref.build(gpu=True)["gpu"]
    if not binary:
        sys.exit("reference sources are not staged: run oracle/build_ref.py where the ISCE2 tree exists")
    os.makedirs(a.out, exist_ok=True)
    with tempfile.TemporaryDirectory() as work:
        for name in (a.cases or list(ref_cases.CASES)):
            out = run_case(binary, name, work)
            np.savez_compressed(os.path.join(a.out, f"ref_{name}.npz"), **out)
            print(f"{name}: {out['offset'].shape[0]} windows", flush=True)


if __name__ == "__main__":
    main()
