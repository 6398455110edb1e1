"""Time the reference PyCuAmpcor (ISCE2's GPU ampcor, built from its sources
by oracle/build_ref.py with NDEBUG, cuFFT, sm_103a) on the burst workload on
this GPU, for comparison with this project's plain chain.

Not a test and not part of the product: a measurement script beside the
fixture generator, run by hand on a GPU machine.  The reference reads its
images from files (the raw-file GDALImage stand-in holds them in host memory)
and copies each chunk's tiles to the device as it goes, as its own controller
does (cuAmpcorController.cpp:37-178, cuAmpcorChunk.cpp:260-372); the time is
the wall time of runAmpcor's process minus that of a one-window run
(process start, CUDA and cuFFT initialisation, file reads).

Usage:  python tests/golden/time_ref_gpu.py [--size 12000x8000]
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import build_ref  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", default="12000x8000")
    a = ap.parse_args()
    import bench
    from isce2_gb300 import synth

    bench.SIZE = tuple(int(x) for x in a.size.split("x"))
    binary = build_ref.build_gpu(release=True)
    if not binary:
        sys.exit("reference sources are not staged: run oracle/build_ref.py where the ISCE2 tree exists")
    sc = synth.scene_burst(*bench.SIZE)
    p = bench.geometry()
    nwin = p["numberWindowDown"] * p["numberWindowAcross"]
    res = {"workload": bench.WORKLOAD, "windows": nwin, "reference": "PyCuAmpcor (contrib/PyCuAmpcor/src), "
           "release build, cuFFT; images from host memory, chunk tiles copied as it runs", "runs": {}}
    with tempfile.TemporaryDirectory() as work:
        names = {}
        for tag, img in (("ref", sc.reference), ("sec", sc.secondary)):
            fn = os.path.join(work, f"{tag}.c64")
            np.ascontiguousarray(img, np.complex64).tofile(fn)
            with open(fn + ".shape", "w") as f:
                f.write(f"{img.shape[0]} {img.shape[1]} 8\n")
            names[tag] = fn

        def run(q, nwdc, nwac, nstreams):
            args = [f"{k}={v}" for k, v in q.items()]
            args += [f"referenceImageName={names['ref']}", f"secondaryImageName={names['sec']}",
                     f"numberWindowDownInChunk={nwdc}", f"numberWindowAcrossInChunk={nwac}",
                     f"nStreams={nstreams}", f"outdir={work}"]
            t0 = time.perf_counter()
            r = subprocess.run([binary, *args], capture_output=True, text=True)
            dt = time.perf_counter() - t0
            if r.returncode != 0:
                raise RuntimeError(f"reference run failed ({r.returncode})\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
            return dt

        one = dict(p, numberWindowDown=1, numberWindowAcross=1)
        t_start = min(run(one, 1, 1, 1) for _ in range(2))
        # cuDenseOffsets.py's defaults (1 x 10 windows per chunk, 2 streams),
        # then larger chunks
        for nwdc, nwac, ns in ((1, 10, 2), (4, 40, 2), (8, 60, 2)):
            t = min(run(p, nwdc, nwac, ns) for _ in range(2))
            res["runs"][f"chunk {nwdc}x{nwac}, {ns} streams"] = {
                "wall_s": t, "startup_s": t_start, "windows_per_s": nwin / max(t - t_start, 1e-9)}
    print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
