"""Generate the golden fixtures in this directory from the FP64 oracle.

Each case stores its seeded inputs, parameters and the oracle's outputs, so
the fixtures pin the oracle (and, in the GPU tests, the CUDA path) against
regressions.  Run from the repository root:  python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from isce2_gb300 import synth  # noqa: E402
from oracle.ampcor_oracle import OracleParams, run_windows  # noqa: E402

CASES = {
    "small_deramp0": dict(shape=(160, 176), dd=-0.7, da=1.3, snr=10.0, seeds=(21, 22),
                          p=dict(windowSizeHeight=32, windowSizeWidth=32, halfSearchRangeDown=8,
                                 halfSearchRangeAcross=8, skipSampleDown=24, skipSampleAcross=24,
                                 rawDataOversamplingFactor=2, corrSurfaceOverSamplingFactor=16,
                                 corrSurfaceZoomInWindow=8, derampMethod=0)),
    "rect_deramp1": dict(shape=(200, 150), dd=1.6, da=-2.2, snr=15.0, seeds=(23, 24),
                         p=dict(windowSizeHeight=48, windowSizeWidth=32, halfSearchRangeDown=10,
                                halfSearchRangeAcross=10, skipSampleDown=32, skipSampleAcross=24,
                                rawDataOversamplingFactor=2, corrSurfaceOverSamplingFactor=32,
                                corrSurfaceZoomInWindow=16, derampMethod=1)),
}


def case_params(c):
    H, W = c["shape"]
    p = dict(c["p"])
    hs = p["halfSearchRangeDown"]
    p.update(referenceImageHeight=H, referenceImageWidth=W, secondaryImageHeight=H, secondaryImageWidth=W,
             referenceStartPixelDownStatic=hs, referenceStartPixelAcrossStatic=hs,
             numberWindowDown=(H - 2 * hs - p["windowSizeHeight"]) // p["skipSampleDown"],
             numberWindowAcross=(W - 2 * hs - p["windowSizeWidth"]) // p["skipSampleAcross"])
    return p


def main():
    for name, c in CASES.items():
        sc = synth.make_pair(c["shape"], d_down=lambda x, v=c["dd"]: v + 0 * x,
                             d_across=lambda x, v=c["da"]: v + 0 * x, snr_db=c["snr"],
                             seed_ref=c["seeds"][0], seed_noise=c["seeds"][1])
        p = case_params(c)
        op = OracleParams(**p)
        out = run_windows(sc.reference, sc.secondary, op, op.constant_gross_starts(0, 0))
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), reference=sc.reference, secondary=sc.secondary,
                            params=np.array(json.dumps(p)),
                            **{k: v for k, v in out.items()})
        print(name, out["offset"].shape)


if __name__ == "__main__":
    main()
