"""Cases run through the reference PyCuAmpcor to pin parity.

Each case names its images (a committed golden fixture, or a seeded scene of
``isce2_gb300.synth`` regenerated on demand) and the PyCuAmpcor properties.
The reference's outputs for these cases are committed as ``ref_<case>.npz``
by ``make_ref_fixtures.py``; the tests load both.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _grid(H, W, p, margin=0):
    """Start pixels at hs (+margin) and as many windows as the range check allows."""
    hsD, hsA = p["halfSearchRangeDown"], p["halfSearchRangeAcross"]
    hs = max(hsD, hsA) + margin
    q = dict(p)
    q.update(referenceImageHeight=H, referenceImageWidth=W, secondaryImageHeight=H, secondaryImageWidth=W,
             referenceStartPixelDownStatic=hs, referenceStartPixelAcrossStatic=hs,
             numberWindowDown=(H - 2 * hs - p["windowSizeHeight"]) // p["skipSampleDown"],
             numberWindowAcross=(W - 2 * hs - p["windowSizeWidth"]) // p["skipSampleAcross"])
    return q


SMALL = dict(windowSizeHeight=32, windowSizeWidth=32, halfSearchRangeDown=8, halfSearchRangeAcross=8,
             skipSampleDown=24, skipSampleAcross=24, rawDataOversamplingFactor=2,
             corrSurfaceOverSamplingFactor=16, corrSurfaceZoomInWindow=8, derampMethod=0)
RECT = dict(windowSizeHeight=48, windowSizeWidth=32, halfSearchRangeDown=10, halfSearchRangeAcross=10,
            skipSampleDown=32, skipSampleAcross=24, rawDataOversamplingFactor=2,
            corrSurfaceOverSamplingFactor=32, corrSurfaceZoomInWindow=16, derampMethod=1)
C1 = dict(windowSizeHeight=64, windowSizeWidth=64, halfSearchRangeDown=20, halfSearchRangeAcross=20,
          skipSampleDown=32, skipSampleAcross=32, rawDataOversamplingFactor=2,
          corrSurfaceOverSamplingFactor=16, corrSurfaceZoomInWindow=8, derampMethod=0)
C2 = dict(windowSizeHeight=128, windowSizeWidth=64, halfSearchRangeDown=32, halfSearchRangeAcross=32,
          skipSampleDown=64, skipSampleAcross=64, rawDataOversamplingFactor=2,
          corrSurfaceOverSamplingFactor=32, corrSurfaceZoomInWindow=16, derampMethod=1)

# name -> (image source, properties, gross offsets: None = constant (0, 0) or
# a seed for varying integer gross offsets in [-2, 2])
CASES = {
    "small_deramp0": (("golden", "small_deramp0"), SMALL, None),
    "rect_deramp1": (("golden", "rect_deramp1"), RECT, None),
    "small_sinc": (("golden", "small_deramp0"), dict(SMALL, corrSurfaceOverSamplingMethod=1), None),
    "rect_timedomain": (("golden", "rect_deramp1"), dict(RECT, algorithm=1), None),
    "small_raw4": (("golden", "small_deramp0"), dict(SMALL, rawDataOversamplingFactor=4,
                                                      corrSurfaceZoomInWindow=16), None),
    "small_raw3": (("golden", "small_deramp0"), dict(SMALL, rawDataOversamplingFactor=3,
                                                      corrSurfaceZoomInWindow=12), None),
    "small_hs_8x6": (("golden", "small_deramp0"), dict(SMALL, halfSearchRangeAcross=6), None),
    "rect_varying_merge": (("golden", "rect_deramp1"), dict(RECT, mergeGrossOffset=1), 7),
    "c1_crop768": (("plain_small", 768), C1, None),
    "c2_crop896x640": (("burst", 896, 640), C2, None),
}


def case_images(name):
    src = CASES[name][0]
    if src[0] == "golden":
        z = np.load(os.path.join(HERE, f"{src[1]}.npz"))
        return z["reference"], z["secondary"]
    from isce2_gb300 import synth
    if src[0] == "plain_small":
        sc = synth.scene_plain_small(src[1])
    elif src[0] == "burst":
        sc = synth.scene_burst(src[1], src[2])
    else:
        raise KeyError(src)
    return sc.reference, sc.secondary


def case_params(name):
    """(properties, varying gross offsets or None) for a case."""
    _, p, gseed = CASES[name]
    ref, _ = case_images(name)
    H, W = ref.shape
    q = _grid(H, W, p, margin=2 if gseed is not None else 0)
    gross = None
    if gseed is not None:
        rng = np.random.default_rng(gseed)
        n = q["numberWindowDown"] * q["numberWindowAcross"]
        gross = rng.integers(-2, 3, size=(2, n)).astype(np.int32)
    return q, gross


def image_digest(ref, sec) -> str:
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(ref, np.complex64).tobytes())
    h.update(np.ascontiguousarray(sec, np.complex64).tobytes())
    return h.hexdigest()[:16]


def load_fixture(name):
    z = np.load(os.path.join(HERE, f"ref_{name}.npz"))
    out = {k: z[k] for k in z.files}
    out["params"] = json.loads(str(out["params"]))
    return out
