"""``PyCuAmpcor``: drop-in replacement of ISCE2's pybind11 class.

Same property names, defaults and methods as
``contrib/PyCuAmpcor/src/PyCuAmpcor.cpp:14-101`` (defaults from
``cuAmpcorParameter.cpp:18-64``), so ``cuDenseOffsets.py`` and the TopsProc /
Alos2Proc dense-offset steps can import it unchanged::

    from isce2_gb300 import PyCuAmpcor

Differences a caller can observe: errors raise ``ValueError`` /
``AmpcorError`` instead of terminating the process, and the engine also
accepts in-memory arrays (``run_arrays``) and device tensors
(``run_device``) besides the file-name mode of ``runAmpcor``.
"""
from __future__ import annotations

import ctypes
import os
import xml.etree.ElementTree as ET

import numpy as np

from . import _lib

RAW_TILE_MODES = {"auto": 0, "shared": 1, "l2": 2, "l2x2": 3}
PRECISION_MODES = {"fp32": 0, "split-bf16": 1, "bf16": 2}

_INT_PROPS = {
    "algorithm": 0, "deviceID": 0, "nStreams": 1, "derampMethod": 1,
    "referenceImageHeight": 1000, "referenceImageWidth": 1000,
    "secondaryImageHeight": 1000, "secondaryImageWidth": 1000,
    "numberWindowDown": 1, "numberWindowAcross": 1,
    "windowSizeHeight": 64, "windowSizeWidth": 64,
    "mergeGrossOffset": 0, "rawDataOversamplingFactor": 2, "corrStatWindowSize": 21,
    "numberWindowDownInChunk": 1, "numberWindowAcrossInChunk": 1, "useMmap": 1,
    "halfSearchRangeAcross": 20, "halfSearchRangeDown": 20,
    "referenceStartPixelAcrossStatic": 0, "referenceStartPixelDownStatic": 0,
    "corrSurfaceOverSamplingMethod": 0, "corrSurfaceOverSamplingFactor": 16,
    "mmapSize": 1, "skipSampleDown": 64, "skipSampleAcross": 64, "corrSurfaceZoomInWindow": 16,
}
_STR_PROPS = {
    "referenceImageName": "reference.slc", "secondaryImageName": "secondary.slc",
    "offsetImageName": "DenseOffset.off", "grossOffsetImageName": "GrossOffset.off",
    "snrImageName": "snr.snr", "covImageName": "cov.cov",
}


class PyCuAmpcor:
    """Dense amplitude cross-correlation offset estimator on one GPU."""

    # Placement of the raw-correlation FFT tile (no reference counterpart):
    # "auto" (shared memory when it fits, else an L2-staged global slot),
    # "shared", "l2" (bit-identical to each other) or "l2x2" (256-thread CTAs,
    # two per SM; equal within float32 rounding).
    rawTile = "auto"
    # Oversampler arithmetic (no reference counterpart): "fp32" FFTs,
    # "split-bf16" or "bf16" tensor-core contractions.
    precision = "fp32"
    # Oversampled-correlation arithmetic (no reference counterpart): "fp32"
    # direct sums, "split-bf16" or "bf16" tensor-core contractions.
    corrPrecision = "fp32"

    def __init__(self):
        L = _lib.lib()
        h = ctypes.c_void_p()
        _lib.check(None, L.ampcor_create(ctypes.byref(h)))
        object.__setattr__(self, "_h", h)
        object.__setattr__(self, "_vals", dict(_INT_PROPS))
        self._vals.update(_STR_PROPS)

    # -- properties -------------------------------------------------------
    def __getattr__(self, name):
        vals = object.__getattribute__(self, "_vals")
        if name in vals:
            return vals[name]
        raise AttributeError(name)

    def __setattr__(self, name, value):
        if name in _INT_PROPS:
            self._vals[name] = int(value)
        elif name in _STR_PROPS:
            self._vals[name] = value.decode() if isinstance(value, bytes) else str(value)
        else:
            object.__setattr__(self, name, value)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.lib().ampcor_destroy(h)
            except Exception:
                pass
            self._h = ctypes.c_void_p()

    def _params(self) -> _lib.AmpcorParams:
        p = _lib.AmpcorParams()
        _lib.lib().ampcor_params_default(ctypes.byref(p))
        for f in _lib.PARAM_FIELDS:
            setattr(p, f, int(self._vals[f]))
        return p

    # -- methods of the reference class ------------------------------------
    def setupParams(self):
        """cuAmpcorParameter::setupParameters (cuAmpcorParameter.cpp:70-109)."""
        L = _lib.lib()
        p = self._params()
        _lib.check(self._h, L.ampcor_set_params(self._h, ctypes.byref(p)))
        _lib.check(self._h, L.ampcor_set_raw_mode(self._h, RAW_TILE_MODES[self.rawTile]))
        _lib.check(self._h, L.ampcor_set_precision(self._h, PRECISION_MODES[self.precision]))
        _lib.check(self._h, L.ampcor_set_corr_precision(self._h, PRECISION_MODES[self.corrPrecision]))
        _lib.check(self._h, L.ampcor_setup(self._h))

    def setConstantGrossOffset(self, goDown: int, goAcross: int):
        """setStartPixels with a constant gross offset (cuAmpcorParameter.cpp:189-205)."""
        _lib.check(self._h, _lib.lib().ampcor_set_constant_gross_offset(self._h, int(goDown), int(goAcross)))

    def setVaryingGrossOffset(self, vD, vA):
        """setStartPixels with per-window gross offsets (cuAmpcorParameter.cpp:170-186)."""
        d = np.ascontiguousarray(np.asarray(vD, dtype=np.int32).ravel())
        a = np.ascontiguousarray(np.asarray(vA, dtype=np.int32).ravel())
        if d.size != a.size:
            raise ValueError("gross offset arrays differ in length")
        _lib.check(self._h, _lib.lib().ampcor_set_varying_gross_offset(
            self._h, d.ctypes.data, a.ctypes.data, d.size))

    def setStartPixels(self, refD, refA, grossD, grossA):
        """The general setStartPixels(int*, int*, int*, int*) (cuAmpcorParameter.cpp:155-167)."""
        arrs = [np.ascontiguousarray(np.asarray(x, dtype=np.int32).ravel()) for x in (refD, refA, grossD, grossA)]
        n = arrs[0].size
        if any(x.size != n for x in arrs):
            raise ValueError("start pixel arrays differ in length")
        _lib.check(self._h, _lib.lib().ampcor_set_start_pixels(self._h, *[x.ctypes.data for x in arrs], n))

    def checkPixelInImageRange(self):
        """cuAmpcorParameter::checkPixelInImageRange (cuAmpcorParameter.cpp:275-331)."""
        _lib.check(self._h, _lib.lib().ampcor_check_range(self._h))

    def geometry(self) -> dict:
        g = _lib.AmpcorGeometry()
        _lib.check(self._h, _lib.lib().ampcor_get_geometry(self._h, ctypes.byref(g)))
        return {f: getattr(g, f) for f in _lib.GEOMETRY_FIELDS}

    def startPixels(self) -> dict:
        n = self.numberWindowDown * self.numberWindowAcross
        out = {k: np.zeros(n, np.int32) for k in ("refD", "refA", "grossD", "grossA")}
        _lib.check(self._h, _lib.lib().ampcor_get_start_pixels(
            self._h, out["refD"].ctypes.data, out["refA"].ctypes.data, out["grossD"].ctypes.data,
            out["grossA"].ctypes.data, n))
        return out

    def set_timing(self, enable: bool = True):
        """Bracket every kernel launch with CUDA events (stage timing)."""
        _lib.check(self._h, _lib.lib().ampcor_set_timing(self._h, int(bool(enable))))

    def read_timing(self) -> dict:
        """Per-stage milliseconds and launch counts since the last read."""
        ms = np.zeros(len(_lib.STAGES), np.float32)
        n = np.zeros(len(_lib.STAGES), np.int64)
        _lib.check(self._h, _lib.lib().ampcor_read_timing(self._h, ms.ctypes.data, n.ctypes.data, len(ms)))
        return {s: (float(ms[i]), int(n[i])) for i, s in enumerate(_lib.STAGES)}

    # -- runs ---------------------------------------------------------------
    def run_arrays(self, reference: np.ndarray, secondary: np.ndarray, diag: bool = False) -> dict:
        """Run on host images (complex64, row-major); returns the fields as
        arrays shaped (numberWindowDown, numberWindowAcross[, k])."""
        ref = np.ascontiguousarray(reference, dtype=np.complex64)
        sec = np.ascontiguousarray(secondary, dtype=np.complex64)
        self._check_image_shapes(ref.shape, sec.shape)
        nD, nA = self.numberWindowDown, self.numberWindowAcross
        off = np.zeros((nD, nA, 2), np.float32)
        snr = np.zeros((nD, nA), np.float32)
        cov = np.zeros((nD, nA, 3), np.float32)
        dg = np.zeros((nD, nA, 8), np.int32) if diag else None
        _lib.check(self._h, _lib.lib().ampcor_run_host(
            self._h, ref.ctypes.data, ref.shape[1], sec.ctypes.data, sec.shape[1],
            off.ctypes.data, snr.ctypes.data, cov.ctypes.data, dg.ctypes.data if diag else None))
        out = {"offset": off, "snr": snr, "cov": cov}
        if diag:
            out["diag"] = dg
        return out

    def run_device(self, reference, secondary, out: dict | None = None, diag: bool = False, stream=None) -> dict:
        """Run on device-resident torch tensors (complex64, 2-D, unit column
        stride).  Asynchronous on ``stream`` (default: torch's current stream)."""
        import torch

        for t in (reference, secondary):
            if not (t.is_cuda and t.dtype == torch.complex64 and t.dim() == 2 and t.stride(1) == 1):
                raise ValueError("images must be 2-D complex64 CUDA tensors with unit column stride")
        self._check_image_shapes(tuple(reference.shape), tuple(secondary.shape))
        nD, nA = self.numberWindowDown, self.numberWindowAcross
        dev = reference.device
        if out is None:
            out = {"offset": torch.empty((nD, nA, 2), dtype=torch.float32, device=dev),
                   "snr": torch.empty((nD, nA), dtype=torch.float32, device=dev),
                   "cov": torch.empty((nD, nA, 3), dtype=torch.float32, device=dev)}
            if diag:
                out["diag"] = torch.empty((nD, nA, 8), dtype=torch.int32, device=dev)
        st = stream if stream is not None else torch.cuda.current_stream(dev)
        _lib.check(self._h, _lib.lib().ampcor_run_device(
            self._h, reference.data_ptr(), reference.stride(0), secondary.data_ptr(), secondary.stride(0),
            out["offset"].data_ptr(), out["snr"].data_ptr(), out["cov"].data_ptr(),
            out["diag"].data_ptr() if "diag" in out else None, ctypes.c_void_p(st.cuda_stream)))
        return out

    def run_status(self, stream=None) -> int:
        """Wait for ``stream`` and check the handle's asynchronous runs: raises
        AmpcorError if a bounded device-side wait gave up (the run's results
        are invalid); returns 0 otherwise (ampcor_run_status)."""
        st = ctypes.c_void_p(stream.cuda_stream) if stream is not None else None
        e = ctypes.c_int32(0)
        _lib.check(self._h, _lib.lib().ampcor_run_status(self._h, st, ctypes.byref(e)))
        return int(e.value)

    def _check_image_shapes(self, rs, ss):
        if rs[0] < self.referenceImageHeight or rs[1] < self.referenceImageWidth:
            raise ValueError(f"reference image {rs} smaller than {self.referenceImageHeight}x{self.referenceImageWidth}")
        if ss[0] < self.secondaryImageHeight or ss[1] < self.secondaryImageWidth:
            raise ValueError(f"secondary image {ss} smaller than {self.secondaryImageHeight}x{self.secondaryImageWidth}")

    def runAmpcor(self):
        """cuAmpcorController::runAmpcor (cuAmpcorController.cpp:37-178):
        read both images by name, run, write the offset, gross offset, SNR and
        covariance fields as raw BIP float32 files."""
        ref = read_image(self.referenceImageName, self.referenceImageHeight, self.referenceImageWidth)
        sec = read_image(self.secondaryImageName, self.secondaryImageHeight, self.secondaryImageWidth)
        res = self.run_arrays(ref, sec)
        st = self.startPixels()
        nD, nA = self.numberWindowDown, self.numberWindowAcross
        gross = np.stack([st["grossD"], st["grossA"]], axis=1).astype(np.float32).reshape(nD, nA, 2)
        res["offset"].tofile(self.offsetImageName)
        gross.tofile(self.grossOffsetImageName)
        res["snr"].tofile(self.snrImageName)
        res["cov"].tofile(self.covImageName)
        return res


# ---------------------------------------------------------------------------
# image input without GDAL: raw complex64 files, ISCE .xml side-cars and
# GDAL VRT raw-band descriptions (the form cuDenseOffsets.py passes)
# ---------------------------------------------------------------------------
_VRT_TYPES = {"CFloat32": np.complex64, "Float32": np.float32, "CInt16": None, "Int16": np.int16}


def read_image(name: str, height: int, width: int) -> np.ndarray:
    """Return a (height, width) complex64 view/array of the image ``name``."""
    if name.endswith(".vrt"):
        root = ET.parse(name).getroot()
        band = root.find("VRTRasterBand")
        dtype = band.get("dataType", "CFloat32")
        src = band.findtext("SourceFilename")
        rel = band.find("SourceFilename").get("relativeToVRT", "0") == "1"
        path = os.path.join(os.path.dirname(name), src) if rel else src
        off = int(band.findtext("ImageOffset") or 0)
        pix = int(band.findtext("PixelOffset") or np.dtype(_VRT_TYPES.get(dtype) or np.int16).itemsize)
        line = int(band.findtext("LineOffset") or pix * width)
        order = (band.findtext("ByteOrder") or "LSB").upper()
        return _read_raw(path, height, width, dtype, off, pix, line, order)
    size = os.path.getsize(name)
    if size == height * width * 8:
        return np.memmap(name, dtype=np.complex64, mode="r", shape=(height, width))
    if size == height * width * 4:
        return np.fromfile(name, dtype=np.float32).reshape(height, width).astype(np.complex64)
    raise ValueError(f"{name}: {size} bytes is neither complex64 nor float32 {height}x{width}")


def _read_raw(path, height, width, dtype, off, pix, line, order):
    endian = "<" if order.startswith("LSB") else ">"
    if dtype == "CFloat32":
        base = np.dtype(endian + "c8")
    elif dtype == "Float32":
        base = np.dtype(endian + "f4")
    elif dtype == "CInt16":
        base = np.dtype([("re", endian + "i2"), ("im", endian + "i2")])
    elif dtype == "Int16":
        base = np.dtype(endian + "i2")
    else:
        raise ValueError(f"unsupported VRT dataType {dtype}")
    mm = np.memmap(path, dtype=np.uint8, mode="r")
    rows = np.lib.stride_tricks.as_strided(mm[off:], shape=(height, width * pix), strides=(line, 1))
    raw = np.ascontiguousarray(rows).reshape(height, width, pix)[:, :, :base.itemsize]
    arr = np.ascontiguousarray(raw).view(base).reshape(height, width)
    if dtype == "CInt16":
        return (arr["re"].astype(np.float32) + 1j * arr["im"].astype(np.float32)).astype(np.complex64)
    return arr.astype(np.complex64)


def parse_vrt_size(name: str):
    """(height, width) from a VRT header."""
    root = ET.parse(name).getroot()
    return int(root.get("rasterYSize")), int(root.get("rasterXSize"))

