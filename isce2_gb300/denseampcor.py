"""DenseAmpcor-compatible front end over the GB300 engine.

ISCE2's CPU dense offset component (components/mroipac/ampcor/DenseAmpcor.py)
lays a grid of window centres over the reference image, runs the Fortran
ampcor (ampcor.F) in row-band processes, and writes BIL float32 images:
offsets (2 bands: down, across), SNR, covariance (3 bands).  Callers
(TopsProc/runDenseOffsets.py, topsStack/denseOffsets.py,
stripmapStack/denseOffsets.py, StripmapProc, Alos2Proc) only see that
parameter surface and those files.  This class keeps the surface, the grid
arithmetic (DenseAmpcor.py:368-412, checkWindows :619-648), the result
filter and the sentinels (-10000 offsets, 0 SNR, 999 covariance:
DenseAmpcor.py:441-449, 520-533), and the output layout (:536-596), and
computes every window with the PyCuAmpcor-semantics engine of this package
in one GPU call (numberThreads is accepted and ignored).

Differences from ampcor.F, by construction: the correlation, oversampling
and sub-pixel estimator are PyCuAmpcor's (amplitude chips, FFT correlation
with NCC normalisation, 2x raw oversampling, zoomed surface arg-max), not the
Fortran's; window sizes must be even; the search half-widths are the
half search ranges of PyCuAmpcor.
"""
from __future__ import annotations

import os

import numpy as np

from .pycuampcor import PyCuAmpcor, read_image

_DEFAULTS = dict(
    windowSizeWidth=64, windowSizeHeight=64, searchWindowSizeWidth=100, searchWindowSizeHeight=100,
    zoomWindowSize=16, oversamplingFactor=16, acrossGrossOffset=None, downGrossOffset=None,
    acrossLooks=1, downLooks=1, skipSampleAcross=None, skipSampleDown=None, prf1=1.0, prf2=1.0,
    rangeSpacing1=1.0, rangeSpacing2=1.0, imageDataType1="", imageDataType2="", scaling_factor=1.0,
    thresholdSNR=0.0, thresholdCov=1000.0, band1=0, band2=0, offsetImageName="dense_ampcor.bil",
    snrImageName="dense_ampcor_snr.bil", covImageName="dense_ampcor_cov.bil", margin=50,
    numberThreads=os.cpu_count() or 1)


def _is_power2(n: int) -> bool:
    return n > 0 and (n & (n - 1)) == 0


class SlcImage:
    """Minimal stand-in for an ISCE image object: a raw file (complex64, or
    float32 for real/magnitude data, or a GDAL VRT with a raw band) of
    `length` lines and `width` samples, or an in-memory array."""

    def __init__(self, filename: str | None = None, width: int | None = None, length: int | None = None,
                 data: np.ndarray | None = None, dataType: str = "CFLOAT"):
        if data is not None:
            length, width = data.shape
        self.filename, self.width, self.length, self.data, self.dataType = filename, width, length, data, dataType

    def getWidth(self) -> int:
        return int(self.width)

    def getLength(self) -> int:
        return int(self.length)

    def getDataType(self) -> str:
        return self.dataType

    def getFilename(self) -> str | None:
        return self.filename


def _as_image(obj):
    if isinstance(obj, np.ndarray):
        return SlcImage(data=obj, dataType="CFLOAT" if np.iscomplexobj(obj) else "FLOAT")
    return obj


def _load(img, kind: str) -> np.ndarray:
    data = getattr(img, "data", None)
    if data is None:
        name = img.getFilename() if hasattr(img, "getFilename") else img.filename
        if kind == "complex":
            data = read_image(name, img.getLength(), img.getWidth())
        else:
            data = np.fromfile(name, dtype=np.float32, count=img.getLength() * img.getWidth()).reshape(
                img.getLength(), img.getWidth())
    if kind == "complex":
        return np.ascontiguousarray(data, dtype=np.complex64)
    # real / magnitude data: correlated as amplitude chips
    return np.ascontiguousarray(np.abs(np.asarray(data)).astype(np.float32)).astype(np.complex64)


def write_isce_xml(path: str, width: int, length: int, bands: int, data_type: str = "FLOAT", scheme: str = "BIL"):
    """A small ISCE-style XML header beside a raw image (width, length,
    bands, data type, interleave scheme, file name)."""
    props = dict(file_name=os.path.basename(path), width=width, length=length, number_bands=bands,
                 data_type=data_type, scheme=scheme, access_mode="read", byte_order="l")
    lines = ["<imageFile>"]
    for k, v in props.items():
        lines.append(f'    <property name="{k}">\n        <value>{v}</value>\n    </property>')
    lines.append("</imageFile>")
    with open(path + ".xml", "w") as f:
        f.write("\n".join(lines) + "\n")


class DenseAmpcor:
    """DenseAmpcor's parameters, grid and outputs over the GPU engine."""

    family = "denseampcor"

    def __init__(self, **kw):
        for k, v in _DEFAULTS.items():
            setattr(self, k, v)
        for k, v in kw.items():
            if k not in _DEFAULTS:
                raise AttributeError(k)
            setattr(self, k, v)
        self.slcImage1 = None
        self.slcImage2 = None
        self.deviceID = 0

    # reference setters (DenseAmpcor.py:650-760)
    def setImageDataType1(self, v): self.imageDataType1 = str(v)
    def setImageDataType2(self, v): self.imageDataType2 = str(v)
    def setImageScalingFactor(self, v): self.scaling_factor = float(v)
    def setSkipSampleAcross(self, v): self.skipSampleAcross = int(v)
    def setSkipSampleDown(self, v): self.skipSampleDown = int(v)
    def setAcrossGrossOffset(self, v): self.acrossGrossOffset = int(v)
    def setDownGrossOffset(self, v): self.downGrossOffset = int(v)
    def setFirstPRF(self, v): self.prf1 = float(v)
    def setSecondPRF(self, v): self.prf2 = float(v)
    def setFirstRangeSpacing(self, v): self.rangeSpacing1 = float(v)
    def setSecondRangeSpacing(self, v): self.rangeSpacing2 = float(v)
    def setWindowSizeWidth(self, v): self.windowSizeWidth = int(v)
    def setWindowSizeHeight(self, v): self.windowSizeHeight = int(v)
    def setSearchWindowSizeWidth(self, v): self.searchWindowSizeWidth = int(v)
    def setSearchWindowSizeHeight(self, v): self.searchWindowSizeHeight = int(v)
    def setZoomWindowSize(self, v): self.zoomWindowSize = int(v)
    def setOversamplingFactor(self, v): self.oversamplingFactor = int(v)

    # ------------------------------------------------------------------
    def checkTypes(self):
        """DenseAmpcor.checkTypes (:597-616)."""
        for i, img in ((1, self.slcImage1), (2, self.slcImage2)):
            name = f"imageDataType{i}"
            t = getattr(self, name)
            if t == "":
                if str(img.getDataType()).upper().startswith("C"):
                    setattr(self, name, "complex")
                else:
                    raise ValueError(f"Undefined value for {name}. Should be complex/real/mag")
            elif t not in ("complex", "real", "mag"):
                raise ValueError(f"{name} should be either complex/real/mag.")

    def checkWindows(self):
        """DenseAmpcor.checkWindows (:619-648)."""
        if self.windowSizeWidth % 2 == 1:
            raise ValueError("Window size width needs to be an even number.")
        if self.windowSizeHeight % 2 == 1:
            raise ValueError("Window size height needs to be an even number.")
        if not _is_power2(self.zoomWindowSize):
            raise ValueError("Zoom window size needs to be a power of 2.")
        if not _is_power2(self.oversamplingFactor):
            raise ValueError("Oversampling factor needs to be a power of 2.")
        if self.searchWindowSizeWidth >= 2 * self.windowSizeWidth:
            raise ValueError("Search Window Size Width should be < 2 * Window Size Width")
        if self.searchWindowSizeHeight >= 2 * self.windowSizeHeight:
            raise ValueError("Search Window Size Height should be < 2 * Window Size Height")
        if self.zoomWindowSize > min(self.searchWindowSizeWidth * 2 + 1, self.searchWindowSizeHeight * 2 + 1):
            raise ValueError("Zoom window size should be <= Search window size * 2 + 1")
        self.pixLocOffAc = self.windowSizeWidth // 2 + self.searchWindowSizeWidth - 1
        self.pixLocOffDn = self.windowSizeHeight // 2 + self.searchWindowSizeHeight - 1

    def grid(self):
        """Window-centre grid (DenseAmpcor.py:368-400)."""
        coarseAcross = int(self.acrossGrossOffset or 0)
        coarseDown = int(self.downGrossOffset or 0)
        if not self.skipSampleAcross or not self.skipSampleDown:
            raise ValueError("skipSampleAcross and skipSampleDown must be set")
        xMargin = 2 * self.searchWindowSizeWidth + self.windowSizeWidth
        yMargin = 2 * self.searchWindowSizeHeight + self.windowSizeHeight
        offAc = max(self.margin, -coarseAcross) + xMargin
        if offAc % self.skipSampleAcross != 0:
            leftlim = offAc
            offAc = self.skipSampleAcross * (1 + int(offAc / self.skipSampleAcross)) - self.pixLocOffAc
            while offAc < leftlim:
                offAc += self.skipSampleAcross
        offDn = max(self.margin, -coarseDown) + yMargin
        if offDn % self.skipSampleDown != 0:
            toplim = offDn
            offDn = self.skipSampleDown * (1 + int(offDn / self.skipSampleDown)) - self.pixLocOffDn
            while offDn < toplim:
                offDn += self.skipSampleDown
        offAcmax = int(coarseAcross + ((self.rangeSpacing1 / self.rangeSpacing2) - 1) * self.lineLength1)
        lastAc = int(min(self.lineLength1, self.lineLength2 - offAcmax) - xMargin - 1 - self.margin)
        offDnmax = int(coarseDown + ((self.prf2 / self.prf1) - 1) * self.fileLength1)
        lastDn = int(min(self.fileLength1, self.fileLength2 - offDnmax) - yMargin - 1 - self.margin)
        self.gridLocAcross = range(offAc + self.pixLocOffAc, lastAc - self.pixLocOffAc, self.skipSampleAcross)
        self.gridLocDown = range(offDn + self.pixLocOffDn, lastDn - self.pixLocOffDn, self.skipSampleDown)
        if len(self.gridLocAcross) == 0 or len(self.gridLocDown) == 0:
            raise ValueError("no window fits the images with these margins and search sizes")
        startAc, endAc = offAc, self.gridLocAcross[-1] - self.pixLocOffAc
        self.numLocationAcross = int((endAc - startAc) / self.skipSampleAcross + 1)
        self.numLocationDown = len(self.gridLocDown)
        self.offsetCols, self.offsetLines = self.numLocationAcross, self.numLocationDown
        return self.gridLocDown, self.gridLocAcross

    # ------------------------------------------------------------------
    def denseampcor(self, slcImage1=None, slcImage2=None):
        """DenseAmpcor.denseampcor (:323-412): grid, GPU run, filter,
        sentinels, BIL outputs."""
        if slcImage1 is not None:
            self.slcImage1 = _as_image(slcImage1)
        if slcImage2 is not None:
            self.slcImage2 = _as_image(slcImage2)
        if self.slcImage1 is None or self.slcImage2 is None:
            raise ValueError("reference and secondary images must be set")
        self.fileLength1, self.lineLength1 = self.slcImage1.getLength(), self.slcImage1.getWidth()
        self.fileLength2, self.lineLength2 = self.slcImage2.getLength(), self.slcImage2.getWidth()
        self.checkTypes()
        self.checkWindows()
        gDn, gAc = self.grid()
        nD, nA = self.numLocationDown, self.numLocationAcross
        locDn = np.repeat(np.asarray(gDn, np.int32), nA)
        locAc = np.tile(np.asarray(gAc[:nA], np.int32), nD)
        ref = _load(self.slcImage1, self.imageDataType1)
        sec = _load(self.slcImage2, self.imageDataType2)

        obj = PyCuAmpcor()
        obj.deviceID = self.deviceID
        obj.referenceImageHeight, obj.referenceImageWidth = ref.shape
        obj.secondaryImageHeight, obj.secondaryImageWidth = sec.shape
        obj.windowSizeHeight, obj.windowSizeWidth = self.windowSizeHeight, self.windowSizeWidth
        obj.halfSearchRangeDown = self.searchWindowSizeHeight
        obj.halfSearchRangeAcross = self.searchWindowSizeWidth
        obj.skipSampleDown, obj.skipSampleAcross = self.skipSampleDown, self.skipSampleAcross
        obj.numberWindowDown, obj.numberWindowAcross = nD, nA
        obj.rawDataOversamplingFactor = 2
        obj.corrSurfaceOverSamplingFactor = self.oversamplingFactor
        obj.corrSurfaceZoomInWindow = self.zoomWindowSize
        # complex chips are oversampled before detection (deramp method 1), as
        # ampcor.F oversamples its complex chips; real / magnitude data are
        # amplitude chips already
        obj.derampMethod = 1 if self.imageDataType1 == "complex" and self.imageDataType2 == "complex" else 0
        obj.mergeGrossOffset = 1  # ampcor.F reports total offsets
        obj.setupParams()
        # window centre (W/2 - 1 past the chip start) -> chip start
        refD = locDn - (self.windowSizeHeight // 2 - 1)
        refA = locAc - (self.windowSizeWidth // 2 - 1)
        n = nD * nA
        obj.setStartPixels(refD, refA, np.full(n, int(self.downGrossOffset or 0), np.int32),
                           np.full(n, int(self.acrossGrossOffset or 0), np.int32))
        obj.checkPixelInImageRange()
        res = obj.run_arrays(ref, sec)
        off = res["offset"].reshape(n, 2)
        snr = res["snr"].reshape(n)
        cov = res["cov"].reshape(n, 3)
        cov1, cov2, cov3 = cov[:, 1], cov[:, 0], cov[:, 2]  # ampcor.F order: across, down, cross
        # ampcor.F's acceptance test (ampcor.F:668,836) with DenseAmpcor's
        # thresholds (SNR 1e-6, covariance thresholdCov), sentinels otherwise
        ok = (snr > 1.0e-6) & (cov1 < self.thresholdCov) & (cov2 < self.thresholdCov) & np.isfinite(off).all(1)
        self.locationDown = locDn.reshape(nD, nA)
        self.locationAcross = locAc.reshape(nD, nA)
        self.locationDownOffset = np.where(ok, off[:, 0], -10000.0).astype(np.float32).reshape(nD, nA)
        self.locationAcrossOffset = np.where(ok, off[:, 1], -10000.0).astype(np.float32).reshape(nD, nA)
        self.snr = np.where(ok, snr, 0.0).astype(np.float32).reshape(nD, nA)
        self.cov1 = np.where(ok, cov1, 999.0).astype(np.float32).reshape(nD, nA)
        self.cov2 = np.where(ok, cov2, 999.0).astype(np.float32).reshape(nD, nA)
        self.cov3 = np.where(ok, cov3, 999.0).astype(np.float32).reshape(nD, nA)
        self.firstSampAc, self.firstSampDown = int(locAc[0]), int(locDn[0])
        self.lastSampAc, self.lastSampDown = int(locAc[-1]), int(locDn[-1])
        # scaled like the reference, sentinels included (DenseAmpcor.py:408-409)
        self.locationDownOffset *= np.float32(self.scaling_factor)
        self.locationAcrossOffset *= np.float32(self.scaling_factor)
        self.write_slantrange_images()

    def write_slantrange_images(self):
        """BIL outputs (DenseAmpcor.py:536-596)."""
        L, C = self.offsetLines, self.offsetCols
        out = np.empty((2 * L, C), np.float32)
        out[::2] = self.locationDownOffset
        out[1::2] = self.locationAcrossOffset
        out.tofile(self.offsetImageName)
        write_isce_xml(self.offsetImageName, C, L, 2)
        self.snr.astype(np.float32).tofile(self.snrImageName)
        write_isce_xml(self.snrImageName, C, L, 1)
        cov = np.empty((3 * L, C), np.float32)
        cov[::3], cov[1::3], cov[2::3] = self.cov1, self.cov2, self.cov3
        cov.tofile(self.covImageName)
        write_isce_xml(self.covImageName, C, L, 3)
