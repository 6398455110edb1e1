"""Offset-field post-processing on the GPU: outlier culling and geometry
decimation onto the offset grid.

``Offoutliers`` keeps the interface of ISCE2's
``isceobj/Util/offoutliers/Offoutliers.py`` (setters, ``offoutliers()``,
``getIndexArray``, ``getAverageOffsetAcross/Down``, ``getRefinedLocations``,
``getRefinedOffsetField``, the ``offsets`` input port with its SNR
pre-cull) and computes on the device through ``ampcor_offoutliers``.
``cull_offset_field`` culls a dense PyCuAmpcor offset field where it lies,
without a host round trip.  ``Offsetpoly`` keeps the interface of
``stdproc/stdproc/offsetpoly/Offsetpoly.py`` and fits on the device through
``ampcor_offsetpoly``.  ``prepare_geometry`` mirrors
``contrib/PyCuAmpcor/examples/cuDenseOffsets.py:400-460`` (``prepareGeometry``)
with ``ampcor_decimate`` in place of ``gdal.Translate``.

There is no CPU implementation here: every computation goes through the CUDA
library (``_lib.lib()`` raises if it is missing).
"""
from __future__ import annotations

import ctypes
import os
import xml.etree.ElementTree as ET

import numpy as np

from . import _lib


def _torch():
    import torch

    return torch


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def offoutliers_device(loc_across, off_across, loc_down, off_down, distance: float, sig=None, snr=None,
                       snr_threshold: float | None = None, stream=None) -> dict:
    """Cull on device tensors (FP64 locations, shifts and sigmas, FP32 SNR, all
    of one length, on one CUDA device).  Returns device tensors ``index``
    (int32, the kept points' 0-based indices in input order), ``count``
    (int32, one element), ``average_across`` / ``average_down`` (float32)
    and ``fit`` (FP64: across intercept, across slope, down intercept, down
    slope).  Asynchronous on ``stream`` (the current stream by default)."""
    torch = _torch()
    xa = loc_across
    n = xa.numel()
    dev = xa.device
    for t in (off_across, loc_down, off_down) + ((sig,) if sig is not None else ()):
        if t.numel() != n or t.dtype != torch.float64 or t.device != dev or not t.is_contiguous():
            raise ValueError("locations, shifts and sigmas must be contiguous float64 tensors of one length and device")
    if xa.dtype != torch.float64 or not xa.is_contiguous():
        raise ValueError("locations must be contiguous float64")
    if snr is not None and (snr.numel() != n or snr.dtype != torch.float32 or snr.device != dev
                            or not snr.is_contiguous()):
        raise ValueError("snr must be a contiguous float32 tensor of the same length and device")
    index = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
    avg = torch.zeros(2, dtype=torch.float32, device=dev)  # average across, average down
    fit = torch.zeros(4, dtype=torch.float64, device=dev)
    count = torch.zeros(1, dtype=torch.int32, device=dev)
    st = stream if stream is not None else torch.cuda.current_stream(dev)
    use_snr = snr is not None and snr_threshold is not None
    _lib.field_check(_lib.lib().ampcor_offoutliers(
        _ptr(xa), _ptr(off_across), _ptr(loc_down), _ptr(off_down), _ptr(sig), _ptr(snr if use_snr else None),
        float(snr_threshold) if use_snr else 0.0, float(distance), n, _ptr(index), _ptr(count),
        _ptr(avg[0:1]), _ptr(avg[1:2]), _ptr(fit), ctypes.c_void_p(st.cuda_stream)))
    return {"index": index, "count": count, "average_across": avg[0:1], "average_down": avg[1:2], "fit": fit}


def cull_offset_field(offset, snr, loc_down, loc_across, distance: float, snr_threshold: float = 2.0,
                      stream=None) -> dict:
    """Cull a dense offset field on the device.  ``offset``: (nD, nA, 2)
    float32 (down, across) as PyCuAmpcor writes it; ``snr``: (nD, nA)
    float32; ``loc_down`` (nD) / ``loc_across`` (nA): the windows' pixel
    locations.  Returns ``offoutliers_device``'s dict; the indices are
    window-row-major (w = i * nA + j)."""
    torch = _torch()
    nD, nA = snr.shape
    dev = snr.device
    ld = torch.as_tensor(loc_down, dtype=torch.float64, device=dev).reshape(nD, 1).expand(nD, nA).contiguous()
    la = torch.as_tensor(loc_across, dtype=torch.float64, device=dev).reshape(1, nA).expand(nD, nA).contiguous()
    off = offset.reshape(nD * nA, 2)
    return offoutliers_device(la.reshape(-1), off[:, 1].to(torch.float64).contiguous(), ld.reshape(-1),
                              off[:, 0].to(torch.float64).contiguous(), distance,
                              snr=snr.reshape(-1).contiguous(), snr_threshold=snr_threshold, stream=stream)


def offsetpoly_device(loc_across, loc_down, offset, snr, ncoef: int = 6, stream=None) -> dict:
    """Offset polynomial on device tensors (FP64, one length, one device).
    Returns device tensors ``coef`` (FP64, ncoef) and ``rank`` (int32, the
    design matrix's singular values kept).  Asynchronous on ``stream``."""
    torch = _torch()
    n = loc_across.numel()
    dev = loc_across.device
    for t in (loc_across, loc_down, offset, snr):
        if t.numel() != n or t.dtype != torch.float64 or t.device != dev or not t.is_contiguous():
            raise ValueError("locations, offsets and SNRs must be contiguous float64 tensors of one length and device")
    coef = torch.zeros(max(int(ncoef), 1), dtype=torch.float64, device=dev)
    rank = torch.zeros(1, dtype=torch.int32, device=dev)
    st = stream if stream is not None else torch.cuda.current_stream(dev)
    _lib.field_check(_lib.lib().ampcor_offsetpoly(_ptr(loc_across), _ptr(loc_down), _ptr(offset), _ptr(snr), n,
                                                  int(ncoef), _ptr(coef), _ptr(rank), ctypes.c_void_p(st.cuda_stream)))
    return {"coef": coef, "rank": rank}


class Offsetpoly:
    """Drop-in for ``stdproc.stdproc.offsetpoly.Offsetpoly``
    (``Offsetpoly.py``): set the locations, offsets and SNRs, call
    ``offsetpoly()``, read ``offsetPoly``; the fit runs on the GPU."""

    def __init__(self):
        self.numberFitCoefficients = 6
        self.numberOffsets = None
        self.locationAcross = []
        self.offset = []
        self.locationDown = []
        self.snr = []
        self.offsetPoly = []
        self.downOffsetPoly = []
        self.deviceID = 0

    def setNumberFitCoefficients(self, var):
        self.numberFitCoefficients = int(var)

    def setLocationAcross(self, var):
        self.locationAcross = var

    def setOffset(self, var):
        self.offset = var

    def setLocationDown(self, var):
        self.locationDown = var

    def setSNR(self, var):
        self.snr = var

    def offsetpoly(self):
        torch = _torch()
        self.numberOffsets = len(self.offset)
        n = self.numberOffsets
        for name in ("locationAcross", "locationDown", "snr"):
            if len(getattr(self, name)) != n:
                raise ValueError(f"{name} has {len(getattr(self, name))} entries, offset {n}")
        dev = torch.device("cuda", self.deviceID)

        def d64(v):
            return torch.as_tensor(np.asarray(v, np.float64), device=dev)

        r = offsetpoly_device(d64(self.locationAcross), d64(self.locationDown), d64(self.offset), d64(self.snr),
                              self.numberFitCoefficients)
        self.offsetPoly = r["coef"].cpu().tolist()


class RefinedOffset:
    """One offset of a refined field (the accessors callers of the
    reference's Offset use)."""

    def __init__(self, across, down, dx, dy, snr):
        self.x, self.y, self.dx, self.dy, self.snr = across, down, dx, dy, snr

    def getCoordinate(self):
        return self.x, self.y

    def getOffset(self):
        return self.dx, self.dy

    def getSignalToNoise(self):
        return self.snr


class Offoutliers:
    """Drop-in for ``isceobj.Util.Offoutliers`` (``Offoutliers.py:37-279``)."""

    def __init__(self):
        self.snrThreshold = 0
        self.indexArray = []
        self.indexArraySize = None
        self.averageOffsetDown = None
        self.averageOffsetAcross = None
        self.numPoints = None
        self.locationAcross = []
        self.locationAcrossOffset = []
        self.locationDown = []
        self.locationDownOffset = []
        self.distance = None
        self.sig = []
        self.snr = []
        self.deviceID = 0
        self._offsets = None

    # input port 'offsets' (Offoutliers.py:78-80,262-279)
    def wireInputPort(self, name="offsets", object=None):
        if name != "offsets":
            raise ValueError(f"unknown port {name}")
        self._offsets = object

    def addOffsets(self):
        offsets = self._offsets
        if not offsets:
            return
        for offset in offsets:
            if offset.getSignalToNoise() < self.snrThreshold:  # OffsetField.cull (Offset.py:364-378)
                continue
            across, down = offset.getCoordinate()
            acrossOffset, downOffset = offset.getOffset()
            self.locationAcross.append(across)
            self.locationDown.append(down)
            self.locationAcrossOffset.append(acrossOffset)
            self.locationDownOffset.append(downOffset)
            self.snr.append(offset.getSignalToNoise())
            self.sig.append(1.0)

    def offoutliers(self):
        """Cull (Offoutliers.py:82-92): fit, distances and selection on the GPU."""
        torch = _torch()
        self.addOffsets()
        self._offsets = None
        self.numPoints = len(self.locationAcross)
        n = self.numPoints
        if not n:
            print("Error. Trying to allocate zero size array")
            raise Exception("Trying to allocate zero size array")
        for name in ("locationAcrossOffset", "locationDown", "locationDownOffset", "sig", "snr"):
            if len(getattr(self, name)) != n:
                print("Error. Trying to allocate zero size array")
                raise Exception(f"{name} has {len(getattr(self, name))} entries, locationAcross {n}")
        if self.distance is None:
            raise ValueError("distance is not set")
        dev = torch.device("cuda", self.deviceID)

        def d64(v):
            return torch.as_tensor(np.asarray(v, np.float64), device=dev)

        r = offoutliers_device(d64(self.locationAcross), d64(self.locationAcrossOffset), d64(self.locationDown),
                               d64(self.locationDownOffset), self.distance, sig=d64(self.sig))
        cnt = int(r["count"].item())
        self.indexArraySize = cnt
        self.indexArray = r["index"][:cnt].cpu().tolist()
        self.averageOffsetAcross = float(r["average_across"].item())
        self.averageOffsetDown = float(r["average_down"].item())

    def setNumberOfPoints(self, var):
        self.numPoints = int(var)

    def setLocationAcross(self, var):
        self.locationAcross = var

    def setLocationAcrossOffset(self, var):
        self.locationAcrossOffset = var

    def setLocationDown(self, var):
        self.locationDown = var

    def setLocationDownOffset(self, var):
        self.locationDownOffset = var

    def setDistance(self, var):
        self.distance = float(var)

    def setSign(self, var):
        """The per-point sigmas of the fits (the reference's name)."""
        self.sig = var

    def setSNR(self, var):
        self.snr = var

    def setSNRThreshold(self, var):
        self.snrThreshold = var

    def setStdWriter(self, var):
        self.stdWriter = var

    def getIndexArray(self):
        return self.indexArray

    def getAverageOffsetDown(self):
        return self.averageOffsetDown

    def getAverageOffsetAcross(self):
        return self.averageOffsetAcross

    def getRefinedLocations(self):
        idx = self.indexArray
        return [[self.locationAcross[i] for i in idx], [self.locationAcrossOffset[i] for i in idx],
                [self.locationDown[i] for i in idx], [self.locationDownOffset[i] for i in idx],
                [self.snr[i] for i in idx], [self.sig[i] for i in idx]]

    def getRefinedOffsetField(self):
        return [RefinedOffset(self.locationAcross[i], self.locationDown[i], self.locationAcrossOffset[i],
                              self.locationDownOffset[i], self.snr[i]) for i in self.indexArray]


def decimate(src, y0: int, x0: int, ystep: int, xstep: int, rows: int, cols: int, stream=None):
    """Nearest-neighbour decimation of a 2-D device tensor (row stride any,
    unit column stride) onto rows x cols; zero outside the source."""
    torch = _torch()
    if src.dim() != 2 or src.stride(1) != 1:
        raise ValueError("src must be a 2-D tensor with unit column stride")
    dst = torch.empty((rows, cols), dtype=src.dtype, device=src.device)
    st = stream if stream is not None else torch.cuda.current_stream(src.device)
    _lib.field_check(_lib.lib().ampcor_decimate(
        _ptr(src), src.shape[0], src.shape[1], src.stride(0), src.element_size(), int(y0), int(x0), int(ystep),
        int(xstep), _ptr(dst), int(rows), int(cols), ctypes.c_void_p(st.cuda_stream)))
    return dst


# raster I/O for prepare_geometry: VRT raw bands in, raw BSQ + ENVI header +
# VRT out (GDAL's ENVI driver writes band-sequential by default)
_GDAL_TYPES = {"Byte": np.uint8, "Int16": np.int16, "UInt16": np.uint16, "Int32": np.int32, "UInt32": np.uint32,
               "Float32": np.float32, "Float64": np.float64}
_ENVI_CODES = {np.uint8: 1, np.int16: 2, np.int32: 3, np.float32: 4, np.float64: 5, np.uint16: 12, np.uint32: 13}


def read_vrt_bands(path: str) -> list[np.ndarray]:
    """Bands of a VRT over a raw file (VRTRawRasterBand), as 2-D arrays."""
    root = ET.parse(path).getroot()
    H, W = int(root.get("rasterYSize")), int(root.get("rasterXSize"))
    bands = []
    for band in root.findall("VRTRasterBand"):
        dt = np.dtype(_GDAL_TYPES[band.get("dataType", "Float32")])
        src = band.find("SourceFilename")
        fn = os.path.join(os.path.dirname(path), src.text) if src.get("relativeToVRT", "0") == "1" else src.text
        off = int(band.findtext("ImageOffset") or 0)
        pix = int(band.findtext("PixelOffset") or dt.itemsize)
        line = int(band.findtext("LineOffset") or pix * W)
        order = (band.findtext("ByteOrder") or "LSB").upper()
        dt = dt.newbyteorder("<" if order.startswith("LSB") else ">")
        mm = np.memmap(fn, dtype=np.uint8, mode="r")
        if off + (H - 1) * line + (W - 1) * pix + dt.itemsize > mm.shape[0]:
            raise ValueError(f"{fn}: {mm.shape[0]} bytes is too short for the {H} x {W} band of {path}")
        rows = np.lib.stride_tricks.as_strided(mm[off:], shape=(H, W, dt.itemsize), strides=(line, pix, 1))
        bands.append(np.ascontiguousarray(rows).view(dt).reshape(H, W).astype(dt.newbyteorder("=")))
    return bands


def write_raster(path: str, bands: list[np.ndarray]) -> None:
    """Raw band-sequential file, an ENVI header beside it and a VRT."""
    H, W = bands[0].shape
    dt = bands[0].dtype
    with open(path, "wb") as f:
        for b in bands:
            f.write(np.ascontiguousarray(b).tobytes())
    code = _ENVI_CODES[dt.type]
    with open(path + ".hdr", "w") as f:
        f.write(f"ENVI\nsamples = {W}\nlines = {H}\nbands = {len(bands)}\nheader offset = 0\n"
                f"file type = ENVI Standard\ndata type = {code}\ninterleave = bsq\nbyte order = 0\n"
                f"data ignore value = 0\n")
    name = {v: k for k, v in _GDAL_TYPES.items()}[dt.type]
    parts = [f'<VRTDataset rasterXSize="{W}" rasterYSize="{H}">']
    for k in range(len(bands)):
        parts.append(
            f'  <VRTRasterBand dataType="{name}" band="{k + 1}" subClass="VRTRawRasterBand">\n'
            f"    <NoDataValue>0</NoDataValue>\n"
            f'    <SourceFilename relativeToVRT="1">{os.path.basename(path)}</SourceFilename>\n'
            f"    <ImageOffset>{k * H * W * dt.itemsize}</ImageOffset>\n"
            f"    <PixelOffset>{dt.itemsize}</PixelOffset>\n    <LineOffset>{W * dt.itemsize}</LineOffset>\n"
            f"    <ByteOrder>LSB</ByteOrder>\n  </VRTRasterBand>")
    parts.append("</VRTDataset>\n")
    with open(path + ".vrt", "w") as f:
        f.write("\n".join(parts))


def prepare_geometry(full_dir, out_dir, x_start, y_start, x_step, y_step, x_win_num, y_win_num,
                     fbases=("lat", "lon", "los", "hgt", "z", "shadowMask", "waterMask"), device: int = 0):
    """Geometry rasters on the offset grid (cuDenseOffsets.py:400-460): for
    each ``{f}.rdr.full`` (or ``{f}.rdr`` when ``out_dir`` differs) with a
    ``.vrt`` header in ``full_dir``, the source window starting at
    (x_start, y_start) of x_win_num*x_step x y_win_num*y_step pixels is
    sampled onto x_win_num x y_win_num by nearest neighbour on the GPU and
    written to ``out_dir/{f}.rdr`` (+ ``.hdr``, ``.vrt``).  Returns the
    written paths."""
    torch = _torch()
    full_dir = os.path.abspath(full_dir)
    out_dir = os.path.abspath(out_dir)
    exts = [".rdr.full", ".rdr"] if full_dir != out_dir else [".rdr.full"]
    exts = [e for e in exts if os.path.isfile(os.path.join(full_dir, f"{fbases[0]}{e}"))]
    if not exts:
        raise ValueError(f"No full resolution {fbases[0]}.rdr* file found in: {full_dir}")
    ext = exts[0]
    os.makedirs(out_dir, exist_ok=True)
    dev = torch.device("cuda", device)
    written = []
    for f in fbases:
        src = os.path.join(full_dir, f"{f}{ext}")
        if not os.path.isfile(src):
            continue
        vrt = src + ".vrt"
        if not os.path.isfile(vrt):
            raise ValueError(f"{src}: no .vrt header beside it")
        bands = read_vrt_bands(vrt)
        outs = []
        for b in bands:
            d = torch.from_numpy(b).to(dev)
            outs.append(decimate(d, y_start, x_start, y_step, x_step, y_win_num, x_win_num).cpu().numpy())
        dst = os.path.join(out_dir, f"{f}.rdr")
        write_raster(dst, outs)
        written.append(dst)
    return written
