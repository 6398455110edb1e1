"""ctypes binding of ``libampcor_gb.so`` (the C ABI in include/ampcor_gb.h).

There is no CPU implementation behind this module: if the library cannot be
loaded, ``lib()`` raises.  Run ``isce2_gb300.build.build()`` (or
``python -m isce2_gb300.build``) to compile it in-tree for sm_103a.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libampcor_gb.so")

AMPCOR_OK = 0
AMPCOR_ERR_ARG = 1
AMPCOR_ERR_RANGE = 2
AMPCOR_ERR_UNSUPPORTED = 3
AMPCOR_ERR_CUDA = 4
AMPCOR_ERR_STATE = 5
AMPCOR_ERR_ALLOC = 6

BATCH_TUNE_CANDIDATES = ["512x1", "256x1", "256x2", "512x1/rawL2", "256x2/rawL2", "chain"]

PARAM_FIELDS = [
    "algorithm", "deviceID", "nStreams", "derampMethod",
    "referenceImageHeight", "referenceImageWidth", "secondaryImageHeight", "secondaryImageWidth",
    "numberWindowDown", "numberWindowAcross", "windowSizeHeight", "windowSizeWidth",
    "halfSearchRangeDown", "halfSearchRangeAcross", "skipSampleDown", "skipSampleAcross",
    "referenceStartPixelDownStatic", "referenceStartPixelAcrossStatic",
    "rawDataOversamplingFactor", "corrStatWindowSize", "corrSurfaceOverSamplingMethod",
    "corrSurfaceOverSamplingFactor", "corrSurfaceZoomInWindow",
    "numberWindowDownInChunk", "numberWindowAcrossInChunk", "mergeGrossOffset", "useMmap", "mmapSize",
]

STAGES = ["raw_correlation", "oversample", "oversampled_correlation", "surface_zoom"]
STAGE_KERNELS = ["k_raw", "k_oversample2", "k_corr_os_tma", "k_zoom"]

GEOMETRY_FIELDS = [
    "numberWindows", "searchWindowSizeHeightRaw", "searchWindowSizeWidthRaw", "zoomWindowSize",
    "halfZoomWindowSizeRaw", "corrRawZoomInHeight", "corrRawZoomInWidth", "fftHeight", "fftWidth",
]


class AmpcorParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in PARAM_FIELDS]


class AmpcorGeometry(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in GEOMETRY_FIELDS]


class AmpcorError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[ampcor status {code}] {msg}")
        self.code = code


_LIB = None

_SIGS = {
    "ampcor_params_default": (None, [ctypes.POINTER(AmpcorParams)]),
    "ampcor_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p)]),
    "ampcor_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "ampcor_set_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(AmpcorParams)]),
    "ampcor_get_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(AmpcorParams)]),
    "ampcor_setup": (ctypes.c_int, [ctypes.c_void_p]),
    "ampcor_get_geometry": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(AmpcorGeometry)]),
    "ampcor_set_constant_gross_offset": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32]),
    "ampcor_set_varying_gross_offset": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]),
    "ampcor_set_start_pixels": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]),
    "ampcor_get_start_pixels": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]),
    "ampcor_check_range": (ctypes.c_int, [ctypes.c_void_p]),
    "ampcor_run_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                         ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p]),
    "ampcor_run_host": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                       ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p]),
    "ampcor_run_device_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                                 ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                 ctypes.c_void_p]),
    "ampcor_run_status": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "ampcor_selftest_wait_timeout": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p]),
    "ampcor_set_timing": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "ampcor_set_raw_mode": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "ampcor_set_precision": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "ampcor_set_corr_precision": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "ampcor_read_timing": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]),
    "ampcor_batch_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int32]),
    "ampcor_batch_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "ampcor_batch_clear": (ctypes.c_int, [ctypes.c_void_p]),
    "ampcor_batch_add": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                        ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p]),
    "ampcor_batch_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]),
    "ampcor_batch_tune": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "ampcor_batch_config": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_void_p]),
    "ampcor_batch_sync": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "ampcor_batch_set_shape": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "ampcor_batch_set_timing": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "ampcor_batch_read_timing": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]),
    "ampcor_batch_last_error": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int64]),
    "ampcor_server_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int32, ctypes.c_int64,
                                            ctypes.c_int32]),
    "ampcor_server_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "ampcor_server_submit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                            ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p]),
    "ampcor_server_progress": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "ampcor_server_poll": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]),
    "ampcor_server_take": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_int32]),
    "ampcor_server_request_info": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                                  ctypes.c_void_p, ctypes.c_void_p]),
    "ampcor_server_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]),
    "ampcor_server_last_error": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int64]),
    "ampcor_last_error": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int64]),
    "ampcor_offoutliers": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_float,
                                          ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "ampcor_decimate": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                       ctypes.c_int32, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                       ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                       ctypes.c_void_p]),
    "ampcor_offsetpoly": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p]),
    "ampcor_field_last_error": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int64]),
    "ampcor_version": (ctypes.c_char_p, []),
}


def lib(path: str | None = None):
    """Load the library (once).  Raises OSError if it is absent."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise OSError(f"{p} is missing: build it with isce2_gb300.build.build() (nvcc, sm_103a)")
    L = ctypes.CDLL(p)
    for name, (res, args) in _SIGS.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _LIB = L
    return L


def exported_symbols() -> list[str]:
    return list(_SIGS)


def last_error(handle) -> str:
    buf = ctypes.create_string_buffer(1024)
    lib().ampcor_last_error(handle, buf, len(buf))
    return buf.value.decode(errors="replace")


def field_check(code: int) -> None:
    """Raise for a failing offset-field call (ampcor_offoutliers, ampcor_offsetpoly, ampcor_decimate)."""
    if code != AMPCOR_OK:
        buf = ctypes.create_string_buffer(1024)
        lib().ampcor_field_last_error(buf, len(buf))
        msg = buf.value.decode(errors="replace")
        if code == AMPCOR_ERR_ARG:
            raise ValueError(f"[ampcor status {code}] {msg}")
        raise AmpcorError(code, msg)


def check(handle, code: int) -> None:
    if code != AMPCOR_OK:
        msg = last_error(handle) if handle else ""
        if code in (AMPCOR_ERR_ARG, AMPCOR_ERR_RANGE):
            raise ValueError(f"[ampcor status {code}] {msg}")
        raise AmpcorError(code, msg)
