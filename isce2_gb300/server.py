"""Offset-tracking request server: continuous batching on one GPU.

A thin wrapper of the native server in ``libampcor_gb.so``
(``ampcor_server_*`` in include/ampcor_gb.h).  The host loop calls
``progress()`` often; it never blocks.  Requests are admitted in arrival
order while their device memory fits the HBM budget, and every step the GPU
runs mixes the windows of all admitted requests.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

STATE_QUEUED, STATE_ACTIVE, STATE_COMPLETE = 0, 1, 2
STAT_NAMES = ["queued", "active", "steps_in_flight", "bytes_used", "peak_bytes", "steps_launched",
              "windows_done", "peak_active"]


class AmpcorServer:
    def __init__(self, device: int = 0, hbm_budget_bytes: int = 150 * 10 ** 9, step_windows: int = 8192,
                 stream=None):
        import torch

        self._h = ctypes.c_void_p()
        _lib.check(None, _lib.lib().ampcor_server_create(ctypes.byref(self._h), device, int(hbm_budget_bytes),
                                                         int(step_windows)))
        self.device = device
        self.stream = stream if stream is not None else torch.cuda.Stream(device)
        self._src = {}   # request id -> (handle object, source images) kept alive until taken
        self._shape = {}

    def _check(self, code: int):
        if code != _lib.AMPCOR_OK:
            buf = ctypes.create_string_buffer(1024)
            _lib.lib().ampcor_server_last_error(self._h, buf, len(buf))
            msg = buf.value.decode(errors="replace")
            if code in (_lib.AMPCOR_ERR_ARG, _lib.AMPCOR_ERR_RANGE):
                raise ValueError(f"[ampcor status {code}] {msg}")
            raise _lib.AmpcorError(code, msg)

    def submit(self, obj, reference, secondary) -> int:
        """Queue a request: a set-up PyCuAmpcor and its images (2-D complex64
        CUDA tensors or NumPy arrays; kept referenced until taken)."""
        on_dev = hasattr(reference, "is_cuda") and reference.is_cuda
        if on_dev:
            ptrs = (reference.data_ptr(), reference.stride(0), secondary.data_ptr(), secondary.stride(0))
        else:
            reference = np.ascontiguousarray(reference, dtype=np.complex64)
            secondary = np.ascontiguousarray(secondary, dtype=np.complex64)
            ptrs = (reference.ctypes.data, reference.shape[1], secondary.ctypes.data, secondary.shape[1])
        rid = ctypes.c_int64()
        self._check(_lib.lib().ampcor_server_submit(self._h, obj._h, ptrs[0], ptrs[1], ptrs[2], ptrs[3],
                                                    1 if on_dev else 0, ctypes.byref(rid)))
        self._src[rid.value] = (obj, reference, secondary)
        self._shape[rid.value] = (obj.numberWindowDown, obj.numberWindowAcross)
        return rid.value

    def progress(self) -> bool:
        """Retire, admit and launch; True while any request is unfinished."""
        busy = ctypes.c_int32()
        self._check(_lib.lib().ampcor_server_progress(self._h, ctypes.c_void_p(self.stream.cuda_stream),
                                                      ctypes.byref(busy)))
        return bool(busy.value)

    def poll(self, max_ids: int = 1024) -> list[int]:
        ids = np.zeros(max_ids, np.int64)
        n = ctypes.c_int32()
        self._check(_lib.lib().ampcor_server_poll(self._h, ids.ctypes.data, max_ids, ctypes.byref(n)))
        return [int(x) for x in ids[:n.value]]

    def info(self, rid: int) -> dict:
        st, nw = ctypes.c_int32(), ctypes.c_int32()
        t = np.zeros(3, np.float64)
        self._check(_lib.lib().ampcor_server_request_info(self._h, rid, ctypes.byref(st), ctypes.byref(nw),
                                                          t.ctypes.data))
        return {"state": st.value, "windows": nw.value, "submitted": float(t[0]), "admitted": float(t[1]),
                "completed": float(t[2])}

    def take(self, rid: int, device: bool = False) -> dict:
        """Fields of a completed request (host NumPy arrays, or CUDA tensors
        with device=True); frees its device memory."""
        nD, nA = self._shape[rid]
        if device:
            import torch
            dev = torch.device("cuda", self.device)
            out = {"offset": torch.empty((nD, nA, 2), dtype=torch.float32, device=dev),
                   "snr": torch.empty((nD, nA), dtype=torch.float32, device=dev),
                   "cov": torch.empty((nD, nA, 3), dtype=torch.float32, device=dev)}
            ptr = {k: v.data_ptr() for k, v in out.items()}
        else:
            out = {"offset": np.empty((nD, nA, 2), np.float32), "snr": np.empty((nD, nA), np.float32),
                   "cov": np.empty((nD, nA, 3), np.float32)}
            ptr = {k: v.ctypes.data for k, v in out.items()}
        self._check(_lib.lib().ampcor_server_take(self._h, rid, ptr["offset"], ptr["snr"], ptr["cov"],
                                                  1 if device else 0))
        self._src.pop(rid, None)
        self._shape.pop(rid, None)
        return out

    def stats(self) -> dict:
        v = np.zeros(len(STAT_NAMES), np.int64)
        self._check(_lib.lib().ampcor_server_stats(self._h, v.ctypes.data, len(STAT_NAMES)))
        return {k: int(x) for k, x in zip(STAT_NAMES, v)}

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.lib().ampcor_server_destroy(h)
            except Exception:
                pass
            self._h = ctypes.c_void_p()
