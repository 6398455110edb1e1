"""Batched runs: many offset jobs of any geometry in one persistent launch.

Each job is a set-up ``PyCuAmpcor`` (after ``setupParams`` and a gross-offset
setter) with its two device-resident images; the outputs are allocated per
job.  ``run`` processes every window of every job in one persistent kernel
(work queue ordered by decreasing cost), optionally replayed from a captured
CUDA graph; ``tune`` times the feasible launch shapes and keeps the fastest.
"""
from __future__ import annotations

import ctypes

from . import _lib


class AmpcorBatch:
    def __init__(self, device: int = 0):
        self._h = ctypes.c_void_p()
        _lib.check(None, _lib.lib().ampcor_batch_create(ctypes.byref(self._h), device))
        self.device = device
        self.jobs = []

    def _check(self, code: int):
        if code != _lib.AMPCOR_OK:
            buf = ctypes.create_string_buffer(1024)
            _lib.lib().ampcor_batch_last_error(self._h, buf, len(buf))
            msg = buf.value.decode(errors="replace")
            if code in (_lib.AMPCOR_ERR_ARG, _lib.AMPCOR_ERR_RANGE):
                raise ValueError(f"[ampcor status {code}] {msg}")
            raise _lib.AmpcorError(code, msg)

    def add(self, obj, reference, secondary, out: dict | None = None) -> dict:
        """Add a job; returns its output tensors (filled by ``run``)."""
        import torch

        for t in (reference, secondary):
            if not (t.is_cuda and t.dtype == torch.complex64 and t.dim() == 2 and t.stride(1) == 1):
                raise ValueError("images must be 2-D complex64 CUDA tensors with unit column stride")
        nD, nA = obj.numberWindowDown, obj.numberWindowAcross
        dev = reference.device
        if out is None:
            out = {"offset": torch.empty((nD, nA, 2), dtype=torch.float32, device=dev),
                   "snr": torch.empty((nD, nA), dtype=torch.float32, device=dev),
                   "cov": torch.empty((nD, nA, 3), dtype=torch.float32, device=dev)}
        idx = ctypes.c_int32()
        self._check(_lib.lib().ampcor_batch_add(
            self._h, obj._h, reference.data_ptr(), reference.stride(0), secondary.data_ptr(), secondary.stride(0),
            out["offset"].data_ptr(), out["snr"].data_ptr(), out["cov"].data_ptr(), ctypes.byref(idx)))
        self.jobs.append((obj, reference, secondary, out))  # keep the tensors alive
        return out

    def run(self, stream=None, graph: bool = False):
        import torch

        st = stream if stream is not None else torch.cuda.current_stream()
        self._check(_lib.lib().ampcor_batch_run(self._h, ctypes.c_void_p(st.cuda_stream), 1 if graph else 0))

    def synchronize(self, stream=None):
        """Wait for the batch's work; raises if a bounded device wait gave up."""
        import torch

        st = stream if stream is not None else torch.cuda.current_stream()
        self._check(_lib.lib().ampcor_batch_sync(self._h, ctypes.c_void_p(st.cuda_stream)))

    def tune(self, stream=None) -> dict:
        import numpy as np
        import torch

        st = stream if stream is not None else torch.cuda.current_stream()
        ms = np.zeros(len(_lib.BATCH_TUNE_CANDIDATES), np.float32)
        self._check(_lib.lib().ampcor_batch_tune(self._h, ctypes.c_void_p(st.cuda_stream), ms.ctypes.data))
        cfg = self.config()
        cfg["candidates_ms"] = {k: float(v) for k, v in zip(_lib.BATCH_TUNE_CANDIDATES, ms)}
        return cfg

    def set_timing(self, enable: bool):
        self._check(_lib.lib().ampcor_batch_set_timing(self._h, 1 if enable else 0))

    def read_timing(self) -> dict:
        """{stage: (milliseconds, launches)} of chain-mode runs since the last read."""
        import numpy as np

        ms = np.zeros(4, np.float32)
        n = np.zeros(4, np.int64)
        self._check(_lib.lib().ampcor_batch_read_timing(self._h, ms.ctypes.data, n.ctypes.data, 4))
        return {k: (float(a), int(c)) for k, a, c in zip(_lib.STAGES, ms, n)}

    def set_shape(self, name: str):
        """Use one of the tuner's launch shapes (see ``_lib.BATCH_TUNE_CANDIDATES``)."""
        self._check(_lib.lib().ampcor_batch_set_shape(self._h, _lib.BATCH_TUNE_CANDIDATES.index(name)))

    def config(self) -> dict:
        nt, per, grid, n, l2 = (ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int64(),
                                ctypes.c_int32())
        self._check(_lib.lib().ampcor_batch_config(self._h, ctypes.byref(nt), ctypes.byref(per), ctypes.byref(grid),
                                                   ctypes.byref(n), ctypes.byref(l2)))
        return {"threads": nt.value, "ctas_per_sm": per.value, "grid": grid.value, "windows": n.value,
                "raw_tile": "l2" if l2.value & 1 else "auto", "mode": "chain" if l2.value & 4 else "fused"}

    def clear(self):
        self._check(_lib.lib().ampcor_batch_clear(self._h))
        self.jobs = []

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.lib().ampcor_batch_destroy(h)
            except Exception:
                pass
            self._h = ctypes.c_void_p()
