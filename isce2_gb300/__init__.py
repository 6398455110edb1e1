"""GB300-native dense amplitude cross-correlation (ampcor) offset estimator.

A from-scratch sm_103a implementation of the offset estimator that ISCE2
ships as ``contrib/PyCuAmpcor`` (GPU) and ``mroipac/ampcor`` (CPU), behind
the same ``PyCuAmpcor`` parameter surface and a C ABI (include/ampcor_gb.h).
"""
from .pycuampcor import PyCuAmpcor, read_image  # noqa: F401
from ._lib import AmpcorError  # noqa: F401
from .batch import AmpcorBatch  # noqa: F401
from .server import AmpcorServer  # noqa: F401
from .denseampcor import DenseAmpcor  # noqa: F401
from .offsets import Offoutliers, Offsetpoly, cull_offset_field, prepare_geometry  # noqa: F401

__all__ = ["PyCuAmpcor", "AmpcorBatch", "AmpcorServer", "DenseAmpcor", "AmpcorError", "read_image", "Offoutliers", "Offsetpoly",
           "cull_offset_field", "prepare_geometry"]
