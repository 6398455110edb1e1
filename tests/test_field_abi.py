"""The offset-field entry points' argument checks through the C ABI, without
a GPU: every rejected call returns before any CUDA call, with a status code
and a message for ampcor_field_last_error."""
import ctypes

import pytest

from isce2_gb300 import _lib

NULL = ctypes.c_void_p(0)
DUMMY = ctypes.c_void_p(64)  # never dereferenced: the checks fail first


def last_error(L):
    buf = ctypes.create_string_buffer(512)
    assert L.ampcor_field_last_error(buf, len(buf)) == _lib.AMPCOR_OK
    return buf.value.decode()


def test_offoutliers_rejects_empty_and_null(built_lib):
    L = built_lib
    rc = L.ampcor_offoutliers(DUMMY, DUMMY, DUMMY, DUMMY, NULL, NULL, 0.0, 1.0, 0, DUMMY, DUMMY, NULL, NULL, NULL,
                              NULL)
    assert rc == _lib.AMPCOR_ERR_ARG and "no offsets" in last_error(L)
    rc = L.ampcor_offoutliers(NULL, DUMMY, DUMMY, DUMMY, NULL, NULL, 0.0, 1.0, 10, DUMMY, DUMMY, NULL, NULL, NULL,
                              NULL)
    assert rc == _lib.AMPCOR_ERR_ARG and "null" in last_error(L)
    rc = L.ampcor_offoutliers(DUMMY, DUMMY, DUMMY, DUMMY, NULL, NULL, 0.0, 1.0, 1 << 31, DUMMY, DUMMY, NULL, NULL,
                              NULL, NULL)
    assert rc == _lib.AMPCOR_ERR_ARG and "too many" in last_error(L)


@pytest.mark.parametrize("ncoef", [0, 11])
def test_offsetpoly_rejects_coefficient_counts(built_lib, ncoef):
    L = built_lib
    rc = L.ampcor_offsetpoly(DUMMY, DUMMY, DUMMY, DUMMY, 10, ncoef, DUMMY, NULL, NULL)
    assert rc == _lib.AMPCOR_ERR_ARG and "coefficients" in last_error(L)


def test_offsetpoly_rejects_empty_and_null(built_lib):
    L = built_lib
    assert L.ampcor_offsetpoly(DUMMY, DUMMY, DUMMY, DUMMY, 0, 6, DUMMY, NULL, NULL) == _lib.AMPCOR_ERR_ARG
    assert L.ampcor_offsetpoly(DUMMY, DUMMY, NULL, DUMMY, 5, 6, DUMMY, NULL, NULL) == _lib.AMPCOR_ERR_ARG
    assert "null" in last_error(L)


@pytest.mark.parametrize("args,msg", [
    ((100, 100, 100, 4, 0, 0, 2, 2, 0, 10), "bad sizes"),      # rows 0
    ((100, 100, 50, 4, 0, 0, 2, 2, 10, 10), "bad sizes"),      # leading dimension below the width
    ((100, 100, 100, 4, 0, 0, 0, 2, 10, 10), "bad sizes"),     # step 0
    ((100, 100, 100, 3, 0, 0, 2, 2, 10, 10), "element size"),  # 3-byte elements
])
def test_decimate_rejects_bad_arguments(built_lib, args, msg):
    L = built_lib
    sr, sc, ld, eb, y0, x0, ys, xs, rows, cols = args
    rc = L.ampcor_decimate(DUMMY, sr, sc, ld, eb, y0, x0, ys, xs, DUMMY, rows, cols, NULL)
    assert rc == _lib.AMPCOR_ERR_ARG and msg in last_error(L)
    assert L.ampcor_decimate(NULL, 10, 10, 10, 4, 0, 0, 1, 1, DUMMY, 1, 1, NULL) == _lib.AMPCOR_ERR_ARG
