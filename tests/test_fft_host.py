"""The shared-memory FFT pass functions driven sequentially on the CPU
(tests/fft_host_harness.cpp) against numpy, for the transform lengths the
kernels use."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    out = str(tmp_path_factory.mktemp("fft") / "harness.so")
    inc = [p for p in ("/usr/local/cuda/include",) if os.path.isdir(p)]
    cmd = [gxx, "-O2", "-std=c++17", "-shared", "-fPIC", *sum([["-I", p] for p in inc], []),
           "-I", os.path.join(ROOT, "isce2_gb300", "csrc"), os.path.join(HERE, "fft_host_harness.cpp"), "-o", out]
    subprocess.run(cmd, check=True)
    L = ctypes.CDLL(out)
    L.h_fft2.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    return L


SIZES = [(8, 8), (105, 105), (192, 128), (136, 72), (256, 128), (17, 13), (30, 42), (41, 41), (2, 2), (7, 1),
         (1, 5), (22, 38), (26, 34), (121, 11), (214, 6), (262, 4), (4, 254), (46, 58), (667, 2), (2, 529),
         (128, 192), (144, 96), (160, 48), (256, 12), (36, 6)]


@pytest.mark.parametrize("n1,n2", SIZES)
@pytest.mark.parametrize("sign", [-1, 1])
def test_dif_and_dit_against_numpy(harness, n1, n2, sign):
    rng = np.random.default_rng(n1 * 1000 + n2)
    x = (rng.standard_normal((n1, n2)) + 1j * rng.standard_normal((n1, n2))).astype(np.complex64)
    d = x.copy()
    assert harness.h_fft2(1, d.ctypes.data, n1, n2, sign) == 0
    ref = np.fft.fft2(x.astype(np.complex128)) if sign < 0 else np.fft.ifft2(x.astype(np.complex128)) * n1 * n2
    f1 = np.array([harness.h_pos_to_freq(n1, p) for p in range(n1)])
    f2 = np.array([harness.h_pos_to_freq(n2, p) for p in range(n2)])
    # a prime factor above 64 runs the O(R^2) generic butterfly: float32
    # rounding grows with the radix
    big = any(max(f for f in range(2, n + 1) if n % f == 0 and all(f % q for q in range(2, f))) > 64
              for n in (n1, n2) if n > 1)
    assert np.abs(d - ref[f1][:, f2]).max() <= (2e-6 if big else 5e-7) * np.abs(ref).max()
    harness.h_fft2(0, d.ctypes.data, n1, n2, -sign)
    assert np.abs(d / (n1 * n2) - x).max() <= 5e-6
    for p in range(n1):
        assert harness.h_freq_to_pos(n1, harness.h_pos_to_freq(n1, p)) == p


def test_good_size(harness):
    assert harness.h_good_size(104) == 105
    assert harness.h_good_size(192) == 192
    assert harness.h_good_size(11) == 12
