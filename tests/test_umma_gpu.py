"""The tcgen05 building blocks (isce2_gb300/csrc/umma.cuh) against numpy:
D = A B^T with bf16 operands, one pass and the 3-pass split."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out = str(tmp_path_factory.mktemp("umma") / "umma.so")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-shared",
                    "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "isce2_gb300", "csrc"),
                    os.path.join(HERE, "umma_harness.cu"), "-o", out], check=True)
    L = ctypes.CDLL(out)
    L.umma_gemm_test.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int] * 3
    return L


@pytest.mark.parametrize("N,K", [(16, 16), (32, 64), (128, 128), (256, 32), (144, 48)])
def test_umma_bf16_split(harness, N, K):
    rng = np.random.default_rng(N * 7 + K)
    A = rng.standard_normal((128, K)).astype(np.float32)
    B = rng.standard_normal((N, K)).astype(np.float32)
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    for split, tol in ((0, 2e-2), (1, 5e-5)):
        D = np.zeros((128, N), np.float32)
        rc = harness.umma_gemm_test(A.ctypes.data, B.ctypes.data, D.ctypes.data, N, K, split)
        assert rc == 0, rc
        err = np.abs(D - ref).max() / np.abs(ref).max()
        assert err < tol, (split, err)


@pytest.fixture(scope="module")
def corr_harness(harness):
    harness.umma_corr_test.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int] * 3
    return harness


@pytest.mark.parametrize("tH,tW", [(8, 16), (16, 40), (64, 96)])
def test_umma_lag_shifted_correlation(corr_harness, tH, tW):
    """The lag-shifted MN-major A operand: 16 x 16 lags of a 2-D correlation."""
    rng = np.random.default_rng(tH * 31 + tW)
    T = rng.standard_normal((tH, tW)).astype(np.float32)
    S = rng.standard_normal((tH + 16, tW + 16)).astype(np.float32)
    ref = np.zeros((16, 16))
    for u in range(16):
        for v in range(16):
            ref[u, v] = (T.astype(np.float64) * S[u:u + tH, v:v + tW]).sum()
    for split, tol in ((0, 2e-2), (1, 5e-5)):
        D = np.zeros((128, 32), np.float32)
        rc = corr_harness.umma_corr_test(T.ctypes.data, S.ctypes.data, D.ctypes.data, tH, tW, split)
        assert rc == 0, rc
        C = np.zeros((16, 16))
        for v in range(16):
            for p in range(8):
                C[:, v] += D[(15 - v) * 8 + p, p:p + 16]
        err = np.abs(C - ref).max() / np.abs(ref).max()
        assert err < tol, (split, err)


def test_mma_issue_rate(harness):
    """Cycles per tcgen05.mma (M = 128, K = 16) issued back to back by one
    thread, for N from 16 to 256 and both A layouts: printed (pytest -s) for
    the kernel notes; the test checks that the probe completes."""
    harness.umma_rate_test.argtypes = [ctypes.c_int] * 4 + [ctypes.c_void_p]
    n = 512
    for mode in (0, 1):
        for N in (16, 32, 64, 128, 256):
            cyc = np.zeros(2, np.int64)
            rc = harness.umma_rate_test(N, mode, n, 1, cyc.ctypes.data)
            assert rc == 0, rc
            assert cyc[1] >= cyc[0] > 0
            print(f"A {'MN-major' if mode else 'K-major'} N {N:3d}: {cyc[0] / n:.1f} cycles per MMA issued, "
                  f"{cyc[1] / n:.1f} to completion")


def test_mma_rate_with_every_sm_issuing(harness):
    """The correlation's MMA (M = 128, N = 32, K = 16, A MN-major) issued by
    one, two and three CTAs on every SM at once: nanoseconds per MMA per SM,
    printed (pytest -s) for the kernel notes; the test checks completion."""
    harness.umma_conc_test.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    n = 2048
    for per in (1, 2, 3):
        ms = ctypes.c_float(0.0)
        rc = harness.umma_conc_test(per, n, ctypes.byref(ms))
        assert rc == 0, rc
        assert ms.value > 0
        print(f"{per} CTA(s) per SM: {ms.value * 1e6 / (n * per):.1f} ns per MMA per SM")
