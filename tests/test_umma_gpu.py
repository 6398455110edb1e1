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
