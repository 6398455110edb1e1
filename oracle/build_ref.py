"""Build the reference's own code as parity checker and timed CPU baseline.

TEST INFRASTRUCTURE.  Nothing in the product package imports this module or
runs what it builds; only the tests' fixture generator, ``bench.py``'s
reference leg and the CPU baseline do.

Two builds, both into the git-ignored ``oracle/_ref/``:

* ``pycuampcor_ref`` - ISCE2's PyCuAmpcor (contrib/PyCuAmpcor/src, every
  ``.cu``/``.cpp`` except the GDAL reader and the pybind11 module) compiled
  for sm_103a with cuFFT, driven by ``ref_pycuampcor_main.cpp``.  GDAL is
  replaced by ``ref_shim/GDALImage.h`` (raw files, same interface).  It is
  built without ``NDEBUG``, so the reference's own debug mode
  (contrib/PyCuAmpcor/src/debug.h:15-17) dumps its intermediate arrays
  (raw peak, clamped zoom start, zoom peak) next to its outputs.  cudaMalloc
  is wrapped at link time to pad every device buffer (see the driver's
  header for the over-read it contains).
* ``ampcor_cpu_ref`` - the reference's C++ CPU port of ampcor.F
  (components/zerodop/GPUampcor/src/Ampcor.cpp, AmpcorMethods.cpp) with an
  in-memory ``DataAccessor`` and a radix-2 FFT in place of its FFTW wrapper
  (``ref_shim/``), run in row bands by ``ref_cpu_ampcor_main.cpp``.

Sources: when the ISCE2 tree is present at ``ISCE2_SRC`` (default
/root/reference), the needed files are staged into ``oracle/_ref/src`` (never
committed); the build then compiles from that staged copy, so a machine
without the tree (the GPU machine) builds from what was staged here.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
STAGE = os.path.join(OUT, "src")
SHIM = os.path.join(HERE, "ref_shim")
ISCE2_SRC = os.environ.get("ISCE2_SRC", "/root/reference")

PYCU_DIR = "contrib/PyCuAmpcor/src"
# cudaUtil.cpp is left out as well: its gpuDeviceList() reads
# cudaDeviceProp::computeMode, which CUDA 13 removed; the driver supplies the
# one function of that file the run path calls, gpuDeviceInit.
PYCU_SKIP = {"GDALImage.cpp", "GDALImage.h", "PyCuAmpcor.cpp", "cudaUtil.cpp"}
CPU_FILES = {"components/zerodop/GPUampcor/src": ["Ampcor.cpp", "AmpcorMethods.cpp"],
             "components/zerodop/GPUampcor/include": ["Ampcor.h", "AmpcorMethods.h", "Constants.h"]}

GPU_BIN = os.path.join(OUT, "pycuampcor_ref")
GPU_BIN_RELEASE = os.path.join(OUT, "pycuampcor_ref_release")
CPU_BIN = os.path.join(OUT, "ampcor_cpu_ref")


def stage() -> bool:
    """Copy the reference files the builds need into oracle/_ref/src."""
    if not os.path.isdir(os.path.join(ISCE2_SRC, PYCU_DIR)):
        return False
    pdst = os.path.join(STAGE, "pycuampcor")
    cdst = os.path.join(STAGE, "cpu")
    os.makedirs(pdst, exist_ok=True)
    os.makedirs(cdst, exist_ok=True)
    src = os.path.join(ISCE2_SRC, PYCU_DIR)
    for f in sorted(os.listdir(src)):
        if f.endswith((".cu", ".cpp", ".h")) and f not in PYCU_SKIP:
            shutil.copyfile(os.path.join(src, f), os.path.join(pdst, f))
        elif f in PYCU_SKIP and os.path.exists(os.path.join(pdst, f)):
            os.remove(os.path.join(pdst, f))
    for d, files in CPU_FILES.items():
        for f in files:
            shutil.copyfile(os.path.join(ISCE2_SRC, d, f), os.path.join(cdst, f))
    return True


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_cpu(force: bool = False) -> str | None:
    """g++ build of the reference CPU port; None when its sources are not staged."""
    cdir = os.path.join(STAGE, "cpu")
    srcs = [os.path.join(cdir, "Ampcor.cpp"), os.path.join(cdir, "AmpcorMethods.cpp"),
            os.path.join(SHIM, "ampcor_fft_shim.cpp"), os.path.join(HERE, "ref_cpu_ampcor_main.cpp")]
    if not all(os.path.exists(s) for s in srcs):
        return None
    deps = srcs + [os.path.join(SHIM, f) for f in os.listdir(SHIM)]
    if force or _newer(CPU_BIN, deps):
        cxx = shutil.which("g++") or "g++"
        _run([cxx, "-O3", "-std=c++17", "-fcx-limited-range", "-pthread", "-w", "-I", SHIM, "-I", cdir,
              *srcs, "-o", CPU_BIN + ".tmp"])
        os.replace(CPU_BIN + ".tmp", CPU_BIN)
    return CPU_BIN


def build_gpu(force: bool = False, release: bool = False) -> str | None:
    """nvcc build of the reference PyCuAmpcor driver; None when not staged.

    The default build leaves NDEBUG undefined, so the reference's debug mode
    dumps every intermediate array (the parity fixtures read them); the
    release build defines NDEBUG, as the reference's own builds do, and is
    the one to time."""
    pdir = os.path.join(STAGE, "pycuampcor")
    if not os.path.isdir(pdir):
        return None
    srcs = [os.path.join(pdir, f) for f in sorted(os.listdir(pdir)) if f.endswith((".cu", ".cpp"))]
    srcs += [os.path.join(SHIM, "GDALImage_raw.cpp"), os.path.join(HERE, "ref_pycuampcor_main.cpp")]
    deps = srcs + [os.path.join(pdir, f) for f in os.listdir(pdir)] + [os.path.join(SHIM, "GDALImage.h")]
    binary = GPU_BIN_RELEASE if release else GPU_BIN
    if not (force or _newer(binary, deps)):
        return binary
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    objdir = os.path.join(OUT, "obj_pycuampcor_release" if release else "obj_pycuampcor")
    os.makedirs(objdir, exist_ok=True)
    # the reference Makefile's flags (contrib/PyCuAmpcor/src/Makefile:9-18) with
    # the architecture set to sm_103a; NDEBUG left undefined: debug dumps on
    flags = ["-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", "-ftz=false",
             "-prec-div=true", "-prec-sqrt=true", "-w", "-I", SHIM, "-I", pdir] + (["-DNDEBUG"] if release else [])

    def one(s):
        o = os.path.join(objdir, os.path.basename(s) + ".o")
        _run([nvcc, *flags, "-c", s, "-o", o])
        return o

    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(one, srcs))
    _run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", *objs, "-o", binary + ".tmp",
          "-Xlinker", "--wrap=cudaMalloc", "-lcufft"])
    os.replace(binary + ".tmp", binary)
    return binary


def build(gpu: bool = False, force: bool = False) -> dict:
    """Stage (where the ISCE2 tree exists) and build; returns what was built."""
    os.makedirs(OUT, exist_ok=True)
    stage()
    out = {"cpu": build_cpu(force)}
    if gpu:
        out["gpu"] = build_gpu(force)
    return out


if __name__ == "__main__":
    print(build(gpu="--gpu" in sys.argv, force="--force" in sys.argv))
