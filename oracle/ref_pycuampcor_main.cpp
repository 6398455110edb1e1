/*
 * ref_pycuampcor_main.cpp - command-line driver of the reference PyCuAmpcor
 * controller, used only to produce reference outputs for the parity
 * fixtures (test infrastructure, never shipped).
 *
 * It does what the reference's Python callers do through the pybind11 class
 * (contrib/PyCuAmpcor/src/PyCuAmpcor.cpp:31-101, examples/cuDenseOffsets.py):
 * set the properties, setupParams(), setConstantGrossOffset() or
 * setVaryingGrossOffset(), checkPixelInImageRange(), runAmpcor().  Arguments
 * are key=value pairs with the Python property names, plus
 *   outdir=DIR          working directory of the run (the reference writes its
 *                       outputs, and in its debug build every intermediate
 *                       array, into the current directory)
 *   grossDown=, grossAcross=   constant gross offset (default 0, 0)
 *   grossFile=FILE      varying gross offsets: int32 down[n] then across[n]
 *
 * Device allocations.  The reference's normaliser kernel lets every thread of
 * a power-of-two block read one search-chip row, so the threads past the row
 * width read into the next row and, for the last window of a batch, up to
 * (block - row width) floats past the end of the buffer
 * (cuCorrNormalization.cu:278,298-300).  Those values never reach a result,
 * but the read itself could leave the allocation.  The link step wraps
 * cudaMalloc (-Wl,--wrap=cudaMalloc) so every device buffer the reference
 * allocates carries kPadBytes of zeroed slack; the read stays inside it.
 */
#include <cuda_runtime.h>
#include <unistd.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <string>
#include <vector>

#include "cuAmpcorController.h"
#include "cuAmpcorParameter.h"
#include "cuArrays.h"
#include "cudaUtil.h"

/* gpuDeviceInit (declared in cudaUtil.h) selects the device the controller
 * runs on (cuAmpcorController.cpp:40).  The reference's cudaUtil.cpp, which
 * defines it, does not compile with CUDA 13 (its gpuDeviceList reads the
 * removed cudaDeviceProp::computeMode), so this driver defines it: check the
 * id and make that device current. */
int gpuDeviceInit(int devID)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || devID < 0 || devID >= n) {
        std::fprintf(stderr, "gpuDeviceInit: device %d not available\n", devID);
        std::exit(EXIT_FAILURE);
    }
    if (cudaSetDevice(devID) != cudaSuccess) std::exit(EXIT_FAILURE);
    return devID;
}

static const size_t kPadBytes = 64 << 10;  // > 1024 floats, the widest normaliser block

static int g_padded_allocs = 0;

extern "C" cudaError_t __real_cudaMalloc(void** p, size_t n);
extern "C" cudaError_t __wrap_cudaMalloc(void** p, size_t n)
{
    ++g_padded_allocs;
    cudaError_t e = __real_cudaMalloc(p, n + kPadBytes);
    if (e == cudaSuccess) e = cudaMemset(*p, 0, n + kPadBytes);
    return e;
}

int main(int argc, char** argv)
{
    std::map<std::string, std::string> kv;
    for (int i = 1; i < argc; ++i) {
        const char* eq = std::strchr(argv[i], '=');
        if (!eq) {
            std::fprintf(stderr, "argument without '=': %s\n", argv[i]);
            return 2;
        }
        kv[std::string(argv[i], eq - argv[i])] = std::string(eq + 1);
    }
    auto has = [&](const char* k) { return kv.count(k) != 0; };
    auto geti = [&](const char* k, int dflt) { return has(k) ? std::atoi(kv[k].c_str()) : dflt; };

    cuAmpcorController ctl;
    cuAmpcorParameter* p = ctl.param;
    // property name -> field, as PyCuAmpcor.cpp:31-76 binds them
    p->algorithm = geti("algorithm", p->algorithm);
    p->deviceID = geti("deviceID", p->deviceID);
    p->nStreams = geti("nStreams", p->nStreams);
    p->derampMethod = geti("derampMethod", p->derampMethod);
    p->referenceImageHeight = geti("referenceImageHeight", p->referenceImageHeight);
    p->referenceImageWidth = geti("referenceImageWidth", p->referenceImageWidth);
    p->secondaryImageHeight = geti("secondaryImageHeight", p->secondaryImageHeight);
    p->secondaryImageWidth = geti("secondaryImageWidth", p->secondaryImageWidth);
    p->numberWindowDown = geti("numberWindowDown", p->numberWindowDown);
    p->numberWindowAcross = geti("numberWindowAcross", p->numberWindowAcross);
    p->windowSizeHeightRaw = geti("windowSizeHeight", p->windowSizeHeightRaw);
    p->windowSizeWidthRaw = geti("windowSizeWidth", p->windowSizeWidthRaw);
    p->mergeGrossOffset = geti("mergeGrossOffset", p->mergeGrossOffset);
    p->rawDataOversamplingFactor = geti("rawDataOversamplingFactor", p->rawDataOversamplingFactor);
    p->corrStatWindowSize = geti("corrStatWindowSize", p->corrStatWindowSize);
    p->numberWindowDownInChunk = geti("numberWindowDownInChunk", p->numberWindowDownInChunk);
    p->numberWindowAcrossInChunk = geti("numberWindowAcrossInChunk", p->numberWindowAcrossInChunk);
    p->useMmap = geti("useMmap", p->useMmap);
    p->halfSearchRangeAcrossRaw = geti("halfSearchRangeAcross", p->halfSearchRangeAcrossRaw);
    p->halfSearchRangeDownRaw = geti("halfSearchRangeDown", p->halfSearchRangeDownRaw);
    p->referenceStartPixelAcross0 = geti("referenceStartPixelAcrossStatic", p->referenceStartPixelAcross0);
    p->referenceStartPixelDown0 = geti("referenceStartPixelDownStatic", p->referenceStartPixelDown0);
    p->oversamplingMethod = geti("corrSurfaceOverSamplingMethod", p->oversamplingMethod);
    p->oversamplingFactor = geti("corrSurfaceOverSamplingFactor", p->oversamplingFactor);
    p->mmapSizeInGB = geti("mmapSize", p->mmapSizeInGB);
    p->skipSampleDownRaw = geti("skipSampleDown", p->skipSampleDownRaw);
    p->skipSampleAcrossRaw = geti("skipSampleAcross", p->skipSampleAcrossRaw);
    p->zoomWindowSize = geti("corrSurfaceZoomInWindow", p->zoomWindowSize);
    if (has("referenceImageName")) p->referenceImageName = kv["referenceImageName"];
    if (has("secondaryImageName")) p->secondaryImageName = kv["secondaryImageName"];
    p->offsetImageName = has("offsetImageName") ? kv["offsetImageName"] : "offset.bip";
    p->grossOffsetImageName = has("grossOffsetImageName") ? kv["grossOffsetImageName"] : "gross.bip";
    p->snrImageName = has("snrImageName") ? kv["snrImageName"] : "snr.bip";
    p->covImageName = has("covImageName") ? kv["covImageName"] : "cov.bip";

    p->setupParameters();  // setupParams()
    if (has("grossFile")) {  // setVaryingGrossOffset(vD, vA)
        const int n = p->numberWindows;
        std::vector<int> buf(2 * (size_t)n);
        std::ifstream in(kv["grossFile"], std::ios::binary);
        if (!in.read(reinterpret_cast<char*>(buf.data()), (std::streamsize)(buf.size() * sizeof(int)))) {
            std::fprintf(stderr, "cannot read %s\n", kv["grossFile"].c_str());
            return 2;
        }
        p->setStartPixels(p->referenceStartPixelDown0, p->referenceStartPixelAcross0, buf.data(), buf.data() + n);
    } else {  // setConstantGrossOffset(goDown, goAcross)
        p->setStartPixels(p->referenceStartPixelDown0, p->referenceStartPixelAcross0, geti("grossDown", 0),
                          geti("grossAcross", 0));
    }
    p->checkPixelInImageRange();
    {   // refuse to run the reference kernels unless its allocations are padded
        cuArrays<float> probe(1, 1);
        probe.allocate();
        if (g_padded_allocs == 0) {
            std::fprintf(stderr, "cudaMalloc is not wrapped: not running the reference kernels\n");
            return 3;
        }
    }
    if (has("outdir") && chdir(kv["outdir"].c_str()) != 0) {
        std::fprintf(stderr, "cannot enter %s\n", kv["outdir"].c_str());
        return 2;
    }
    ctl.runAmpcor();
    std::printf("ref_pycuampcor: %d windows done\n", p->numberWindows);
    return 0;
}
