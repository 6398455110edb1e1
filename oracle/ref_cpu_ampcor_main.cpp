/*
 * ref_cpu_ampcor_main.cpp - runs the reference's C++ CPU ampcor
 * (components/zerodop/GPUampcor/src/Ampcor.cpp, AmpcorMethods.cpp: the C++
 * port of mroipac ampcor.F) on a window grid, one thread per band of window
 * rows, the way DenseAmpcor splits a scene into row bands across processes
 * (components/mroipac/ampcor/DenseAmpcor.py:402-436).  Test infrastructure:
 * it is the timed reference CPU baseline, never part of the product.
 *
 * Arguments (key=value):
 *   ref=, sec=        raw row-major complex64 images, shape in "<name>.shape"
 *   windowSizeHeight, windowSizeWidth, halfSearchRangeDown,
 *   halfSearchRangeAcross, skipSampleDown, skipSampleAcross,
 *   referenceStartPixelDownStatic, referenceStartPixelAcrossStatic,
 *   numberWindowDown, numberWindowAcross      the PyCuAmpcor window grid
 *   corrSurfaceOverSamplingFactor (default 16), corrSurfaceZoomInWindow (16)
 *   threads=N         row bands run concurrently (default: all host cores)
 *   out=FILE          per accepted window: int32 centre down, centre across,
 *                     then float32 offset down, offset across, snr, cov1-3
 *   summary=FILE      one JSON line: windows, accepted, seconds, threads
 *
 * Window (k, l) has its reference chip at (startD + k*skipD, startA +
 * l*skipA) and its search chip hs pixels above and left of it, as in
 * PyCuAmpcor.  Ampcor.cpp addresses lines as y + yy - 2 (0-based,
 * Ampcor.cpp:574) and columns as x + xx - 1 (:604), so the band of rows
 * [k0, k1) is run with firstRow = startD + k0*skipD + 2 - hsD and lastRow =
 * firstRow + (k1 - k0 - 1)*skipD + 1; that lastRow keeps the row loop
 * (:557) to exactly k1 - k0 iterations, the count the output arrays are
 * sized for (:145-147).  Skips must be at least 2 for the same reason.
 */
#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "Ampcor.h"
#include "DataAccessor.h"

struct Image {
    int h = 0, w = 0, px = 0;
    std::vector<char> bytes;
};

static bool load(const std::string& fn, Image& im)
{
    std::ifstream shp(fn + ".shape");
    if (!(shp >> im.h >> im.w >> im.px) || im.px != 8) return false;
    im.bytes.resize((size_t)im.h * im.w * im.px);
    std::ifstream in(fn, std::ios::binary);
    return (bool)in.read(im.bytes.data(), (std::streamsize)im.bytes.size());
}

struct Row {
    int32_t cd, ca;
    float od, oa, snr, c1, c2, c3;
};

int main(int argc, char** argv)
{
    std::map<std::string, std::string> kv;
    for (int i = 1; i < argc; ++i) {
        const char* eq = std::strchr(argv[i], '=');
        if (eq) kv[std::string(argv[i], eq - argv[i])] = eq + 1;
    }
    auto geti = [&](const char* k, int d) { return kv.count(k) ? std::atoi(kv[k].c_str()) : d; };
    Image ref, sec;
    if (!load(kv["ref"], ref) || !load(kv["sec"], sec)) {
        std::fprintf(stderr, "cannot load the images\n");
        return 2;
    }
    const int Wh = geti("windowSizeHeight", 64), Ww = geti("windowSizeWidth", 64);
    const int hsD = geti("halfSearchRangeDown", 20), hsA = geti("halfSearchRangeAcross", 20);
    const int skD = geti("skipSampleDown", 64), skA = geti("skipSampleAcross", 64);
    const int sD = geti("referenceStartPixelDownStatic", hsD), sA = geti("referenceStartPixelAcrossStatic", hsA);
    const int nD = geti("numberWindowDown", 1), nA = geti("numberWindowAcross", 1);
    const int ovs = geti("corrSurfaceOverSamplingFactor", 16), zoom = geti("corrSurfaceZoomInWindow", 16);
    int nth = geti("threads", (int)std::thread::hardware_concurrency());
    if (skD < 2 || skA < 2 || nD < 1 || nA < 1 || sA < hsA || nth < 1) {
        std::fprintf(stderr, "unsupported grid\n");
        return 2;
    }
    nth = std::min(nth, nD);
    DataAccessor acc1(ref.bytes.data(), ref.w, ref.h, 8), acc2(sec.bytes.data(), sec.w, sec.h, 8);
    DataAccessor sink(nullptr, 8, 0, 4);

    std::vector<std::vector<Row> > out(nth);
    auto band = [&](int t) {
        const int k0 = (int)((int64_t)nD * t / nth), k1 = (int)((int64_t)nD * (t + 1) / nth);
        if (k1 <= k0) return;
        Ampcor a;
        a.imgAccessor1 = (uint64_t)(uintptr_t)&acc1;
        a.imgAccessor2 = (uint64_t)(uintptr_t)&acc2;
        a.offImgAccessor = (uint64_t)(uintptr_t)&sink;
        a.offQualImgAccessor = (uint64_t)(uintptr_t)&sink;
        a.imgDatatypes[0] = a.imgDatatypes[1] = DTYPE_COMPLEX;
        a.isMag[0] = a.isMag[1] = 0;
        a.imgWidths[0] = ref.w;
        a.imgWidths[1] = sec.w;
        a.imgBands[0] = a.imgBands[1] = 0;
        a.refChipWidth = Ww;
        a.refChipHeight = Wh;
        a.schMarginX = hsA;
        a.schMarginY = hsD;
        a.rowSkip = skD;
        a.colSkip = skA;
        a.firstRow = sD + k0 * skD + 2 - hsD;
        a.lastRow = a.firstRow + (k1 - k0 - 1) * skD + 1;
        a.firstCol = sA + 1 - hsA;
        a.lastCol = a.firstCol + (nA - 1) * skA + 1;
        a.nLookAcross = a.nLookDown = 1;
        a.osampFact = ovs;
        a.zoomWinSize = zoom;
        a.acrossGrossOff = a.downGrossOff = 0;
        a.snrThresh = 0.f;
        a.covThresh = 1000.f;
        a.xScaleFactor = a.yScaleFactor = 1.f;
        a.corr_debug = a.corr_display = false;
        a.usr_enable_gpu = false;
        a.ampcor();
        for (int i = 0; i < a.numRowTable; ++i)
            out[t].push_back(Row{a.getLocationDownAt(i), a.getLocationAcrossAt(i), a.getLocationDownOffsetAt(i),
                                 a.getLocationAcrossOffsetAt(i), a.getSnrAt(i), a.getCov1At(i), a.getCov2At(i),
                                 a.getCov3At(i)});
    };
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<std::thread> pool;
    for (int t = 0; t < nth; ++t) pool.emplace_back(band, t);
    for (auto& th : pool) th.join();
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();

    size_t accepted = 0;
    if (kv.count("out")) {
        std::ofstream f(kv["out"], std::ios::binary);
        for (auto& v : out) {
            f.write(reinterpret_cast<const char*>(v.data()), (std::streamsize)(v.size() * sizeof(Row)));
            accepted += v.size();
        }
    } else {
        for (auto& v : out) accepted += v.size();
    }
    char line[256];
    std::snprintf(line, sizeof line, "{\"windows\": %d, \"accepted\": %zu, \"seconds\": %.6f, \"threads\": %d}\n",
                  nD * nA, accepted, secs, nth);
    if (kv.count("summary")) {
        std::ofstream s(kv["summary"]);
        s << line;
    }
    std::fputs(line, stderr);
    return 0;
}
