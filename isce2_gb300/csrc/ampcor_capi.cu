// Host orchestration and the C ABI (include/ampcor_gb.h).
//
// Geometry follows cuAmpcorParameter (contrib/PyCuAmpcor/src/cuAmpcorParameter.cpp);
// the run replaces cuAmpcorController::runAmpcor + cuAmpcorChunk::run with
// four batched launches per window batch on one stream.  Nothing here
// computes results on the CPU: without a working device every run call
// returns AMPCOR_ERR_CUDA.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ampcor_gb.h"
#include "ampcor_kernels.h"
#include "umma.cuh"
#include "ampcor_internal.h"
#include "ampcor_plan.h"
#include "umma.cuh"

using namespace ampcor;

static int fail(ampcor_handle* h, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (h) h->err = buf;
    return code;
}

#define CUDA_TRY(h, call)                                                                         \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return fail(h, AMPCOR_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));      \
    } while (0)

extern "C" {

const char* ampcor_version(void) { return "ampcor-gb300 0.1 (sm_103a)"; }

void ampcor_params_default(ampcor_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->algorithm = 0;
    p->deviceID = 0;
    p->nStreams = 1;
    p->derampMethod = 1;
    p->windowSizeWidth = 64;
    p->windowSizeHeight = 64;
    p->halfSearchRangeDown = 20;
    p->halfSearchRangeAcross = 20;
    p->skipSampleAcross = 64;
    p->skipSampleDown = 64;
    p->rawDataOversamplingFactor = 2;
    p->corrSurfaceZoomInWindow = 16;
    p->corrSurfaceOverSamplingFactor = 16;
    p->corrSurfaceOverSamplingMethod = 0;
    p->referenceImageWidth = 1000;
    p->referenceImageHeight = 1000;
    p->secondaryImageWidth = 1000;
    p->secondaryImageHeight = 1000;
    p->numberWindowDown = 1;
    p->numberWindowAcross = 1;
    p->numberWindowDownInChunk = 1;
    p->numberWindowAcrossInChunk = 1;
    p->referenceStartPixelDownStatic = 0;
    p->referenceStartPixelAcrossStatic = 0;
    p->corrStatWindowSize = 21;
    p->useMmap = 1;
    p->mmapSize = 1;
    p->mergeGrossOffset = 0;
}

int ampcor_create(ampcor_handle** out) {
    if (!out) return AMPCOR_ERR_ARG;
    ampcor_handle* h = new (std::nothrow) ampcor_handle();
    if (!h) return AMPCOR_ERR_ALLOC;
    ampcor_params_default(&h->p);
    *out = h;
    return AMPCOR_OK;
}

static void release_device(ampcor_handle* h) {
    if (h->dev < 0) return;
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(h->dev);
    for (cudaEvent_t e : h->ev_start) cudaEventDestroy(e);
    for (cudaEvent_t e : h->ev_end) cudaEventDestroy(e);
    h->ev_start.clear();
    h->ev_end.clear();
    h->ev_stage.clear();
    h->ev_used = 0;
    cudaFree(h->d_coords);
    cudaFree(h->d_res);
    cudaFree(h->d_ws);
    cudaFree(h->d_ref);
    cudaFree(h->d_sec);
    cudaFree(h->d_out);
    cudaFree(h->d_diag);
    cudaFree(h->d_errw);
    h->d_errw = nullptr;
    cudaFree(h->d_tc);
    h->d_tc = nullptr;
    h->d_coords = nullptr; h->d_res = nullptr; h->d_ws = nullptr; h->d_ref = nullptr;
    h->d_sec = nullptr; h->d_out = nullptr; h->d_diag = nullptr;
    h->coords_cap = h->res_cap = h->ws_cap = h->ref_cap = h->sec_cap = h->out_cap = h->diag_cap = 0;
    cudaSetDevice(cur);
    h->dev = -1;
}

int ampcor_destroy(ampcor_handle* h) {
    if (!h) return AMPCOR_ERR_ARG;
    release_device(h);
    delete h;
    return AMPCOR_OK;
}

int ampcor_set_params(ampcor_handle* h, const ampcor_params* p) {
    if (!h || !p) return AMPCOR_ERR_ARG;
    h->p = *p;
    h->is_setup = false;
    h->has_starts = false;
    return AMPCOR_OK;
}

int ampcor_get_params(const ampcor_handle* h, ampcor_params* p) {
    if (!h || !p) return AMPCOR_ERR_ARG;
    *p = h->p;
    return AMPCOR_OK;
}

int ampcor_setup(ampcor_handle* h) {
    if (!h) return AMPCOR_ERR_ARG;
    h->err.clear();
    const ampcor_params& p = h->p;
    if (p.numberWindowDown <= 0 || p.numberWindowAcross <= 0)
        return fail(h, AMPCOR_ERR_ARG, "Incorrect number of windows! (%d, %d)", p.numberWindowDown, p.numberWindowAcross);
    if ((long long)p.numberWindowDown * p.numberWindowAcross > (1LL << 30))
        return fail(h, AMPCOR_ERR_ARG, "too many windows");
    if (p.windowSizeHeight <= 0 || p.windowSizeWidth <= 0)
        return fail(h, AMPCOR_ERR_ARG, "window size must be positive (%d, %d)", p.windowSizeHeight, p.windowSizeWidth);
    if (p.halfSearchRangeDown < 1 || p.halfSearchRangeAcross < 1)
        return fail(h, AMPCOR_ERR_ARG, "half search ranges must be >= 1");
    if (p.rawDataOversamplingFactor < 1 || p.rawDataOversamplingFactor > 8)
        return fail(h, AMPCOR_ERR_ARG, "rawDataOversamplingFactor must be in [1, 8]");
    if (p.corrSurfaceOverSamplingFactor < 1)
        return fail(h, AMPCOR_ERR_ARG, "corrSurfaceOverSamplingFactor must be >= 1");
    if (p.corrStatWindowSize < 1) return fail(h, AMPCOR_ERR_ARG, "corrStatWindowSize must be >= 1");
    if (p.corrSurfaceOverSamplingMethod != 0 && p.corrSurfaceOverSamplingMethod != 1)
        return fail(h, AMPCOR_ERR_ARG, "corrSurfaceOverSamplingMethod must be 0 (FFT) or 1 (sinc), got %d",
                    p.corrSurfaceOverSamplingMethod);

    WindowPlan& P = h->plan;
    P = WindowPlan{};
    const int raw = p.rawDataOversamplingFactor;
    P.Wh = p.windowSizeHeight;
    P.Ww = p.windowSizeWidth;
    P.hsD = p.halfSearchRangeDown;
    P.hsA = p.halfSearchRangeAcross;
    // cuAmpcorParameter.cpp:73-97, including the swapped half ranges
    P.Hs = P.Wh + 2 * P.hsA;
    P.Ws = P.Ww + 2 * P.hsD;
    P.NX = P.Hs - P.Wh + 1;
    P.NY = P.Ws - P.Ww + 1;
    P.statH = std::min(p.corrStatWindowSize, 2 * P.hsD + 1);
    P.statW = std::min(p.corrStatWindowSize, 2 * P.hsA + 1);
    P.raw = raw;
    P.deramp = p.derampMethod;
    P.zoom = std::min(p.corrSurfaceZoomInWindow, std::min(P.hsA, P.hsD) * 2 * raw);
    P.hz = P.zoom / (2 * raw);
    if (P.zoom < 2 || P.hz < 1)
        return fail(h, AMPCOR_ERR_UNSUPPORTED, "zoom window %d too small for raw factor %d", P.zoom, raw);
    P.Hz = P.Wh + 2 * P.hz;
    P.Wz = P.Ww + 2 * P.hz;
    P.osWh = raw * P.Wh;
    P.osWw = raw * P.Ww;
    P.osHz = raw * P.Hz;
    P.osWz = raw * P.Wz;
    P.zp = 2 * P.hz * raw;
    P.ovs = p.corrSurfaceOverSamplingFactor;
    P.M = P.zoom * P.ovs;
    // coarse step of the zoom scan: about ovs/4, at most 128 coarse samples per axis
    {
        int want = std::max(std::max(1, P.ovs / 4), (P.M + 127) / 128);
        int zs = 1;
        for (int d = 1; d <= P.M; ++d)
            if (P.M % d == 0 && d <= want) zs = d;
        if (P.M / zs > 128)
            for (int d = zs; d <= P.M; ++d)
                if (P.M % d == 0 && P.M / d <= 128) { zs = d; break; }
        P.zs = zs;
    }
    P.method = p.corrSurfaceOverSamplingMethod;
    P.osratio = 1.0f / (float)(P.ovs * raw);
    P.P = fft_good_size(P.Hs);
    P.Q = fft_good_size(P.Ws);
    if (!fft_plan_make(P.P, &P.fP) || !fft_plan_make(P.Q, &P.fQ))
        return fail(h, AMPCOR_ERR_UNSUPPORTED, "no FFT plan for %d x %d", P.P, P.Q);
    if (!fft_plan_make(P.Wh, &P.fRefH) || !fft_plan_make(P.Ww, &P.fRefW) || !fft_plan_make(P.Hz, &P.fSchH) ||
        !fft_plan_make(P.Wz, &P.fSchW))
        return fail(h, AMPCOR_ERR_UNSUPPORTED,
                    "window sizes (%d, %d) / zoom-in chip (%d, %d) have a prime factor above %d", P.Wh, P.Ww, P.Hz,
                    P.Wz, kMaxGenericRadix);
    if ((long long)P.M * P.M >= (1LL << 31)) return fail(h, AMPCOR_ERR_UNSUPPORTED, "zoomed surface too large");
    // The sinc interpolator reads the zp x zp surface with indices wrapped once
    // (cuSincOverSampler.cu:131-146); they stay inside it only when the zoom
    // window equals the kept surface and spans at least the 8-tap kernel, and
    // its (4 ovs + 1)^2 output points are distinct only when zoom > 4.
    if (P.method == 1 && (P.zoom != P.zp || P.zp < kSincLen))
        return fail(h, AMPCOR_ERR_UNSUPPORTED,
                    "sinc surface oversampling needs a zoom window (%d) that is a multiple of 2*raw and at least %d",
                    P.zoom, kSincLen);
    // kept oversampled surfaces outside the register-blocked kernels' sides
    // run the direct-sum correlation (plain runs only; the batched paths
    // reject such jobs)
    if (P.zp > kMaxDirectZp)
        return fail(h, AMPCOR_ERR_UNSUPPORTED, "oversampled search range 2*hz*raw = %d above %d", P.zp,
                    kMaxDirectZp);
    {
        const bool fits = raw_smem_bytes(P) <= kSmemLimit;
        if (h->raw_mode == 1 && !fits)
            return fail(h, AMPCOR_ERR_UNSUPPORTED, "raw correlation tile %d x %d does not fit in shared memory",
                        P.P, P.Q);
        P.rawL2 = (h->raw_mode >= 2 || (h->raw_mode == 0 && !fits)) ? 1 : 0;
        if (P.rawL2) {
            P.rawGl = h->raw_mode == 3 ? 16 : 32;
            while (P.rawGl > 2 && raw_l2_smem_bytes(P) > kSmemLimit) P.rawGl -= 2;
            P.rawNt = h->raw_mode == 3 ? 256 : 0;
        }
    }
    if (os2_applies(P) && os2_smem_bytes(P) > kSmemLimit) {
        P.osL2 = 1;
        P.osGl = 32;
        while (P.osGl > 2 && os2_l2_smem_bytes(P) > kSmemLimit) P.osGl -= 2;
    }
    if (h->precision) {
        if (!os_tc_applies(P))
            return fail(h, AMPCOR_ERR_UNSUPPORTED,
                        "tensor-core oversampling needs raw = 2, even chip sides and sides up to %d (chips %d x %d, "
                        "%d x %d)", kOsTcMaxSide, P.Wh, P.Ww, P.Hz, P.Wz);
        P.osTc = h->precision;
    }
    if (h->corr_precision) {
        const int bg = cos_tc_band_groups(P);
        if (!bg)
            return fail(h, AMPCOR_ERR_UNSUPPORTED,
                        "tensor-core oversampled correlation needs a kept surface of at most %d x %d lags (%d), "
                        "oversampled chip rows of whole 16-byte units and bands that fit shared memory "
                        "(oversampled search chip %d x %d)",
                        kCosTcMaxZp, kCosTcMaxZp, P.zp, P.osHz, P.osWz);
        P.cosTc = h->corr_precision;
        P.cosTcBg = bg;
    }
    // large zoom windows: a coarser first grid of the pruned zoom scan (the
    // scan stays exact, only more cells are refined) until the stage fits
    while (P.method == 0 && zoom_smem_bytes(P) > kSmemLimit) {
        int next = 0;
        for (int d = P.zs + 1; d <= P.M / 4; ++d)
            if (P.M % d == 0) { next = d; break; }
        if (!next) break;
        P.zs = next;
    }
    const size_t sm[4] = {P.rawL2 ? raw_l2_smem_bytes(P) : raw_smem_bytes(P),
                          P.osL2 ? os2_l2_smem_bytes(P) : os2_applies(P) ? os2_smem_bytes(P) : os_smem_bytes(P),
                          corr_os_supported(P.zp) ? corr_os_smem_bytes(P) : 0, zoom_smem_bytes(P)};
    const char* nm[4] = {"raw correlation", "oversampler", "oversampled correlation", "surface zoom"};
    for (int i = 0; i < 4; ++i)
        if (sm[i] > kSmemLimit)
            return fail(h, AMPCOR_ERR_UNSUPPORTED, "%s stage needs %zu bytes of shared memory (limit %zu)", nm[i],
                        sm[i], kSmemLimit);

    ampcor_geometry& g = h->geo;
    g.numberWindows = p.numberWindowDown * p.numberWindowAcross;
    g.searchWindowSizeHeightRaw = P.Hs;
    g.searchWindowSizeWidthRaw = P.Ws;
    g.zoomWindowSize = P.zoom;
    g.halfZoomWindowSizeRaw = P.hz;
    g.corrRawZoomInHeight = P.statH;
    g.corrRawZoomInWidth = P.statW;
    g.fftHeight = P.P;
    g.fftWidth = P.Q;
    const size_t n = (size_t)g.numberWindows;
    h->refD.assign(n, 0);
    h->refA.assign(n, 0);
    h->grossD.assign(n, 0);
    h->grossA.assign(n, 0);
    h->coords.assign(n, WindowCoords{});
    h->is_setup = true;
    h->has_starts = false;
    h->coords_dirty = true;
    return AMPCOR_OK;
}

int ampcor_get_geometry(const ampcor_handle* h, ampcor_geometry* g) {
    if (!h || !g) return AMPCOR_ERR_ARG;
    if (!h->is_setup) return AMPCOR_ERR_STATE;
    *g = h->geo;
    return AMPCOR_OK;
}

static void fill_coords(ampcor_handle* h) {
    const size_t n = h->refD.size();
    for (size_t i = 0; i < n; ++i) {
        WindowCoords& c = h->coords[i];
        c.refD = h->refD[i];
        c.refA = h->refA[i];
        // cuAmpcorParameter.cpp:161,164
        c.secD = h->refD[i] + h->grossD[i] - h->p.halfSearchRangeDown;
        c.secA = h->refA[i] + h->grossA[i] - h->p.halfSearchRangeAcross;
    }
    h->has_starts = true;
    h->coords_dirty = true;
}

int ampcor_set_constant_gross_offset(ampcor_handle* h, int32_t goDown, int32_t goAcross) {
    if (!h) return AMPCOR_ERR_ARG;
    if (!h->is_setup) return fail(h, AMPCOR_ERR_STATE, "setupParams must be called first");
    const ampcor_params& p = h->p;
    for (int row = 0; row < p.numberWindowDown; ++row)
        for (int col = 0; col < p.numberWindowAcross; ++col) {
            const size_t i = (size_t)row * p.numberWindowAcross + col;
            h->refD[i] = p.referenceStartPixelDownStatic + row * p.skipSampleDown;
            h->refA[i] = p.referenceStartPixelAcrossStatic + col * p.skipSampleAcross;
            h->grossD[i] = goDown;
            h->grossA[i] = goAcross;
        }
    fill_coords(h);
    return AMPCOR_OK;
}

int ampcor_set_varying_gross_offset(ampcor_handle* h, const int32_t* vD, const int32_t* vA, int64_t n) {
    if (!h || !vD || !vA) return AMPCOR_ERR_ARG;
    if (!h->is_setup) return fail(h, AMPCOR_ERR_STATE, "setupParams must be called first");
    if (n != (int64_t)h->refD.size())
        return fail(h, AMPCOR_ERR_ARG, "gross offsets have %lld entries, expected %zu", (long long)n, h->refD.size());
    const ampcor_params& p = h->p;
    for (int row = 0; row < p.numberWindowDown; ++row)
        for (int col = 0; col < p.numberWindowAcross; ++col) {
            const size_t i = (size_t)row * p.numberWindowAcross + col;
            h->refD[i] = p.referenceStartPixelDownStatic + row * p.skipSampleDown;
            h->refA[i] = p.referenceStartPixelAcrossStatic + col * p.skipSampleAcross;
            h->grossD[i] = vD[i];
            h->grossA[i] = vA[i];
        }
    fill_coords(h);
    return AMPCOR_OK;
}

int ampcor_set_start_pixels(ampcor_handle* h, const int32_t* refD, const int32_t* refA, const int32_t* grossD,
                            const int32_t* grossA, int64_t n) {
    if (!h || !refD || !refA || !grossD || !grossA) return AMPCOR_ERR_ARG;
    if (!h->is_setup) return fail(h, AMPCOR_ERR_STATE, "setupParams must be called first");
    if (n != (int64_t)h->refD.size())
        return fail(h, AMPCOR_ERR_ARG, "start pixels have %lld entries, expected %zu", (long long)n, h->refD.size());
    std::copy(refD, refD + n, h->refD.begin());
    std::copy(refA, refA + n, h->refA.begin());
    std::copy(grossD, grossD + n, h->grossD.begin());
    std::copy(grossA, grossA + n, h->grossA.begin());
    fill_coords(h);
    return AMPCOR_OK;
}

int ampcor_get_start_pixels(const ampcor_handle* h, int32_t* refD, int32_t* refA, int32_t* grossD, int32_t* grossA,
                            int64_t n) {
    if (!h) return AMPCOR_ERR_ARG;
    if (!h->is_setup || !h->has_starts) return AMPCOR_ERR_STATE;
    if (n != (int64_t)h->refD.size()) return AMPCOR_ERR_ARG;
    if (refD) std::copy(h->refD.begin(), h->refD.end(), refD);
    if (refA) std::copy(h->refA.begin(), h->refA.end(), refA);
    if (grossD) std::copy(h->grossD.begin(), h->grossD.end(), grossD);
    if (grossA) std::copy(h->grossA.begin(), h->grossA.end(), grossA);
    return AMPCOR_OK;
}

// cuAmpcorParameter::checkPixelInImageRange (cuAmpcorParameter.cpp:275-331),
// plus the extent of the zoom-in chip, which the kernels read from the image.
static int check_range_impl(ampcor_handle* h) {
    const ampcor_params& p = h->p;
    const WindowPlan& P = h->plan;
    for (int row = 0; row < p.numberWindowDown; ++row)
        for (int col = 0; col < p.numberWindowAcross; ++col) {
            const size_t i = (size_t)row * p.numberWindowAcross + col;
            const WindowCoords& c = h->coords[i];
            if (c.refD < 0)
                return fail(h, AMPCOR_ERR_RANGE, "Reference Window start pixel out ot range in Down, window (%d,%d), pixel %d", row, col, c.refD);
            if (c.refA < 0)
                return fail(h, AMPCOR_ERR_RANGE, "Reference Window start pixel out ot range in Across, window (%d,%d), pixel %d", row, col, c.refA);
            if (c.refD + P.Wh >= p.referenceImageHeight)
                return fail(h, AMPCOR_ERR_RANGE, "Reference Window end pixel out ot range in Down, window (%d,%d), pixel %d", row, col, c.refD + P.Wh);
            if (c.refA + P.Ww >= p.referenceImageWidth)
                return fail(h, AMPCOR_ERR_RANGE, "Reference Window end pixel out ot range in Across, window (%d,%d), pixel %d", row, col, c.refA + P.Ww);
            if (c.secD < 0)
                return fail(h, AMPCOR_ERR_RANGE, "Secondary Window start pixel out ot range in Down, window (%d,%d), pixel %d", row, col, c.secD);
            if (c.secA < 0)
                return fail(h, AMPCOR_ERR_RANGE, "Secondary Window start pixel out ot range in Across, window (%d,%d), pixel %d", row, col, c.secA);
            const int endD = c.secD + std::max(P.Hs, P.Wh + 2 * P.hsD);
            const int endA = c.secA + std::max(P.Ws, P.Ww + 2 * P.hsA);
            if (endD >= p.secondaryImageHeight)
                return fail(h, AMPCOR_ERR_RANGE, "Secondary Window end pixel out ot range in Down, window (%d,%d), pixel %d", row, col, endD);
            if (endA >= p.secondaryImageWidth)
                return fail(h, AMPCOR_ERR_RANGE, "Secondary Window end pixel out ot range in Across, window (%d,%d), pixel %d", row, col, endA);
        }
    return AMPCOR_OK;
}

int ampcor_check_range(ampcor_handle* h) {
    if (!h) return AMPCOR_ERR_ARG;
    if (!h->is_setup || !h->has_starts) return fail(h, AMPCOR_ERR_STATE, "setupParams and start pixels first");
    h->err.clear();
    return check_range_impl(h);
}

}  // extern "C"

// Shift tables of the tensor-core oversampler: the half-sample shift of a
// length-n line, S[j'][j] = (1/n) sum_f e^{2 pi i f (j - j')/n} e^{-i pi sf/n}
// (sf the signed frequency), in real form [[Sr, -Si], [Si, Sr]] padded to
// 2*pad16(n), split into bf16 hi + lo, in the K-major core-matrix layout the
// kernel's B operand uses.  Computed in FP64.
static uint16_t host_bf16(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    return (uint16_t)((u + 0x7FFFu + ((u >> 16) & 1u)) >> 16);  // round to nearest even
}

static float host_bf16_float(uint16_t b) {
    const uint32_t u = (uint32_t)b << 16;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

static void build_shift_table(int n, std::vector<uint16_t>& out) {
    const int np = (n + 15) & ~15, K = 2 * np;
    out.assign(2 * (size_t)K * K, 0);
    std::vector<double> c(n), sn(n);
    for (int jp = 0; jp < n; ++jp)
        for (int j = 0; j < n; ++j) {
            double sr = 0.0, si = 0.0;
            for (int f = 0; f < n; ++f) {
                const int sf = 2 * f < n ? f : f - n;
                const double ang = 2.0 * M_PI * (double)f * (double)(j - jp) / n - M_PI * (double)sf / n;
                sr += std::cos(ang);
                si += std::sin(ang);
            }
            sr /= n;
            si /= n;
            const int rr[4] = {jp, jp, np + jp, np + jp}, kk[4] = {j, np + j, j, np + j};
            const double vv[4] = {sr, -si, si, sr};
            for (int q = 0; q < 4; ++q) {
                const float x = (float)vv[q];
                const uint16_t hi = host_bf16(x);
                const uint16_t lo = host_bf16(x - host_bf16_float(hi));
                const size_t o = umma::core_offset(rr[q], kk[q], K) / 2;
                out[o] = hi;
                out[(size_t)K * K + o] = lo;
            }
        }
}

template <typename T>
static int grow(ampcor_handle* h, T** ptr, size_t* cap, size_t count) {
    if (*cap >= count && *ptr) return AMPCOR_OK;
    cudaFree(*ptr);
    *ptr = nullptr;
    *cap = 0;
    cudaError_t e = cudaMalloc((void**)ptr, std::max<size_t>(count, 1) * sizeof(T));
    if (e != cudaSuccess) {
        *ptr = nullptr;
        return fail(h, AMPCOR_ERR_ALLOC, "cudaMalloc(%zu bytes): %s", count * sizeof(T), cudaGetErrorString(e));
    }
    *cap = count;
    return AMPCOR_OK;
}

extern "C" {

// Selects the handle's device and creates its device error word.
static int ensure_device(ampcor_handle* h) {
    if (h->dev >= 0 && h->dev != h->p.deviceID) release_device(h);
    CUDA_TRY(h, cudaSetDevice(h->p.deviceID));
    h->dev = h->p.deviceID;
    if (!h->d_errw) {
        CUDA_TRY(h, cudaMalloc(&h->d_errw, 256));
        CUDA_TRY(h, cudaMemset(h->d_errw, 0, 256));
    }
    return AMPCOR_OK;
}

static int prepare_device(ampcor_handle* h) {
    int rc0 = ensure_device(h);
    if (rc0) return rc0;
    {
        const WindowPlan& P = h->plan;
        // attributes of the kernels this geometry launches (the others may
        // need more shared memory than a block can have)
        if (!P.rawL2)
            CUDA_TRY(h, cudaFuncSetAttribute(k_raw, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)raw_smem_bytes(P)));
        if (!os2_applies(P) && !P.osL2)
            CUDA_TRY(h, cudaFuncSetAttribute(k_oversample, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)os_smem_bytes(P)));
        CUDA_TRY(h, cudaFuncSetAttribute(k_zoom, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)zoom_smem_bytes(P)));
        if (P.rawL2) {
            CUDA_TRY(h, cudaDeviceGetAttribute(&h->nsm, cudaDevAttrMultiProcessorCount, h->dev));
            const int occ = raw_l2_blocks_per_sm(P);
            if (occ < 1) return fail(h, AMPCOR_ERR_UNSUPPORTED, "the L2-staged raw kernel does not fit");
            h->raw_l2_grid = occ * h->nsm;
        }
        if (P.osL2) {
            CUDA_TRY(h, cudaFuncSetAttribute(k_oversample2_l2, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)os2_l2_smem_bytes(P)));
            CUDA_TRY(h, cudaDeviceGetAttribute(&h->nsm, cudaDevAttrMultiProcessorCount, h->dev));
            int occ = 0;
            CUDA_TRY(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_oversample2_l2, kOs2L2Threads,
                                                                       os2_l2_smem_bytes(P)));
            h->os_l2_grid = std::max(1, occ) * h->nsm;
        }
        if (P.osTc && !h->d_tc) {
            const int sides[4] = {P.Ww, P.Wh, P.Wz, P.Hz};
            std::vector<uint16_t> all, one;
            for (int k = 0; k < 4; ++k) {
                h->tc_off[k] = all.size() * 2;
                build_shift_table(sides[k], one);
                all.insert(all.end(), one.begin(), one.end());
            }
            CUDA_TRY(h, cudaMalloc(&h->d_tc, all.size() * 2));
            CUDA_TRY(h, cudaMemcpy(h->d_tc, all.data(), all.size() * 2, cudaMemcpyHostToDevice));
            CUDA_TRY(h, cudaFuncSetAttribute(k_oversample_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)os_tc_smem_bytes(P)));
        }
    }
    return AMPCOR_OK;
}

// Workspace of one window batch: a device error word, then the raw-stage
// box-sum scratch, the oversampled chips and the oversampled surfaces, each
// starting on a 256-byte boundary (the TMA-staged kernel reads the chips
// through tensor maps whose base must be 16-byte aligned).
struct WsLayout {
    int* err;
    float2* vbox;
    unsigned char* rawSlots;  // L2-staged raw tile / oversampler chip: one slot per resident CTA
    float* osRef;
    float* osSch;
    float* surf;
    size_t bytes;
};

static size_t a256(size_t b) { return (b + 255) & ~(size_t)255; }

static WsLayout ws_layout(const WindowPlan& P, size_t batch, unsigned char* base, int raw_grid = 0,
                          int os_grid = 0) {
    WsLayout L;
    size_t off = 0;
    L.err = reinterpret_cast<int*>(base + off);
    off += 256;
    L.vbox = reinterpret_cast<float2*>(base + off);
    off += P.rawL2 ? 0 : a256(batch * P.NX * P.Ws * sizeof(float2));
    L.rawSlots = base + off;
    // the raw and oversampling stages run one after the other: they share the slots
    off += std::max(P.rawL2 ? (size_t)raw_grid * raw_l2_slot_bytes(P) : 0,
                    P.osL2 ? (size_t)os_grid * os2_l2_slot_bytes(P) : 0);
    L.osRef = reinterpret_cast<float*>(base + off);
    off += a256(batch * P.osWh * P.osWw * sizeof(float));
    L.osSch = reinterpret_cast<float*>(base + off);
    off += a256(batch * P.osHz * P.osWz * sizeof(float));
    L.surf = reinterpret_cast<float*>(base + off);
    off += a256(batch * P.zp * P.zp * sizeof(float));
    L.bytes = off;
    return L;
}

static size_t ws_layout_floats(const WindowPlan& P, size_t batch, int raw_grid, int os_grid) {
    return (ws_layout(P, batch, nullptr, raw_grid, os_grid).bytes + sizeof(float) - 1) / sizeof(float);
}

static int stage_begin(ampcor_handle* h, int stage, cudaStream_t st) {
    h->launches[stage] += 1;
    if (!h->timing) return AMPCOR_OK;
    if (h->ev_used == h->ev_start.size()) {
        cudaEvent_t a, b;
        CUDA_TRY(h, cudaEventCreate(&a));
        CUDA_TRY(h, cudaEventCreate(&b));
        h->ev_start.push_back(a);
        h->ev_end.push_back(b);
        h->ev_stage.push_back(stage);
    }
    h->ev_stage[h->ev_used] = stage;
    CUDA_TRY(h, cudaEventRecord(h->ev_start[h->ev_used], st));
    return AMPCOR_OK;
}

static int stage_end(ampcor_handle* h, cudaStream_t st) {
    if (!h->timing) return AMPCOR_OK;
    CUDA_TRY(h, cudaEventRecord(h->ev_end[h->ev_used], st));
    h->ev_used += 1;
    return AMPCOR_OK;
}

// errw: device error word the kernels set when a bounded wait gives up; null
// uses the workspace's word, zeroed first (ampcor_run_host reads it back).
static int run_impl(ampcor_handle* h, const void* ref, int64_t ref_ld, const void* sec, int64_t sec_ld, float* offset,
                    float* snr, float* cov, int32_t* diag, cudaStream_t st, int* errw = nullptr) {
    const WindowPlan& P = h->plan;
    const int nwin = h->geo.numberWindows;
    int rc;
    if (h->coords_dirty) {
        if ((rc = grow(h, &h->d_coords, &h->coords_cap, (size_t)nwin))) return rc;
        CUDA_TRY(h, cudaMemcpyAsync(h->d_coords, h->coords.data(), (size_t)nwin * sizeof(WindowCoords),
                                    cudaMemcpyHostToDevice, st));
        h->coords_dirty = false;
    }
    if ((rc = grow(h, &h->d_res, &h->res_cap, (size_t)nwin))) return rc;
    const size_t per = (size_t)P.osWh * P.osWw + (size_t)P.osHz * P.osWz + (size_t)P.zp * P.zp +
                       2 * (size_t)P.NX * P.Ws;
    size_t batch = std::max<size_t>(1, std::min<size_t>((size_t)nwin, kWorkspaceBudget / (per * sizeof(float))));
    const int raw_grid = P.rawL2 ? (int)std::min<size_t>(batch, (size_t)h->raw_l2_grid) : 0;
    const int os_grid = P.osL2 ? (int)std::min<size_t>(2 * batch, (size_t)h->os_l2_grid) : 0;
    const size_t ws_floats = ws_layout_floats(P, batch, raw_grid, os_grid);
    if ((rc = grow(h, &h->d_ws, &h->ws_cap, ws_floats))) return rc;
    WsLayout L = ws_layout(P, batch, reinterpret_cast<unsigned char*>(h->d_ws), raw_grid, os_grid);
    int* derr = errw ? errw : L.err;
    float2* vbox = L.vbox;
    float* osRef = L.osRef;
    float* osSch = L.osSch;
    float* surf = L.surf;
    if (!errw) CUDA_TRY(h, cudaMemsetAsync(derr, 0, sizeof(int), st));
    const cfloat* R = static_cast<const cfloat*>(ref);
    const cfloat* S = static_cast<const cfloat*>(sec);
    for (int w0 = 0; w0 < nwin; w0 += (int)batch) {
        const int wend = std::min(nwin, w0 + (int)batch);
        const int nb = wend - w0;
        if ((rc = stage_begin(h, 0, st))) return rc;
        if (P.rawL2)
            CUDA_TRY(h, launch_raw_l2(P, std::min(nb, raw_grid), st, R, ref_ld, S, sec_ld, h->d_coords, w0, wend,
                                      h->d_res, L.rawSlots, raw_l2_slot_bytes(P)));
        else
            k_raw<<<nb, 512, raw_smem_bytes(P), st>>>(P, R, ref_ld, S, sec_ld, h->d_coords, w0, wend, h->d_res,
                                                      vbox);
        if ((rc = stage_end(h, st))) return rc;
        if ((rc = stage_begin(h, 1, st))) return rc;
        if (P.osTc) {
            const uint4* tab = reinterpret_cast<const uint4*>(h->d_tc);
            k_oversample_tc<<<dim3(nb, 2), kOsTcThreads, os_tc_smem_bytes(P), st>>>(
                P, R, ref_ld, S, sec_ld, h->d_coords, w0, wend, h->d_res, osRef, osSch, tab + h->tc_off[0] / 16,
                tab + h->tc_off[1] / 16, tab + h->tc_off[2] / 16, tab + h->tc_off[3] / 16, derr);
        } else if (P.osL2)
            k_oversample2_l2<<<std::min(2 * nb, os_grid), kOs2L2Threads, os2_l2_smem_bytes(P), st>>>(
                P, R, ref_ld, S, sec_ld, h->d_coords, w0, wend, h->d_res, osRef, osSch, L.rawSlots,
                os2_l2_slot_bytes(P));
        else
            launch_oversample(P, nb, st, R, ref_ld, S, sec_ld, h->d_coords, w0, wend, h->d_res, osRef, osSch);
        if ((rc = stage_end(h, st))) return rc;
        if ((rc = stage_begin(h, 2, st))) return rc;
        launch_corr_os_best(P, nb, st, w0, wend, h->d_res, osRef, osSch, surf, derr);
        if ((rc = stage_end(h, st))) return rc;
        if ((rc = stage_begin(h, 3, st))) return rc;
        k_zoom<<<nb, 256, zoom_smem_bytes(P), st>>>(P, w0, wend, h->d_res, h->d_coords, surf, h->p.mergeGrossOffset,
                                                     reinterpret_cast<float2*>(offset), snr, cov, diag);
        if ((rc = stage_end(h, st))) return rc;
        CUDA_TRY(h, cudaGetLastError());
    }
    return AMPCOR_OK;
}

static int run_checks(ampcor_handle* h, const void* ref, int64_t ref_ld, const void* sec, int64_t sec_ld,
                      const float* offset, const float* snr, const float* cov) {
    if (!h) return AMPCOR_ERR_ARG;
    h->err.clear();
    if (!h->is_setup || !h->has_starts)
        return fail(h, AMPCOR_ERR_STATE, "setupParams and a gross-offset setter must be called before runAmpcor");
    if (!ref || !sec || !offset || !snr || !cov) return fail(h, AMPCOR_ERR_ARG, "null image or output pointer");
    if (ref_ld < h->p.referenceImageWidth || sec_ld < h->p.secondaryImageWidth)
        return fail(h, AMPCOR_ERR_ARG, "leading dimension smaller than the image width");
    return check_range_impl(h);
}

int ampcor_run_device(ampcor_handle* h, const void* ref, int64_t ref_ld, const void* sec, int64_t sec_ld,
                      float* offset, float* snr, float* cov, int32_t* diag, void* stream) {
    int rc = run_checks(h, ref, ref_ld, sec, sec_ld, offset, snr, cov);
    if (rc) return rc;
    if ((rc = prepare_device(h))) return rc;
    h->last_run = 1;
    return run_impl(h, ref, ref_ld, sec, sec_ld, offset, snr, cov, diag, static_cast<cudaStream_t>(stream),
                    h->d_errw);
}

int ampcor_run_host(ampcor_handle* h, const void* ref, int64_t ref_ld, const void* sec, int64_t sec_ld,
                    float* offset, float* snr, float* cov, int32_t* diag) {
    int rc = run_checks(h, ref, ref_ld, sec, sec_ld, offset, snr, cov);
    if (rc) return rc;
    if ((rc = prepare_device(h))) return rc;
    const size_t nref = (size_t)ref_ld * h->p.referenceImageHeight;
    const size_t nsec = (size_t)sec_ld * h->p.secondaryImageHeight;
    const size_t nwin = (size_t)h->geo.numberWindows;
    if ((rc = grow(h, reinterpret_cast<cfloat**>(&h->d_ref), &h->ref_cap, nref))) return rc;
    if ((rc = grow(h, reinterpret_cast<cfloat**>(&h->d_sec), &h->sec_cap, nsec))) return rc;
    if ((rc = grow(h, &h->d_out, &h->out_cap, nwin * 6))) return rc;
    if (diag && (rc = grow(h, &h->d_diag, &h->diag_cap, nwin * 8))) return rc;
    cudaStream_t st = nullptr;
    CUDA_TRY(h, cudaMemcpyAsync(h->d_ref, ref, nref * sizeof(cfloat), cudaMemcpyHostToDevice, st));
    CUDA_TRY(h, cudaMemcpyAsync(h->d_sec, sec, nsec * sizeof(cfloat), cudaMemcpyHostToDevice, st));
    float* doff = h->d_out;
    float* dsnr = doff + 2 * nwin;
    float* dcov = dsnr + nwin;
    rc = run_impl(h, h->d_ref, ref_ld, h->d_sec, sec_ld, doff, dsnr, dcov, diag ? h->d_diag : nullptr, st);
    if (rc) return rc;
    CUDA_TRY(h, cudaMemcpyAsync(offset, doff, 2 * nwin * sizeof(float), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(h, cudaMemcpyAsync(snr, dsnr, nwin * sizeof(float), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(h, cudaMemcpyAsync(cov, dcov, 3 * nwin * sizeof(float), cudaMemcpyDeviceToHost, st));
    if (diag) CUDA_TRY(h, cudaMemcpyAsync(diag, h->d_diag, 8 * nwin * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    int derr = 0;
    CUDA_TRY(h, cudaMemcpyAsync(&derr, h->d_ws, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(h, cudaStreamSynchronize(st));
    if (derr) return fail(h, AMPCOR_ERR_CUDA, "a device-side wait gave up (results of this run are invalid)");
    return AMPCOR_OK;
}

int ampcor_set_timing(ampcor_handle* h, int enable) {
    if (!h) return AMPCOR_ERR_ARG;
    h->timing = enable != 0;
    h->ev_used = 0;
    for (long long& c : h->launches) c = 0;
    return AMPCOR_OK;
}

int ampcor_set_precision(ampcor_handle* h, int32_t mode) {
    if (!h) return AMPCOR_ERR_ARG;
    if (mode < 0 || mode > 2) return fail(h, AMPCOR_ERR_ARG, "precision mode %d is not 0, 1 or 2", mode);
    h->precision = mode;
    h->is_setup = false;
    h->has_starts = false;
    cudaFree(h->d_tc);
    h->d_tc = nullptr;
    return AMPCOR_OK;
}

int ampcor_set_corr_precision(ampcor_handle* h, int32_t mode) {
    if (!h) return AMPCOR_ERR_ARG;
    if (mode < 0 || mode > 2) return fail(h, AMPCOR_ERR_ARG, "correlation precision mode %d is not 0, 1 or 2", mode);
    h->corr_precision = mode;
    h->is_setup = false;
    h->has_starts = false;
    return AMPCOR_OK;
}

int ampcor_set_raw_mode(ampcor_handle* h, int32_t mode) {
    if (!h) return AMPCOR_ERR_ARG;
    if (mode < 0 || mode > 3) return fail(h, AMPCOR_ERR_ARG, "raw mode %d is not 0, 1, 2 or 3", mode);
    h->raw_mode = mode;
    h->is_setup = false;
    h->has_starts = false;
    return AMPCOR_OK;
}

int ampcor_read_timing(ampcor_handle* h, float* ms, int64_t* launches, int32_t nstage) {
    if (!h || nstage < kNumStages) return AMPCOR_ERR_ARG;
    h->err.clear();
    for (int s = 0; s < kNumStages; ++s) {
        if (ms) ms[s] = 0.f;
        if (launches) launches[s] = h->launches[s];
    }
    if (ms) {
        for (size_t i = 0; i < h->ev_used; ++i) {
            float t = 0.f;
            CUDA_TRY(h, cudaEventSynchronize(h->ev_end[i]));
            CUDA_TRY(h, cudaEventElapsedTime(&t, h->ev_start[i], h->ev_end[i]));
            ms[h->ev_stage[i]] += t;
        }
    }
    h->ev_used = 0;
    for (long long& c : h->launches) c = 0;
    return AMPCOR_OK;
}

int ampcor_last_error(const ampcor_handle* h, char* buf, int64_t n) {
    if (!h || !buf || n <= 0) return AMPCOR_ERR_ARG;
    std::snprintf(buf, (size_t)n, "%s", h->err.c_str());
    return AMPCOR_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free run.
//
// Some callers cannot call cudaMalloc: hosts that hand the whole device to
// their own memory pool before loading this library (a serving process whose
// allocator owns every byte, a framework that forbids driver allocations on
// its hot path because cudaMalloc can synchronise the device or fail under
// memory pressure).  For them, ampcor_run_device_noalloc takes its working
// memory from one file-scope device array of AMPCOR_NOALLOC_SCRATCH_BYTES
// instead of the handle's cudaMalloc'd workspace.  The array is part of the
// loaded module, so every GPU on which the library is used holds it until the
// process exits.
// ---------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_noalloc_scratch[AMPCOR_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int kMaxNoallocDevices = 64;
void* g_noalloc_addr[kMaxNoallocDevices] = {};
size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }
}  // namespace

// Device address of the scratch array on the current device (looked up once
// per device; host code must not use the array's name as an address).
static int noalloc_scratch(ampcor_handle* h, int dev, unsigned char** out) {
    if (dev < 0 || dev >= kMaxNoallocDevices)
        return fail(h, AMPCOR_ERR_ARG, "device %d outside the allocation-free table", dev);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr)
            return fail(h, AMPCOR_ERR_CUDA, "cudaGetSymbolAddress(scratch) failed: %s", cudaGetErrorString(e));
        g_noalloc_addr[dev] = p;
    }
    *out = static_cast<unsigned char*>(g_noalloc_addr[dev]);
    return AMPCOR_OK;
}

extern "C" int ampcor_run_device_noalloc(ampcor_handle* h, const void* ref, int64_t ref_ld, const void* sec,
                                         int64_t sec_ld, float* offset, float* snr, float* cov, void* stream) {
    int rc = run_checks(h, ref, ref_ld, sec, sec_ld, offset, snr, cov);
    if (rc) return rc;
    const WindowPlan& P = h->plan;
    if (P.rawL2 || P.osL2 || P.osTc)
        return fail(h, AMPCOR_ERR_UNSUPPORTED,
                    "allocation-free run: windows of %d x %d need the L2-staged path; use ampcor_run_device",
                    P.Wh, P.Ww);
    // device selection and kernel attributes only: nothing here allocates or frees
    CUDA_TRY(h, cudaSetDevice(h->p.deviceID));
    CUDA_TRY(h, cudaFuncSetAttribute(k_raw, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)raw_smem_bytes(P)));
    if (!os2_applies(P))
        CUDA_TRY(h, cudaFuncSetAttribute(k_oversample, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)os_smem_bytes(P)));
    CUDA_TRY(h, cudaFuncSetAttribute(k_zoom, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)zoom_smem_bytes(P)));
    unsigned char* base = nullptr;
    if ((rc = noalloc_scratch(h, h->p.deviceID, &base))) return rc;
    const int nwin = h->geo.numberWindows;
    const size_t coords_b = align256((size_t)nwin * sizeof(WindowCoords));
    const size_t res_b = align256((size_t)nwin * sizeof(RawResult));
    const size_t per_f = (size_t)P.osWh * P.osWw + (size_t)P.osHz * P.osWz + (size_t)P.zp * P.zp +
                         2 * (size_t)P.NX * P.Ws;  // floats per window, as in the allocating path
    // layout: [0, 256) the device error word (the first int, kept until
    // ampcor_run_status reads it), then coordinates, results, workspace
    const size_t head = 256;
    const size_t fixed = head + coords_b + res_b + 256;  // + the workspace's own (unused) word
    if (fixed + per_f * sizeof(float) + 256 > (size_t)AMPCOR_NOALLOC_SCRATCH_BYTES)
        return fail(h, AMPCOR_ERR_UNSUPPORTED,
                    "allocation-free run needs %zu bytes for %d windows (plus %zu per window in flight) but its "
                    "static scratch holds %zu; use ampcor_run_device or fewer windows per call",
                    fixed, nwin, per_f * sizeof(float), (size_t)AMPCOR_NOALLOC_SCRATCH_BYTES);
    size_t batch = std::min<size_t>((size_t)nwin,
                                    ((size_t)AMPCOR_NOALLOC_SCRATCH_BYTES - fixed - 256) / (per_f * sizeof(float)));
    // the 256-byte alignment of each workspace region may cost a little more
    while (batch > 1 &&
           head + coords_b + res_b + ws_layout(P, batch, nullptr).bytes > (size_t)AMPCOR_NOALLOC_SCRATCH_BYTES)
        --batch;
    if (head + coords_b + res_b + ws_layout(P, batch, nullptr).bytes > (size_t)AMPCOR_NOALLOC_SCRATCH_BYTES)
        return fail(h, AMPCOR_ERR_UNSUPPORTED, "allocation-free run: one window's workspace does not fit the static scratch");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int* errw = reinterpret_cast<int*>(base);
    WindowCoords* d_coords = reinterpret_cast<WindowCoords*>(base + head);
    RawResult* d_res = reinterpret_cast<RawResult*>(base + head + coords_b);
    WsLayout L = ws_layout(P, batch, base + head + coords_b + res_b);
    float2* vbox = L.vbox;
    float* osRef = L.osRef;
    float* osSch = L.osSch;
    float* surf = L.surf;
    // Every byte a stage reads is written earlier in this call (coordinates
    // below, results and workspace by the preceding stage).  The error word
    // starts at zero with the module and is cleared by ampcor_run_status.
    h->last_run = 2;
    CUDA_TRY(h, cudaMemcpyAsync(d_coords, h->coords.data(), (size_t)nwin * sizeof(WindowCoords),
                                cudaMemcpyHostToDevice, st));
    const cfloat* R = static_cast<const cfloat*>(ref);
    const cfloat* S = static_cast<const cfloat*>(sec);
    for (int w0 = 0; w0 < nwin; w0 += (int)batch) {
        const int wend = std::min(nwin, w0 + (int)batch);
        const int nb = wend - w0;
        k_raw<<<nb, 512, raw_smem_bytes(P), st>>>(P, R, ref_ld, S, sec_ld, d_coords, w0, wend, d_res, vbox);
        launch_oversample(P, nb, st, R, ref_ld, S, sec_ld, d_coords, w0, wend, d_res, osRef, osSch);
        launch_corr_os_best(P, nb, st, w0, wend, d_res, osRef, osSch, surf, errw);
        k_zoom<<<nb, 256, zoom_smem_bytes(P), st>>>(P, w0, wend, d_res, d_coords, surf, h->p.mergeGrossOffset,
                                                     reinterpret_cast<float2*>(offset), snr, cov, nullptr);
        CUDA_TRY(h, cudaGetLastError());
    }
    return AMPCOR_OK;
}

// Reads and clears the device error word of the handle's last device run
// (the handle's own word for ampcor_run_device, the word at the head of the
// device's static scratch for ampcor_run_device_noalloc) after `stream` has
// finished.  Allocates nothing: the word is copied to a local through a
// stream-ordered copy.
extern "C" int ampcor_run_status(ampcor_handle* h, void* stream, int32_t* device_error) {
    if (!h) return AMPCOR_ERR_ARG;
    h->err.clear();
    if (device_error) *device_error = 0;
    int* word = nullptr;
    if (h->last_run == 1) {
        word = h->d_errw;
    } else if (h->last_run == 2) {
        unsigned char* base = nullptr;
        int rc = noalloc_scratch(h, h->p.deviceID, &base);
        if (rc) return rc;
        word = reinterpret_cast<int*>(base);
    } else {
        return AMPCOR_OK;  // no asynchronous run yet
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int v = 0;
    CUDA_TRY(h, cudaSetDevice(h->p.deviceID));
    CUDA_TRY(h, cudaMemcpyAsync(&v, word, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(h, cudaMemsetAsync(word, 0, sizeof(int), st));
    CUDA_TRY(h, cudaStreamSynchronize(st));
    if (device_error) *device_error = v;
    if (v) return fail(h, AMPCOR_ERR_CUDA, "a device-side wait of the run gave up: its results are invalid");
    return AMPCOR_OK;
}

// A bounded mbarrier wait on a barrier nothing arrives at: it gives up after
// `polls` polls and sets the error word, then the kernel returns normally.
__global__ void k_wait_selftest(int* err, unsigned polls) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) umma::mbar_init(&bar, 1);
    __syncthreads();
    if (!umma::mbar_wait(&bar, 0, polls) && threadIdx.x == 0) atomicExch(err, 1);
}

extern "C" int ampcor_selftest_wait_timeout(ampcor_handle* h, uint32_t polls, void* stream) {
    if (!h || polls == 0 || polls > (1u << 20)) return AMPCOR_ERR_ARG;
    h->err.clear();
    int rc = ensure_device(h);
    if (rc) return rc;
    k_wait_selftest<<<1, 32, 0, static_cast<cudaStream_t>(stream)>>>(h->d_errw, polls);
    CUDA_TRY(h, cudaGetLastError());
    h->last_run = 1;
    return AMPCOR_OK;
}

// ---------------------------------------------------------------------------
// Batched runs: many jobs (each a set-up handle with its own geometry and
// images) in one persistent launch.  No counterpart in the reference, whose
// controller runs one image pair per call (cuAmpcorController.cpp:37-178).
// ---------------------------------------------------------------------------
struct ampcor_batch {
    int dev = 0;
    std::vector<BatchJob> jobs;
    std::vector<WindowCoords*> d_coords;  // one device copy per job
    std::vector<double> cost;             // per-window cost estimate per job
    std::vector<int> nwin;
    BatchJob* d_jobs = nullptr;
    size_t jobs_cap = 0;
    int2* d_items = nullptr;
    size_t items_cap = 0;
    int nitems = 0;
    int* d_next = nullptr;
    unsigned char* d_scratch = nullptr;
    size_t scratch_cap = 0;
    bool dirty = true;
    int nt = 512;             // threads per CTA (autotuned)
    int per_sm = 1;           // CTAs per SM (autotuned)
    int raw_l2 = 0;           // 1: every job's raw tile L2-staged (autotuned)
    int bulk = 0;             // 1: bulk-copied, double-buffered oversampled correlation (autotuned)
    int mode = 0;             // 0: one fused persistent kernel; 1: chain of four stage kernels per wave
    bool shape_chosen = false;  // set by ampcor_batch_set_shape / ampcor_batch_tune
    ChainPlan chain;          // chain mode: waves and workspace sizes
    // chain stage timing (non-graph runs while enabled)
    struct Timer : ChainTimer {
        mutable std::vector<cudaEvent_t> ev0, ev1;
        mutable std::vector<int> stage;
        mutable size_t used = 0;
        cudaError_t begin(int s, cudaStream_t st) const override {
            if (used == ev0.size()) {
                cudaEvent_t a, b;
                cudaError_t e = cudaEventCreate(&a);
                if (e == cudaSuccess) e = cudaEventCreate(&b);
                if (e != cudaSuccess) return e;
                ev0.push_back(a);
                ev1.push_back(b);
                stage.push_back(s);
            }
            stage[used] = s;
            return cudaEventRecord(ev0[used], st);
        }
        cudaError_t end(int, cudaStream_t st) const override { return cudaEventRecord(ev1[used++], st); }
        ~Timer() override {
            for (cudaEvent_t e : ev0) cudaEventDestroy(e);
            for (cudaEvent_t e : ev1) cudaEventDestroy(e);
        }
    } timer;
    bool timing = false;
    WaveLayout wl{};
    unsigned char* d_wave = nullptr;
    size_t wave_cap = 0;
    size_t smem = 0;
    SlotLayout slot{};
    int grid = 0;
    cudaGraphExec_t gexec = nullptr;
    cudaStream_t gstream = nullptr;
    std::string err;
};

static int bfail(ampcor_batch* b, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (b) b->err = buf;
    return code;
}

#define BCUDA_TRY(b, call)                                                                        \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return bfail(b, AMPCOR_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));     \
    } while (0)

static void batch_drop_graph(ampcor_batch* b) {
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    b->gexec = nullptr;
    b->gstream = nullptr;
}

extern "C" int ampcor_batch_create(ampcor_batch** out, int32_t deviceID) {
    if (!out) return AMPCOR_ERR_ARG;
    ampcor_batch* b = new (std::nothrow) ampcor_batch();
    if (!b) return AMPCOR_ERR_ALLOC;
    b->dev = deviceID;
    *out = b;
    return AMPCOR_OK;
}

extern "C" int ampcor_batch_clear(ampcor_batch* b) {
    if (!b) return AMPCOR_ERR_ARG;
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(b->dev);
    for (WindowCoords* c : b->d_coords) cudaFree(c);
    cudaSetDevice(cur);
    b->d_coords.clear();
    b->jobs.clear();
    b->cost.clear();
    b->nwin.clear();
    b->nitems = 0;
    b->dirty = true;
    batch_drop_graph(b);
    return AMPCOR_OK;
}

extern "C" int ampcor_batch_destroy(ampcor_batch* b) {
    if (!b) return AMPCOR_ERR_ARG;
    ampcor_batch_clear(b);
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(b->dev);
    cudaFree(b->d_jobs);
    cudaFree(b->d_items);
    cudaFree(b->d_next);
    cudaFree(b->d_scratch);
    cudaFree(b->d_wave);
    cudaSetDevice(cur);
    delete b;
    return AMPCOR_OK;
}

extern "C" int ampcor_batch_add(ampcor_batch* b, ampcor_handle* h, const void* ref, int64_t ref_ld, const void* sec,
                                int64_t sec_ld, float* offset, float* snr, float* cov, int32_t* job_index) {
    if (!b || !h) return AMPCOR_ERR_ARG;
    b->err.clear();
    int rc = run_checks(h, ref, ref_ld, sec, sec_ld, offset, snr, cov);
    if (rc) return bfail(b, rc, "job %zu: %s", b->jobs.size(), h->err.c_str());
    if (h->p.deviceID != b->dev) return bfail(b, AMPCOR_ERR_ARG, "job on device %d, batch on %d", h->p.deviceID, b->dev);
    if (!corr_os_supported(h->plan.zp))
        return bfail(b, AMPCOR_ERR_UNSUPPORTED,
                     "job %zu: kept oversampled surface side %d runs only through ampcor_run_device",
                     b->jobs.size(), h->plan.zp);
    {
        WindowPlan P = h->plan;
        if (!fit_plan_smem(P, 256, kSmemLimit - 4096))
            return bfail(b, AMPCOR_ERR_UNSUPPORTED,
                         "job geometry needs more shared memory than the persistent kernel has");
    }
    BCUDA_TRY(b, cudaSetDevice(b->dev));
    const int n = h->geo.numberWindows;
    WindowCoords* dc = nullptr;
    BCUDA_TRY(b, cudaMalloc(&dc, (size_t)n * sizeof(WindowCoords)));
    cudaError_t e = cudaMemcpy(dc, h->coords.data(), (size_t)n * sizeof(WindowCoords), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(dc);
        return bfail(b, AMPCOR_ERR_CUDA, "coordinate upload failed: %s", cudaGetErrorString(e));
    }
    BatchJob J{};
    J.P = h->plan;
    J.ref = static_cast<const cfloat*>(ref);
    J.sec = static_cast<const cfloat*>(sec);
    J.ldr = ref_ld;
    J.lds = sec_ld;
    J.coords = dc;
    J.offset = reinterpret_cast<float2*>(offset);
    J.snr = snr;
    J.cov = cov;
    J.merge = h->p.mergeGrossOffset;
    b->jobs.push_back(J);
    // the tensor-core correlation runs in chain mode only: a batch whose shape
    // was not chosen takes the chain when such a job arrives
    if (J.P.cosTc && !b->shape_chosen) b->mode = 1;
    b->d_coords.push_back(dc);
    b->nwin.push_back(n);
    const WindowPlan& P = h->plan;
    b->cost.push_back((double)P.P * P.Q * 14.0 + (double)(P.Hz * P.Wz + P.Wh * P.Ww) * 60.0 +
                      (double)P.osWh * P.osWw * P.zp * P.zp + (double)P.M * P.M / 16.0);
    b->dirty = true;
    batch_drop_graph(b);
    if (job_index) *job_index = (int32_t)b->jobs.size() - 1;
    return AMPCOR_OK;
}

constexpr size_t kWaveBudget = size_t(2) << 30;

static int chain_prepare(ampcor_batch* b, const std::vector<int2>& items, const std::vector<WindowPlan>& plans,
                         int sms) {
    std::string msg;
    if (!plan_chain(plans, items, sms, kWaveBudget, &b->chain, &msg))
        return bfail(b, AMPCOR_ERR_UNSUPPORTED, "%s", msg.c_str());
    const size_t need = b->chain.bytes();
    if (b->wave_cap < need) {
        cudaFree(b->d_wave);
        b->d_wave = nullptr;
        b->wave_cap = 0;
        BCUDA_TRY(b, cudaMalloc(&b->d_wave, need));
        b->wave_cap = need;
    }
    chain_layout(b->chain, b->d_wave, &b->wl);
    b->grid = (int)b->chain.waves.size();
    return AMPCOR_OK;
}

static int batch_prepare(ampcor_batch* b, cudaStream_t st) {
    if (!b->dirty) return AMPCOR_OK;
    BCUDA_TRY(b, cudaSetDevice(b->dev));
    // the fused kernel correlates the oversampled chips on the FMA pipes
    // only: a job that asked for the tensor-core correlation runs in chain mode
    if (b->mode == 0)
        for (const BatchJob& J : b->jobs)
            if (J.P.cosTc)
                return bfail(b, AMPCOR_ERR_UNSUPPORTED,
                             "a job uses the tensor-core oversampled correlation, which the fused kernel does not "
                             "run: use the chain shape");
    // work list: every window of every job, most expensive first
    std::vector<int2> items;
    for (size_t j = 0; j < b->jobs.size(); ++j)
        for (int w = 0; w < b->nwin[j]; ++w) items.push_back(make_int2((int)j, w));
    std::stable_sort(items.begin(), items.end(),
                     [&](const int2& x, const int2& y) { return b->cost[x.x] > b->cost[y.x]; });
    b->nitems = (int)items.size();
    // effective plans: with raw_l2 every raw tile is L2-staged in groups of
    // 16 lines, which frees shared memory for a second CTA per SM
    std::vector<BatchJob> djobs(b->jobs);
    std::vector<WindowPlan> plans;
    for (BatchJob& J : djobs) {
        if (b->raw_l2 && !J.P.rawL2) {
            J.P.rawL2 = 1;
            J.P.rawGl = 16;
        }
        if (b->mode == 1) {
            // chain: each stage kernel needs only its own body to fit (next to
            // the kernel's static plan copy); the oversampled correlation is
            // double-buffered when that fits
            const size_t lim = kSmemLimit - 4096;
            if (wave_stage_smem(J.P, 0) > lim && !J.P.rawL2) {
                J.P.rawL2 = 1;
                J.P.rawGl = 32;
                while (J.P.rawGl > 2 && raw_l2_smem_bytes(J.P) > lim) J.P.rawGl -= 2;
            }
            if (wave_stage_smem(J.P, 1) > lim && !J.P.osL2 && os2_applies(J.P)) {
                J.P.osL2 = 1;
                J.P.osGl = 32;
                while (J.P.osGl > 2 && os2_l2_smem_bytes(J.P) > lim) J.P.osGl -= 2;
            }
            J.P.cosCols = 0;
            if (corr_os_bulk_applies(J.P))
                for (int c : {32, 16})
                    if (corr_os_bulk_smem_bytes(J.P, c, kWaveCosThreads) <= lim) {
                        J.P.cosCols = c;
                        break;
                    }
            plans.push_back(J.P);
            continue;
        }
        // what still does not fit the launch's thread count moves to L2; with
        // one CTA per SM the oversampled correlation is double-buffered
        fit_plan_smem(J.P, b->nt, kSmemLimit - 4096);
        if (b->bulk && b->per_sm == 1) plan_enable_bulk_corr(J.P, b->nt, kSmemLimit - 4096);
        plans.push_back(J.P);
    }
    // shared memory of the launch: the largest stage body of any job at the
    // launch's thread count (the zoom and oversampled-correlation bodies keep
    // per-warp / per-thread scratch)
    auto smem_for = [&](int nt) {
        size_t m = 0;
        for (const WindowPlan& P : plans) m = std::max(m, batch_smem_bytes(P, nt));
        return m;
    };
    b->smem = smem_for(b->nt);
    b->slot = batch_slot_layout(plans.data(), (int)plans.size());
    if (b->jobs_cap < b->jobs.size()) {
        cudaFree(b->d_jobs);
        b->d_jobs = nullptr;
        BCUDA_TRY(b, cudaMalloc(&b->d_jobs, b->jobs.size() * sizeof(BatchJob)));
        b->jobs_cap = b->jobs.size();
    }
    if (b->items_cap < items.size()) {
        cudaFree(b->d_items);
        b->d_items = nullptr;
        BCUDA_TRY(b, cudaMalloc(&b->d_items, items.size() * sizeof(int2)));
        b->items_cap = items.size();
    }
    if (!b->d_next) BCUDA_TRY(b, cudaMalloc(&b->d_next, 2 * sizeof(int)));  // work counter, error word
    BCUDA_TRY(b, cudaMemcpyAsync(b->d_jobs, djobs.data(), djobs.size() * sizeof(BatchJob), cudaMemcpyHostToDevice, st));
    BCUDA_TRY(b, cudaMemcpyAsync(b->d_items, items.data(), items.size() * sizeof(int2), cudaMemcpyHostToDevice, st));
    BCUDA_TRY(b, cudaStreamSynchronize(st));  // host vectors go out of scope
    int sms = 0;
    BCUDA_TRY(b, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->dev));
    if (b->mode == 1) {
        int rc = chain_prepare(b, items, plans, sms);
        if (rc) return rc;
        b->dirty = false;
        return AMPCOR_OK;
    }
    int fit = persist_blocks_per_sm(b->nt, b->per_sm, b->smem);
    if (fit < 1) {  // fall back to the largest launch that fits
        b->nt = 256;
        b->per_sm = 1;
        b->smem = smem_for(b->nt);
        fit = persist_blocks_per_sm(b->nt, b->per_sm, b->smem);
        if (fit < 1) return bfail(b, AMPCOR_ERR_UNSUPPORTED, "persistent kernel does not fit (smem %zu)", b->smem);
    }
    b->per_sm = std::min(b->per_sm, fit);
    b->grid = sms * b->per_sm;
    const size_t need = (size_t)sms * 2 * b->slot.bytes;  // room for up to two CTAs per SM
    if (b->scratch_cap < need) {
        cudaFree(b->d_scratch);
        b->d_scratch = nullptr;
        BCUDA_TRY(b, cudaMalloc(&b->d_scratch, need));
        b->scratch_cap = need;
    }
    b->dirty = false;
    return AMPCOR_OK;
}

static int batch_launch(ampcor_batch* b, cudaStream_t st) {
    BCUDA_TRY(b, cudaMemsetAsync(b->d_next, 0, 2 * sizeof(int), st));
    if (b->mode == 1) {
        BCUDA_TRY(b, launch_chain(b->chain, b->wl, b->d_jobs, b->d_items, st, b->d_next + 1,
                                  b->timing ? &b->timer : nullptr));
        return AMPCOR_OK;
    }
    BCUDA_TRY(b, launch_persist(b->nt, b->per_sm, b->grid, b->smem, st, b->d_jobs, b->d_items, b->nitems,
                                b->d_next, b->d_scratch, b->slot));
    return AMPCOR_OK;
}

/* flags bit 0: capture the launch in a CUDA graph on the first run and replay
 * it while the job set is unchanged (needs a non-default stream). */
extern "C" int ampcor_batch_run(ampcor_batch* b, void* stream, int32_t flags) {
    if (!b) return AMPCOR_ERR_ARG;
    b->err.clear();
    if (b->jobs.empty()) return bfail(b, AMPCOR_ERR_STATE, "no jobs in the batch");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int rc = batch_prepare(b, st);
    if (rc) return rc;
    BCUDA_TRY(b, cudaSetDevice(b->dev));
    if (!(flags & 1) || b->timing) return batch_launch(b, st);
    if (!st) return bfail(b, AMPCOR_ERR_ARG, "graph replay needs a non-default stream");
    if (!b->gexec || b->gstream != st) {
        batch_drop_graph(b);
        cudaGraph_t g = nullptr;
        BCUDA_TRY(b, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        rc = batch_launch(b, st);
        cudaError_t e = cudaStreamEndCapture(st, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return bfail(b, AMPCOR_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&b->gexec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return bfail(b, AMPCOR_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
        b->gstream = st;
    }
    BCUDA_TRY(b, cudaGraphLaunch(b->gexec, st));
    return AMPCOR_OK;
}

/* Autotuner: times every feasible launch shape (threads per CTA x CTAs per
 * SM x raw-tile placement) on the current job set and keeps the fastest
 * (read it back with ampcor_batch_config); ms_out (optional,
 * AMPCOR_BATCH_TUNE_CANDIDATES entries) gets the measured times of
 * (512,1,auto), (256,1,auto), (256,2,auto), (512,1,L2), (256,2,L2), chain,
 * negative where infeasible ("chain": four stage kernels per wave of items
 * instead of one fused kernel). */
extern "C" int ampcor_batch_tune(ampcor_batch* b, void* stream, float* ms_out) {
    if (!b) return AMPCOR_ERR_ARG;
    b->err.clear();
    if (b->jobs.empty()) return bfail(b, AMPCOR_ERR_STATE, "no jobs in the batch");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int cand[AMPCOR_BATCH_TUNE_CANDIDATES][5] = {
        {512, 1, 0, 0, 0}, {256, 1, 0, 0, 0}, {256, 2, 0, 0, 0}, {512, 1, 1, 0, 0}, {256, 2, 1, 0, 0},
        {512, 1, 0, 0, 1}};
    float best = 1e30f;
    int fail_rc = AMPCOR_OK;
    int bnt = b->nt, bper = b->per_sm, bl2 = b->raw_l2, bbulk = b->bulk, bmode = b->mode;
    cudaEvent_t e0, e1;
    BCUDA_TRY(b, cudaSetDevice(b->dev));
    BCUDA_TRY(b, cudaEventCreate(&e0));
    BCUDA_TRY(b, cudaEventCreate(&e1));
    for (int c = 0; c < AMPCOR_BATCH_TUNE_CANDIDATES; ++c) {
        if (ms_out) ms_out[c] = -1.f;
        b->nt = cand[c][0];
        b->per_sm = cand[c][1];
        b->raw_l2 = cand[c][2];
        b->bulk = cand[c][3];
        b->mode = cand[c][4];
        b->dirty = true;
        batch_drop_graph(b);
        int rc = batch_prepare(b, st);
        if (rc || (b->mode == 0 && b->per_sm != cand[c][1])) continue;  // shape does not fit
        float t = 0.f;
        if ((rc = batch_launch(b, st))) {  // warm-up
            fail_rc = rc;
            break;
        }
        cudaEventRecord(e0, st);
        if ((rc = batch_launch(b, st))) {
            fail_rc = rc;
            break;
        }
        cudaEventRecord(e1, st);
        const cudaError_t se = cudaEventSynchronize(e1);
        if (se != cudaSuccess) {
            fail_rc = bfail(b, AMPCOR_ERR_CUDA, "tuning run of shape %d failed: %s", c, cudaGetErrorString(se));
            break;
        }
        cudaEventElapsedTime(&t, e0, e1);
        if (ms_out) ms_out[c] = t;
        if (t < best) {
            best = t;
            bnt = cand[c][0];
            bper = cand[c][1];
            bl2 = cand[c][2];
            bbulk = cand[c][3];
            bmode = cand[c][4];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (fail_rc) return fail_rc;  // the message is in b->err
    if (best == 1e30f) return bfail(b, AMPCOR_ERR_UNSUPPORTED, "no batched launch shape fits these jobs");
    b->nt = bnt;
    b->per_sm = bper;
    b->raw_l2 = bl2;
    b->bulk = bbulk;
    b->mode = bmode;
    b->shape_chosen = true;
    b->dirty = true;
    batch_drop_graph(b);
    return batch_prepare(b, st);
}

/* Stage timing of chain-mode runs without graph replay: every stage launch
 * is bracketed by CUDA events; ampcor_batch_read_timing waits for them and
 * returns per stage (raw, oversampling, oversampled correlation, zoom) the
 * summed milliseconds and the launches since the last read. */
extern "C" int ampcor_batch_set_timing(ampcor_batch* b, int32_t enable) {
    if (!b) return AMPCOR_ERR_ARG;
    b->timing = enable != 0;
    b->timer.used = 0;
    batch_drop_graph(b);
    return AMPCOR_OK;
}

extern "C" int ampcor_batch_read_timing(ampcor_batch* b, float* ms, int64_t* launches, int32_t nstage) {
    if (!b || nstage < 4) return AMPCOR_ERR_ARG;
    for (int s = 0; s < 4; ++s) {
        if (ms) ms[s] = 0.f;
        if (launches) launches[s] = 0;
    }
    for (size_t i = 0; i < b->timer.used; ++i) {
        float t = 0.f;
        BCUDA_TRY(b, cudaEventSynchronize(b->timer.ev1[i]));
        BCUDA_TRY(b, cudaEventElapsedTime(&t, b->timer.ev0[i], b->timer.ev1[i]));
        if (ms) ms[b->timer.stage[i]] += t;
        if (launches) launches[b->timer.stage[i]] += 1;
    }
    b->timer.used = 0;
    return AMPCOR_OK;
}

/* Select one of the tuner's launch shapes by index (0 ..
 * AMPCOR_BATCH_TUNE_CANDIDATES-1, the order of ampcor_batch_tune's ms_out). */
extern "C" int ampcor_batch_set_shape(ampcor_batch* b, int32_t candidate) {
    if (!b || candidate < 0 || candidate >= AMPCOR_BATCH_TUNE_CANDIDATES) return AMPCOR_ERR_ARG;
    static const int cand[AMPCOR_BATCH_TUNE_CANDIDATES][5] = {
        {512, 1, 0, 0, 0}, {256, 1, 0, 0, 0}, {256, 2, 0, 0, 0}, {512, 1, 1, 0, 0}, {256, 2, 1, 0, 0},
        {512, 1, 0, 0, 1}};
    b->nt = cand[candidate][0];
    b->per_sm = cand[candidate][1];
    b->raw_l2 = cand[candidate][2];
    b->bulk = cand[candidate][3];
    b->mode = cand[candidate][4];
    b->shape_chosen = true;
    b->dirty = true;
    batch_drop_graph(b);
    return AMPCOR_OK;
}

/* Wait for the batch's work on `stream`; AMPCOR_ERR_CUDA if a bounded
 * device-side wait of the last run gave up (its results are invalid). */
extern "C" int ampcor_batch_sync(ampcor_batch* b, void* stream) {
    if (!b) return AMPCOR_ERR_ARG;
    b->err.clear();
    BCUDA_TRY(b, cudaSetDevice(b->dev));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    BCUDA_TRY(b, cudaStreamSynchronize(st));
    if (!b->d_next) return AMPCOR_OK;
    int e = 0;
    BCUDA_TRY(b, cudaMemcpy(&e, b->d_next + 1, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) return bfail(b, AMPCOR_ERR_CUDA, "a device-side wait gave up (results of the last run are invalid)");
    return AMPCOR_OK;
}

extern "C" int ampcor_batch_config(const ampcor_batch* b, int32_t* nt, int32_t* per_sm, int32_t* grid, int64_t* nitems,
                                   int32_t* raw_l2) {
    if (!b) return AMPCOR_ERR_ARG;
    if (raw_l2) *raw_l2 = b->raw_l2 | (b->bulk << 1) | (b->mode << 2);
    if (nt) *nt = b->nt;
    if (per_sm) *per_sm = b->per_sm;
    if (grid) *grid = b->grid;
    if (nitems) *nitems = b->nitems;
    return AMPCOR_OK;
}

extern "C" int ampcor_batch_last_error(const ampcor_batch* b, char* buf, int64_t n) {
    if (!b || !buf || n <= 0) return AMPCOR_ERR_ARG;
    std::snprintf(buf, (size_t)n, "%s", b->err.c_str());
    return AMPCOR_OK;
}
