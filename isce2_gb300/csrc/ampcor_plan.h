// Per-run geometry shared by the host orchestration and the kernels.
#pragma once
#include "fft_smem.cuh"

namespace ampcor {

// Everything a kernel needs to process one window; built once per setup from
// the PyCuAmpcor parameter surface (cuAmpcorParameter.cpp:70-109).
struct WindowPlan {
    // raw stage
    int Wh, Ww;        // reference chip (windowSizeHeightRaw/WidthRaw)
    int hsD, hsA;      // half search ranges (down, across)
    int Hs, Ws;        // search chip: Wh + 2 hsA, Ww + 2 hsD (reference quirk)
    int NX, NY;        // raw correlation surface Hs-Wh+1, Ws-Ww+1
    int statH, statW;  // SNR box (corrRawZoomInHeight/Width)
    int P, Q;          // padded FFT tile for the raw correlation
    int rawL2;         // 1: the P x Q tile lives in an L2-resident global slot
    int rawGl;         // lines per shared-memory group of the L2-staged tile
    int rawNt;         // threads of the plain L2-staged raw kernel: 0 (512 x 1 CTA/SM) or 256 (x 2)
    // oversampling stage
    int raw;           // rawDataOversamplingFactor
    int deramp;        // derampMethod
    int osL2;          // 1: oversampler chips staged through an L2-resident global slot
    int osGl;          // lines per shared-memory group of the L2-staged oversampler
    int osTc;          // oversampler on tensor cores: 0 off (FFT, FP32), 1 split-BF16 (3 passes), 2 BF16
    int zoom, hz;      // clamped zoom window and half zoom (raw pixels)
    int Hz, Wz;        // zoom-in search chip Wh+2hz, Ww+2hz
    int osWh, osWw;    // oversampled reference raw*Wh, raw*Ww
    int osHz, osWz;    // oversampled search raw*Hz, raw*Wz
    int zp;            // kept oversampled surface 2*hz*raw (last row/col dropped)
    // correlation surface zoom
    int ovs;           // corrSurfaceOverSamplingFactor
    int M;             // zoom*ovs, side of the zoomed surface
    int zs;            // coarse step of the pruned zoom scan (divides M)
    int cosCols;       // persistent kernel: columns per bulk-copied chunk of the
                       // oversampled correlation (0: chunks loaded by the threads)
    int method;        // 0 FFT, 1 sinc
    int cosTc;         // oversampled correlation on tensor cores: 0 off (FP32 FMA), 1 split-BF16, 2 BF16
    int cosTcBg;       // 8-row template groups per streamed band of the tensor-core correlation
    float osratio;     // 1/(ovs*raw) in float
    FftPlan1D fP, fQ;        // raw correlation tile
    FftPlan1D fRefH, fRefW;  // oversampler of the reference chip
    FftPlan1D fSchH, fSchW;  // oversampler of the zoom-in search chip
};

// Small per-window results of the raw stage, written by the raw kernel and
// read by the later stages.
struct RawResult {
    int locX, locY;      // raw arg-max (down, across) = offsetInit before clamping
    int startX, startY;  // clamped zoom-in start (cuDetermineSecondaryExtractOffset)
    int shiftX, shiftY;  // recorded centre shift
    float maxval;
    float snr;
    float covxx, covyy, covxy;
    float refMean;       // mean amplitude of the oversampled reference chip
    float pad;
};

// Per-window pixel coordinates (chip origins in the full images).
struct WindowCoords {
    int refD, refA, secD, secA;
};

}  // namespace ampcor
