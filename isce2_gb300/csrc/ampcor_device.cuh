// Dense amplitude cross-correlation kernels for sm_103a.
//
// One CTA processes one window per stage; the chips are gathered straight
// from the device-resident images (no per-chunk staging copy), every FFT runs
// in shared memory (fft_smem.cuh), and the only HBM intermediates are the
// oversampled amplitude chips and the 2-D oversampled correlation surface.
//
// Stage map to the reference (contrib/PyCuAmpcor/src):
//   k_raw        cuAmpcorChunk.cpp:18-106  (gather, |z|, mean, FFT correlation,
//                normalisation, maxloc, variance, SNR, zoom-start clamp)
//   k_oversample cuAmpcorChunk.cpp:113-137 (deramp, C2C oversampling, |z|)
//   k_corr_os    cuAmpcorChunk.cpp:147-169 (oversampled correlation + normalisation)
//   k_zoom       cuAmpcorChunk.cpp:176-214 (R2R surface oversampling, maxloc,
//                sub-pixel offset, insert)
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <cuda.h>

#include <algorithm>
#include <string>
#include <vector>

#include "ampcor_plan.h"
#include "ampcor_kernels.h"
#include "umma.cuh"

namespace ampcor {

#define FULLMASK 0xffffffffu

__device__ __forceinline__ float amp(cfloat z) { return sqrtf(z.x * z.x + z.y * z.y); }
__device__ __forceinline__ float amp2(float2 z) { return sqrtf(z.x * z.x + z.y * z.y); }

__device__ __forceinline__ cfloat ld_c(const cfloat* p) {
    float2 v = __ldg(reinterpret_cast<const float2*>(p));
    return {v.x, v.y};
}

__device__ inline double block_sum(double v, double* red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULLMASK, v, o);
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (wid == 0) {
        double t = lane < nw ? red[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(FULLMASK, t, o);
        if (lane == 0) red[32] = t;
    }
    __syncthreads();
    return red[32];
}

// Block-strided gather with U elements per thread in flight: load(t) runs for
// t = t0, t0 + nt, ... (U of them, t < n) before store(t, value) consumes them
// in the same order.  A plain strided loop issues one dependent global load
// per iteration and leaves the SM idle for the load latency; the per-thread
// element order (and so any accumulation inside store) is unchanged.
// S2 - S1^2 / n of a box (the NCC denominator's search term) with the
// subtraction in FP64: the box sums are exact float sums of non-negative
// terms, and the difference cancels where the box is nearly uniform
// (cuCorrNormalization.cu:290-311 forms it in float).
__device__ __forceinline__ float var_fp64(float s1, float s2, double invn) {
    const double a = (double)s1;
    return (float)((double)s2 - a * a * invn);
}

template <int U, typename T, typename L, typename S>
__device__ __forceinline__ void block_gather(int n, L load, S store) {
    const int nt = blockDim.x;
    for (int t0 = threadIdx.x; t0 < n; t0 += U * nt) {
        T v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int t = t0 + u * nt;
            if (t < n) v[u] = load(t);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int t = t0 + u * nt;
            if (t < n) store(t, v[u]);
        }
    }
}

// One complex sample copied global -> shared without passing through
// registers (cp.async, 8 bytes; both addresses 8-byte aligned), and the wait
// for every copy this thread issued.
__device__ __forceinline__ void cp_async_c(cfloat* dst, const cfloat* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(umma::smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Arg-max order of cudaKernel_maxloc2D<512> (cuOffset.cu:23-84): larger value
// wins; among equal values the one whose idx%512 has the smaller 9-bit
// bit-reversal wins (the tree reduction keeps the lower slot on ties), then
// the smaller idx (each thread keeps its first strictly larger value).
__device__ __forceinline__ unsigned tie_key(int idx) { return __brev((unsigned)(idx & 511)) >> 23; }

__device__ __forceinline__ bool better(float av, int ai, float bv, int bi) {
    if (bi < 0) return ai >= 0;
    if (ai < 0) return false;
    if (av > bv) return true;
    if (av < bv) return false;
    unsigned ka = tie_key(ai), kb = tie_key(bi);
    return ka < kb || (ka == kb && ai < bi);
}

// block-wide arg-max; idx < 0 marks "no candidate"
__device__ inline void block_argmax(float& v, int& idx, float* redv, int* redi) {
    for (int o = 16; o > 0; o >>= 1) {
        float ov = __shfl_xor_sync(FULLMASK, v, o);
        int oi = __shfl_xor_sync(FULLMASK, idx, o);
        if (better(ov, oi, v, idx)) { v = ov; idx = oi; }
    }
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if (lane == 0) { redv[wid] = v; redi[wid] = idx; }
    __syncthreads();
    if (wid == 0) {
        float tv = lane < nw ? redv[lane] : -INFINITY;
        int ti = lane < nw ? redi[lane] : -1;
        for (int o = 16; o > 0; o >>= 1) {
            float ov = __shfl_xor_sync(FULLMASK, tv, o);
            int oi = __shfl_xor_sync(FULLMASK, ti, o);
            if (better(ov, oi, tv, ti)) { tv = ov; ti = oi; }
        }
        if (lane == 0) { redv[32] = tv; redi[32] = ti; }
    }
    __syncthreads();
    v = redv[32];
    idx = redi[32];
}

// Exact window sums along one line for the lags v0 .. v0+G-1 (G <= 32, G <=
// Wn), computed by one warp: lane l < G returns the sums of both components of
// x(j) over j in [v0+l, v0+l+Wn).  Each sum is split into a core common to
// the group, [v0+G-1, v0+Wn-1], a head [v0+l, v0+G-2] and a tail
// [v0+Wn, v0+l+Wn-1]; every partial sum adds non-negative terms lying inside
// the window, so no value outside a window can cancel into it (a bright
// target next to a dark window does not leak).
template <typename F>
__device__ __forceinline__ float2 warp_box_group(F x, int Wn, int v0, int G) {
    const int lane = threadIdx.x & 31;
    float c1 = 0.f, c2 = 0.f;
    // the core, kPre loads per lane issued before they are summed (so that
    // their latencies overlap), in the same order as a plain loop
    constexpr int kPre = 8;
    const int jend = v0 + Wn - 1;
    int j = v0 + G - 1 + lane;
    for (; j + 32 * (kPre - 1) <= jend; j += 32 * kPre) {
        float2 a[kPre];
#pragma unroll
        for (int k = 0; k < kPre; ++k) a[k] = x(j + 32 * k);
#pragma unroll
        for (int k = 0; k < kPre; ++k) {
            c1 += a[k].x;
            c2 += a[k].y;
        }
    }
    {
        float2 a[kPre];
#pragma unroll
        for (int k = 0; k < kPre; ++k) a[k] = j + 32 * k <= jend ? x(j + 32 * k) : make_float2(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < kPre; ++k)
            if (j + 32 * k <= jend) {
                c1 += a[k].x;
                c2 += a[k].y;
            }
    }
    for (int o = 16; o > 0; o >>= 1) {
        c1 += __shfl_xor_sync(FULLMASK, c1, o);
        c2 += __shfl_xor_sync(FULLMASK, c2, o);
    }
    if (G == 1) return make_float2(c1, c2);  // one lag: no head or tail (the scans add zeros)
    float2 h = lane < G - 1 ? x(v0 + lane) : make_float2(0.f, 0.f);
    float2 t = lane < G - 1 ? x(v0 + Wn + lane) : make_float2(0.f, 0.f);
    for (int o = 1; o < 32; o <<= 1) {  // inclusive suffix scan of h
        const float a = __shfl_down_sync(FULLMASK, h.x, o), b = __shfl_down_sync(FULLMASK, h.y, o);
        if (lane + o < 32) { h.x += a; h.y += b; }
    }
    for (int o = 1; o < 32; o <<= 1) {  // inclusive prefix scan of t
        const float a = __shfl_up_sync(FULLMASK, t.x, o), b = __shfl_up_sync(FULLMASK, t.y, o);
        if (lane >= o) { t.x += a; t.y += b; }
    }
    float tx = __shfl_up_sync(FULLMASK, t.x, 1), ty = __shfl_up_sync(FULLMASK, t.y, 1);
    if (lane == 0) { tx = 0.f; ty = 0.f; }
    return make_float2(c1 + (h.x + tx), c2 + (h.y + ty));
}

__host__ __device__ inline size_t align16(size_t b) { return (b + 15) & ~(size_t)15; }

__device__ __forceinline__ int sm_count() {
    uint32_t n;
    asm("mov.u32 %0, %%nsmid;" : "=r"(n));
    return (int)n;
}

// Prefetch into L2 the rows x cols complex64 chip at p (row pitch ld
// elements): one prefetch per 128-byte line, spread over the block.  Used
// for the chips of a window a CTA (or the CTA that follows it on the SM)
// gathers next, so that the gather finds them in L2 instead of HBM.
__device__ __forceinline__ void prefetch_chip_l2(const cfloat* p, long long ld, int rows, int cols) {
    // addresses 128 bytes apart from the row start, then the row's last
    // byte (a row that straddles one more line): every address lies inside
    // the chip
    const int bytes = cols * 8, lines = (bytes + 127) / 128 + 1;
    for (int t = threadIdx.x; t < rows * lines; t += blockDim.x) {
        const int i = t / lines, l = t - (t / lines) * lines;
        const int off = l + 1 < lines ? 128 * l : bytes - 1;
        const char* a = reinterpret_cast<const char*>(p + (long long)i * ld) + off;
        asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
    }
}

// ---------------------------------------------------------------------------
// raw stage
// ---------------------------------------------------------------------------
__host__ __device__ inline int odd_ld(int n) { return n | 1; }

#ifdef AMPCOR_PART_PLAIN
size_t raw_smem_bytes(const WindowPlan& P) {
    return align16((size_t)P.P * odd_ld(P.Q) * sizeof(cfloat)) + align16((size_t)P.NX * P.NY * sizeof(float)) +
           align16((size_t)(P.P + P.Q) * sizeof(cfloat)) + 40 * sizeof(double) + 40 * 8 +
           align16((size_t)(P.P + P.Q) * sizeof(int));
}
#endif

// Arg-max reduction, SNR, covariance and zoom-start clamp of the raw stage
// (cuOffset.cu:23-100, cuEstimateStats.cu:20-128, cuOffset.cu:190-224), from
// the normalised surface rn (NX x NY) and each thread's best candidate.
__device__ __forceinline__ void raw_finish(const WindowPlan& P, const float* rn, float bv, int bi, double* red,
                                           float* redv, int* redi, RawResult* __restrict__ out) {
    const int NX = P.NX, NY = P.NY, Wh = P.Wh, Ww = P.Ww;
    block_argmax(bv, bi, redv, redi);
    if (bi < 0) { bi = 0; bv = -FLT_MAX; }
    const int px = bi / NY, py = bi - (bi / NY) * NY;

    // SNR over the statistics box (cuArraysCopyExtractCorr + cuArraysSumCorr + estimateSnr)
    float sacc = 0.f;
    int cnt = 0;
    for (int t = threadIdx.x; t < P.statH * P.statW; t += blockDim.x) {
        const int ox = t / P.statW, oy = t - (t / P.statW) * P.statW;
        const int ix = ox + px - P.statH / 2, iy = oy + py - P.statW / 2;
        if (ix >= 0 && iy >= 0 && ix < NX && iy < NY) {
            const float c = rn[ix * NY + iy];
            sacc = fmaf(c, c, sacc);
            cnt += 1;
        }
    }
    const double ssum = block_sum((double)sacc, red);
    const double ccnt = block_sum((double)cnt, red);

    if (threadIdx.x == 0) {
        RawResult r;
        r.locX = px;
        r.locY = py;
        r.maxval = bv;
        const double pk = bv;
        const double meanc = (ssum - pk * pk) / (ccnt - 1.0);
        r.snr = (float)(pk * pk / meanc);
        // covariance (cudaKernel_estimateVar, cuEstimateStats.cu:49-128)
        if (px - 1 < 0 || py - 1 < 0 || px + 1 >= NX || py + 1 >= NY) {
            r.covxx = 99.f; r.covyy = 99.f; r.covxy = 0.f;
        } else {
            auto at = [&](int dx, int dy) { return (double)rn[(px + dx) * NY + py + dy]; };
            const double ts = (double)(Wh * Ww);
            double dxx = -(at(1, 0) + at(-1, 0) - 2.0 * at(0, 0)) * ts;
            double dyy = -(at(0, 1) + at(0, -1) - 2.0 * at(0, 0)) * ts;
            double dxy = (at(1, 1) + at(-1, -1) - at(1, -1) - at(-1, 1)) * 0.25 * ts;
            double n2 = fmax(1.0 - pk, 0.0);
            double n4 = n2 * n2 * 0.5 * ts;
            n2 = n2 * 2.0;
            const double u = dxy * dxy - dxx * dyy;
            if (fabs(u) < 1e-2) {
                r.covxx = 99.f; r.covyy = 99.f; r.covxy = 0.f;
            } else {
                const double u2 = u * u;
                r.covxx = (float)((-n2 * u * dyy + n4 * (dyy * dyy + dxy * dxy)) / u2);
                r.covyy = (float)((-n2 * u * dxx + n4 * (dxx * dxx + dxy * dxy)) / u2);
                r.covxy = (float)((n2 * u * dxy - n4 * (dxx + dyy) * dxy) / u2);
            }
        }
        // zoom-in start clamp (dev_adjustOffset, cuOffset.cu:190-224)
        auto clampz = [](int oldR, int newR, int loc, int& start, int& shift) {
            start = loc - newR;
            shift = 0;
            const int rb = 2 * (oldR - newR);
            if (start < 0) { shift = -start; start = 0; }
            else if (start > rb) { shift = start - rb; start = rb; }
        };
        clampz(P.hsD, P.hz, px, r.startX, r.shiftX);
        clampz(P.hsA, P.hz, py, r.startY, r.shiftY);
        r.refMean = 0.f;
        r.pad = 0.f;
        *out = r;
    }
}

// Raw stage of one window (the whole CTA): results to *out, box-sum scratch V.
// GU: chip loads in flight per thread (block_gather); `k_raw` takes 4.  The
// multi-window kernels (wave, fused) take GU = 0: there the deeper register
// gather spills (their plan fields live in registers), so the search chip is
// copied into the tile by cp.async, which holds no registers, and the
// reference chip is gathered one load deep.  GU = 1 is the plain loop.
template <int GU = 1>
__device__ __forceinline__ void raw_body(const WindowPlan& P, unsigned char* smem, const cfloat* __restrict__ ref,
                                         long long ldr, const cfloat* __restrict__ sec, long long lds,
                                         const WindowCoords wc, float2* __restrict__ V, RawResult* __restrict__ out) {
    const int Wh = P.Wh, Ww = P.Ww, Hs = P.Hs, Ws = P.Ws, NX = P.NX, NY = P.NY, PP = P.P, QQ = P.Q;
    const int LD = odd_ld(QQ);  // odd row pitch (in cfloat) keeps every FFT pass free of bank conflicts
    cfloat* buf = reinterpret_cast<cfloat*>(smem);
    float* rn = reinterpret_cast<float*>(smem + align16((size_t)PP * LD * sizeof(cfloat)));
    cfloat* twP = reinterpret_cast<cfloat*>(reinterpret_cast<unsigned char*>(rn) + align16((size_t)NX * NY * 4));
    cfloat* twQ = twP + PP;
    double* red = reinterpret_cast<double*>(reinterpret_cast<unsigned char*>(twP) + align16((size_t)(PP + QQ) * 8));
    float* redv = reinterpret_cast<float*>(red + 40);
    int* redi = reinterpret_cast<int*>(redv + 40);
    int* partP = redi + 40;   // position of the conjugate frequency, per axis
    int* partQ = partP + PP;
    const FastDiv dQ(QQ), dNY(NY), dWw(Ww), dHs(Hs), dNX(NX), dWs(Ws);

    const cfloat* rp = ref + (long long)wc.refD * ldr + wc.refA;
    const cfloat* sp = sec + (long long)wc.secD * lds + wc.secA;

    if constexpr (GU == 0) {
        for (int t = threadIdx.x; t < Hs * Ws; t += blockDim.x) {
            const int i = (int)dWs.div(t), j = t - i * Ws;
            cp_async_c(buf + i * LD + j, sp + (long long)i * lds + j);
        }
        cp_async_wait_all();
        __syncthreads();
    }

    // packed real pair z = t + i s on the padded P x LD tile; R2 = sum t^2
    block_fill_roots(twP, PP);
    block_fill_roots(twQ, QQ);
    for (int t = threadIdx.x; t < PP; t += blockDim.x) {
        const int f = fft_pos_to_freq(P.fP, t);
        partP[t] = fft_freq_to_pos(P.fP, f ? PP - f : 0);
    }
    for (int t = threadIdx.x; t < QQ; t += blockDim.x) {
        const int f = fft_pos_to_freq(P.fQ, t);
        partQ[t] = fft_freq_to_pos(P.fQ, f ? QQ - f : 0);
    }
    // packed real pair z = t + i s on the padded P x LD tile, t still
    // without its mean; the reference chip is read once
    float part = 0.f;
    if constexpr (GU == 0) {
        for (int t = threadIdx.x; t < PP * QQ; t += blockDim.x) {
            const int i = (int)dQ.div(t), j = t - i * QQ;
            float tv = 0.f, sv = 0.f;
            if (i < Wh && j < Ww) {
                tv = amp(ld_c(rp + (long long)i * ldr + j));
                part += tv;
            }
            if (i < Hs && j < Ws) sv = amp(buf[i * LD + j]);
            buf[i * LD + j] = {tv, sv};
        }
    } else if constexpr (GU == 1) {
        for (int t = threadIdx.x; t < PP * QQ; t += blockDim.x) {
            const int i = (int)dQ.div(t), j = t - i * QQ;
            float tv = 0.f, sv = 0.f;
            if (i < Wh && j < Ww) {
                tv = amp(ld_c(rp + (long long)i * ldr + j));
                part += tv;
            }
            if (i < Hs && j < Ws) sv = amp(ld_c(sp + (long long)i * lds + j));
            buf[i * LD + j] = {tv, sv};
        }
    } else {
        block_gather<GU, float4>(
            PP * QQ,
            [&](int t) {
                const int i = (int)dQ.div(t), j = t - i * QQ;
                cfloat a = {0.f, 0.f}, b = {0.f, 0.f};
                if (i < Wh && j < Ww) a = ld_c(rp + (long long)i * ldr + j);
                if (i < Hs && j < Ws) b = ld_c(sp + (long long)i * lds + j);
                return make_float4(a.x, a.y, b.x, b.y);
            },
            [&](int t, float4 v) {
                const int i = (int)dQ.div(t), j = t - i * QQ;
                float tv = 0.f, sv = 0.f;
                if (i < Wh && j < Ww) {
                    tv = amp(cfloat{v.x, v.y});
                    part += tv;
                }
                if (i < Hs && j < Ws) sv = amp(cfloat{v.z, v.w});
                buf[i * LD + j] = {tv, sv};
            });
    }
    // reference mean (cuArraysSubtractMean, cuCorrNormalization.cu:98-123),
    // removed in place; R2 = sum t^2
    const float mean = (float)(block_sum((double)part, red) / (double)(Wh * Ww));  // also a barrier
    float r2part = 0.f;
    for (int t = threadIdx.x; t < Wh * Ww; t += blockDim.x) {
        const int i = (int)dWw.div(t), j = t - i * Ww;
        const float tv = buf[i * LD + j].x - mean;
        buf[i * LD + j].x = tv;
        r2part = fmaf(tv, tv, r2part);
    }
    const float R2 = (float)block_sum((double)r2part, red);  // also a barrier

    // box sums S1, S2 of the search amplitude for every lag: column sums over
    // the template height (into the per-window scratch V), then row sums of V
    {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
        const int Gv = min(32, Wh), ngv = (NX + Gv - 1) / Gv;
        for (int task = warp; task < Ws * ngv; task += nwarp) {
            const int g = task / Ws, j = task - g * Ws, v0 = g * Gv, G = min(Gv, NX - v0);
            const float2 r = warp_box_group([&](int i) {
                const float a = buf[i * LD + j].y;
                return make_float2(a, a * a);
            }, Wh, v0, G);
            if (lane < G) V[(size_t)(v0 + lane) * Ws + j] = r;
        }
        __syncthreads();
        const double invnd = 1.0 / (double)(Wh * Ww);
        const int Gh = min(32, Ww), ngh = (NY + Gh - 1) / Gh;
        for (int task = warp; task < NX * ngh; task += nwarp) {
            const int u = task / ngh, g = task - u * ngh, v0 = g * Gh, G = min(Gh, NY - v0);
            const float2* row = V + (size_t)u * Ws;
            const float2 r = warp_box_group([&](int j) { return row[j]; }, Ww, v0, G);
            if (lane < G) rn[u * NY + v0 + lane] = var_fp64(r.x, r.y, invnd);
        }
        __syncthreads();
    }

    // forward transforms (rows holding data, then every column)
    block_fft_lines(true, P.fQ, buf, dHs, LD, 1, true, twQ, -1);
    block_fft_lines(true, P.fP, buf, dQ, 1, LD, true, twP, -1);
    // conj(T) * S, separating the two real spectra through Z(f) and Z(-f)
    for (int t = threadIdx.x; t < PP * QQ; t += blockDim.x) {
        const int p1 = (int)dQ.div(t), p2 = t - p1 * QQ;
        const int t2 = partP[p1] * QQ + partQ[p2];
        if (t2 < t) continue;
        const int a1 = p1 * LD + p2, a2 = partP[p1] * LD + partQ[p2];
        const cfloat Z1 = buf[a1], Z2 = buf[a2];
        const cfloat T = {0.5f * (Z1.x + Z2.x), 0.5f * (Z1.y - Z2.y)};
        const cfloat D = {0.5f * (Z1.x - Z2.x), 0.5f * (Z1.y + Z2.y)};
        const cfloat S = {D.y, -D.x};
        const cfloat C = cmul(cconj(T), S);
        buf[a1] = C;
        if (t2 != t) buf[a2] = cconj(C);
    }
    __syncthreads();
    block_fft_lines(false, P.fP, buf, dQ, 1, LD, true, twP, +1);
    block_fft_lines(false, P.fQ, buf, dNX, LD, 1, true, twQ, +1);

    // normalised correlation (cuCorrNormalize_kernel, :286-312) and arg-max
    const float scale = 1.0f / ((float)PP * (float)QQ);
    float bv = -INFINITY;
    int bi = -1;
    for (int t = threadIdx.x; t < NX * NY; t += blockDim.x) {
        const int u = (int)dNY.div(t), v = t - u * NY;
        const float c = buf[u * LD + v].x * scale;
        const float norm2 = rn[t] * R2;
        const float val = c / sqrtf(norm2 + FLT_EPSILON);
        rn[t] = val;
        if (!isnan(val) && better(val, t, bv, bi)) { bv = val; bi = t; }
    }
    raw_finish(P, rn, bv, bi, red, redv, redi, out);
}

#ifdef AMPCOR_PART_PLAIN
__global__ void __launch_bounds__(512) k_raw(const __grid_constant__ WindowPlan P, const cfloat* __restrict__ ref, long long ldr,
                                             const cfloat* __restrict__ sec, long long lds,
                                             const WindowCoords* __restrict__ coords, int w0, int wend,
                                             RawResult* __restrict__ res, float2* __restrict__ vbox) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int w = w0 + blockIdx.x;
    if (w >= wend) return;
    // the window the CTA that follows this one on the SM will gather (CTAs
    // start in index order, one per SM at this kernel's shared memory)
    const int wn = w + sm_count();
    if (wn < wend) {
        const WindowCoords c = coords[wn];
        prefetch_chip_l2(ref + (long long)c.refD * ldr + c.refA, ldr, P.Wh, P.Ww);
        prefetch_chip_l2(sec + (long long)c.secD * lds + c.secA, lds, P.Hs, P.Ws);
    }
    raw_body<4>(P, smem, ref, ldr, sec, lds, coords[w], vbox + (size_t)(w - w0) * P.NX * P.Ws, &res[w]);
}
#endif

// ---------------------------------------------------------------------------
// raw stage with the FFT tile in an L2-resident global slot
// ---------------------------------------------------------------------------
// For search chips whose P x Q tile does not fit in shared memory (a 256 x 256
// window with a +-48 search needs a 352 x 352 tile, ~1 MB).  The same 1-D
// transforms as raw_body run on groups of rawGl lines staged through shared
// memory; between the passes the tile sits column-major in the CTA's slot
// (T[q*P + i]), so every slot access moves runs of consecutive elements:
//   1. rows 0..Hs-1: build z = t + i s, forward row FFT, store columns;
//   2. column groups closed under f -> -f (a frequency and its conjugate sit
//      side by side in the group order): forward column FFT, conj(T) S,
//      inverse column FFT, store the first NX rows;
//   3. rows 0..NX-1: inverse row FFT, normalise, arg-max.
// Each line sees exactly the arithmetic of raw_body, so both paths give
// bit-identical surfaces.  The search amplitude is also kept column-major
// (A[j*Hs + i]) for the box sums of the normalisation.
#ifdef AMPCOR_PART_PLAIN
size_t raw_l2_smem_bytes(const WindowPlan& P) {
    const size_t lines = (size_t)P.rawGl * odd_ld(std::max(P.P, P.Q)) * sizeof(cfloat);
    return align16(lines) + align16((size_t)P.NX * P.NY * sizeof(float)) +
           align16((size_t)(P.P + P.Q) * sizeof(cfloat)) + 40 * sizeof(double) + 40 * 8 +
           align16((size_t)(P.P + P.Q) * sizeof(int));
}
#endif

// Global slot bytes of one window: tile, column-major amplitude, box sums.
#ifdef AMPCOR_PART_PLAIN
size_t raw_l2_slot_bytes(const WindowPlan& P) {
    auto a256 = [](size_t b) { return (b + 255) & ~(size_t)255; };
    return a256((size_t)P.P * P.Q * sizeof(cfloat)) + a256((size_t)P.Hs * P.Ws * sizeof(float)) +
           a256((size_t)P.NX * P.Ws * sizeof(float2));
}
#endif

__device__ __forceinline__ void raw_l2_body(const WindowPlan& P, unsigned char* smem, const cfloat* __restrict__ ref,
                                            long long ldr, const cfloat* __restrict__ sec, long long lds,
                                            const WindowCoords wc, unsigned char* __restrict__ slot,
                                            RawResult* __restrict__ out) {
    const int Wh = P.Wh, Ww = P.Ww, Hs = P.Hs, Ws = P.Ws, NX = P.NX, NY = P.NY, PP = P.P, QQ = P.Q;
    const int Gl = P.rawGl;
    const int LDL = odd_ld(max(PP, QQ));
    const int tid = threadIdx.x, nt = blockDim.x;
    cfloat* buf = reinterpret_cast<cfloat*>(smem);
    float* rn = reinterpret_cast<float*>(smem + align16((size_t)Gl * LDL * sizeof(cfloat)));
    cfloat* twP = reinterpret_cast<cfloat*>(reinterpret_cast<unsigned char*>(rn) + align16((size_t)NX * NY * 4));
    cfloat* twQ = twP + PP;
    double* red = reinterpret_cast<double*>(reinterpret_cast<unsigned char*>(twP) + align16((size_t)(PP + QQ) * 8));
    float* redv = reinterpret_cast<float*>(red + 40);
    int* redi = reinterpret_cast<int*>(redv + 40);
    int* partP = redi + 40;  // position of the conjugate row frequency
    int* colOrd = partP + PP;  // column positions in conjugate-pair order
    const size_t tOff = ((size_t)PP * QQ * sizeof(cfloat) + 255) & ~(size_t)255;
    const size_t aOff = tOff + (((size_t)Hs * Ws * sizeof(float) + 255) & ~(size_t)255);
    cfloat* T = reinterpret_cast<cfloat*>(slot);
    float* A = reinterpret_cast<float*>(slot + tOff);
    float2* V = reinterpret_cast<float2*>(slot + aOff);
    const FastDiv dQ(QQ), dP(PP), dNY(NY), dWw(Ww);

    const cfloat* rp = ref + (long long)wc.refD * ldr + wc.refA;
    const cfloat* sp = sec + (long long)wc.secD * lds + wc.secA;

    // the reference mean and R2 with raw_body's element-to-thread order, so
    // that both give the same bits
    float part = 0.f;
    for (int t = tid; t < PP * QQ; t += nt) {
        const int i = (int)dQ.div(t), j = t - i * QQ;
        if (i < Wh && j < Ww) part += amp(ld_c(rp + (long long)i * ldr + j));
    }
    const float mean = (float)(block_sum((double)part, red) / (double)(Wh * Ww));
    float r2part = 0.f;
    for (int t = tid; t < Wh * Ww; t += nt) {
        const int i = (int)dWw.div(t), j = t - i * Ww;
        const float tv = amp(ld_c(rp + (long long)i * ldr + j)) - mean;
        r2part = fmaf(tv, tv, r2part);
    }

    block_fill_roots(twP, PP);
    block_fill_roots(twQ, QQ);
    for (int t = tid; t < PP; t += nt) {
        const int f = fft_pos_to_freq(P.fP, t);
        partP[t] = fft_freq_to_pos(P.fP, f ? PP - f : 0);
    }
    const int npair = (QQ - 1) / 2;
    for (int q = tid; q < QQ; q += nt) {
        const int f = fft_pos_to_freq(P.fQ, q);
        int k;
        if (f == 0) k = 2 * npair;
        else if (2 * f == QQ) k = 2 * npair + 1;
        else if (f < QQ - f) k = 2 * (f - 1);
        else k = 2 * (QQ - f - 1) + 1;
        colOrd[k] = q;
    }

    // 1. forward row transforms of rows 0..Hs-1
    for (int i0 = 0; i0 < Hs; i0 += Gl) {
        const int nr = min(Gl, Hs - i0);
        const FastDiv dn(nr);
        for (int t = tid; t < nr * QQ; t += nt) {
            const int r = (int)dQ.div(t), j = t - r * QQ, i = i0 + r;
            float tv = 0.f, sv = 0.f;
            if (i < Wh && j < Ww) tv = amp(ld_c(rp + (long long)i * ldr + j)) - mean;
            if (j < Ws) sv = amp(ld_c(sp + (long long)i * lds + j));
            buf[r * LDL + j] = {tv, sv};
        }
        __syncthreads();
        for (int t = tid; t < nr * Ws; t += nt) {
            const int j = (int)dn.div(t), r = t - j * nr;
            A[(size_t)j * Hs + i0 + r] = buf[r * LDL + j].y;
        }
        __syncthreads();
        block_fft_lines(true, P.fQ, buf, dn, LDL, 1, true, twQ, -1);
        for (int t = tid; t < nr * QQ; t += nt) {
            const int q = (int)dn.div(t), r = t - q * nr;
            T[(size_t)q * PP + i0 + r] = buf[r * LDL + q];
        }
        __syncthreads();
    }
    const float R2 = (float)block_sum((double)r2part, red);

    // box sums S1, S2 of the search amplitude (as raw_body, from A)
    {
        const int lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
        const int Gv = min(32, Wh), ngv = (NX + Gv - 1) / Gv;
        for (int task = warp; task < Ws * ngv; task += nwarp) {
            const int g = task / Ws, j = task - g * Ws, v0 = g * Gv, G = min(Gv, NX - v0);
            const float* col = A + (size_t)j * Hs;
            const float2 r = warp_box_group([&](int i) {
                const float a = col[i];
                return make_float2(a, a * a);
            }, Wh, v0, G);
            if (lane < G) V[(size_t)(v0 + lane) * Ws + j] = r;
        }
        __syncthreads();
        const double invnd = 1.0 / (double)(Wh * Ww);
        const int Gh = min(32, Ww), ngh = (NY + Gh - 1) / Gh;
        for (int task = warp; task < NX * ngh; task += nwarp) {
            const int u = task / ngh, g = task - u * ngh, v0 = g * Gh, G = min(Gh, NY - v0);
            const float2* row = V + (size_t)u * Ws;
            const float2 r = warp_box_group([&](int j) { return row[j]; }, Ww, v0, G);
            if (lane < G) rn[u * NY + v0 + lane] = var_fp64(r.x, r.y, invnd);
        }
        __syncthreads();
    }

    // 2. column groups: forward transform, conj(T) * S, inverse transform
    for (int c0 = 0; c0 < QQ; c0 += Gl) {
        const int nc = min(Gl, QQ - c0);
        const FastDiv dn(nc);
        for (int t = tid; t < nc * PP; t += nt) {
            const int k = (int)dP.div(t), i = t - k * PP;
            buf[k * LDL + i] = i < Hs ? T[(size_t)colOrd[c0 + k] * PP + i] : cfloat{0.f, 0.f};
        }
        __syncthreads();
        block_fft_lines(true, P.fP, buf, dn, LDL, 1, true, twP, -1);
        for (int t = tid; t < nc * PP; t += nt) {
            const int k = (int)dP.div(t), p1 = t - k * PP;
            const int kl = c0 + k, k2 = (kl < 2 * npair ? (kl ^ 1) : kl) - c0, p2 = partP[p1];
            const int t2 = k2 * PP + p2;
            if (t2 < t) continue;
            const int a1 = k * LDL + p1, a2 = k2 * LDL + p2;
            const cfloat Z1 = buf[a1], Z2 = buf[a2];
            const cfloat Tv = {0.5f * (Z1.x + Z2.x), 0.5f * (Z1.y - Z2.y)};
            const cfloat D = {0.5f * (Z1.x - Z2.x), 0.5f * (Z1.y + Z2.y)};
            const cfloat S = {D.y, -D.x};
            const cfloat C = cmul(cconj(Tv), S);
            buf[a1] = C;
            if (t2 != t) buf[a2] = cconj(C);
        }
        __syncthreads();
        block_fft_lines(false, P.fP, buf, dn, LDL, 1, true, twP, +1);
        for (int t = tid; t < nc * NX; t += nt) {
            const int k = t / NX, u = t - k * NX;
            T[(size_t)colOrd[c0 + k] * PP + u] = buf[k * LDL + u];
        }
        __syncthreads();
    }

    // 3. inverse row transforms of rows 0..NX-1, normalisation, arg-max
    const float scale = 1.0f / ((float)PP * (float)QQ);
    float bv = -INFINITY;
    int bi = -1;
    for (int u0 = 0; u0 < NX; u0 += Gl) {
        const int nr = min(Gl, NX - u0);
        const FastDiv dn(nr);
        for (int t = tid; t < nr * QQ; t += nt) {
            const int q = (int)dn.div(t), r = t - q * nr;
            buf[r * LDL + q] = T[(size_t)q * PP + u0 + r];
        }
        __syncthreads();
        block_fft_lines(false, P.fQ, buf, dn, LDL, 1, true, twQ, +1);
        for (int t = tid; t < nr * NY; t += nt) {
            const int r = (int)dNY.div(t), v = t - r * NY, idx = (u0 + r) * NY + v;
            const float c = buf[r * LDL + v].x * scale;
            const float norm2 = rn[idx] * R2;
            const float val = c / sqrtf(norm2 + FLT_EPSILON);
            rn[idx] = val;
            if (!isnan(val) && better(val, idx, bv, bi)) { bv = val; bi = idx; }
        }
        __syncthreads();
    }
    raw_finish(P, rn, bv, bi, red, redv, redi, out);
}

// Plain-path launch: a grid of `gridDim.x` CTAs, each looping over windows
// with its own global slot (slot_bytes apart), so the slots stay in L2.
#ifdef AMPCOR_PART_PLAIN
template <int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) k_raw_l2(const __grid_constant__ WindowPlan P, const cfloat* __restrict__ ref,
                                                     long long ldr, const cfloat* __restrict__ sec, long long lds,
                                                     const WindowCoords* __restrict__ coords, int w0, int wend,
                                                     RawResult* __restrict__ res, unsigned char* __restrict__ slots,
                                                     size_t slot_bytes) {
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned char* slot = slots + (size_t)blockIdx.x * slot_bytes;
    for (int w = w0 + blockIdx.x; w < wend; w += gridDim.x) {
        raw_l2_body(P, smem, ref, ldr, sec, lds, coords[w], slot, &res[w]);
        __syncthreads();
    }
}
#endif
#ifdef AMPCOR_PART_PLAIN
// The L2-staged raw stage at 512 threads x 1 CTA per SM (P.rawNt 0) or 256
// threads x 2 CTAs per SM (P.rawNt 256, shared line groups of 16).
static const void* raw_l2_fn(const WindowPlan& P) {
    return P.rawNt == 256 ? (const void*)k_raw_l2<256, 2> : (const void*)k_raw_l2<512, 1>;
}

int raw_l2_threads(const WindowPlan& P) { return P.rawNt == 256 ? 256 : 512; }

int raw_l2_blocks_per_sm(const WindowPlan& P) {
    int n = 0;
    const size_t sm = raw_l2_smem_bytes(P);
    if (cudaFuncSetAttribute(raw_l2_fn(P), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
        return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, raw_l2_fn(P), raw_l2_threads(P), sm) != cudaSuccess)
        return 0;
    return n;
}

cudaError_t launch_raw_l2(const WindowPlan& P, int grid, cudaStream_t st, const cfloat* ref, long long ldr,
                          const cfloat* sec, long long lds, const WindowCoords* coords, int w0, int wend,
                          RawResult* res, unsigned char* slots, size_t slot_bytes) {
    const size_t sm = raw_l2_smem_bytes(P);
    cudaError_t e = cudaFuncSetAttribute(raw_l2_fn(P), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    if (P.rawNt == 256)
        k_raw_l2<256, 2><<<grid, 256, sm, st>>>(P, ref, ldr, sec, lds, coords, w0, wend, res, slots, slot_bytes);
    else
        k_raw_l2<512, 1><<<grid, 512, sm, st>>>(P, ref, ldr, sec, lds, coords, w0, wend, res, slots, slot_bytes);
    return cudaGetLastError();
}
#endif

// ---------------------------------------------------------------------------
// oversampling stage: blockIdx.y = 0 reference chip, 1 zoom-in search chip
// ---------------------------------------------------------------------------
#ifdef AMPCOR_PART_PLAIN
size_t os_smem_bytes(const WindowPlan& P) {
    const int a = P.Wh * odd_ld(P.Ww), b = P.Hz * odd_ld(P.Wz);
    const int n = a > b ? a : b;
    const int l = (P.Wh + P.Ww) > (P.Hz + P.Wz) ? (P.Wh + P.Ww) : (P.Hz + P.Wz);
    return 2 * align16((size_t)n * sizeof(cfloat)) + 2 * align16((size_t)l * sizeof(cfloat)) + 40 * sizeof(double);
}
#endif

// Oversampling of one chip (which = 0 reference, 1 zoom-in search chip) into
// `out` (raw N1 x raw N2 amplitudes); the reference mean goes to rw->refMean.
// GU: chip loads in flight per thread, as raw_body (0: cp.async copies, used
// by every kernel)
template <int GU = 1>
__device__ __forceinline__ void os_body(const WindowPlan& P, unsigned char* smem, int which,
                                        const cfloat* __restrict__ ref, long long ldr,
                                        const cfloat* __restrict__ sec, long long lds, const WindowCoords wc,
                                        RawResult* __restrict__ rw, float* __restrict__ out) {
    const int N1 = which ? P.Hz : P.Wh, N2 = which ? P.Wz : P.Ww;
    const FftPlan1D& fH = which ? P.fSchH : P.fRefH;
    const FftPlan1D& fW = which ? P.fSchW : P.fRefW;
    const int n = N1 * N2;
    const int LD = odd_ld(N2);
    const int a0 = P.Wh * odd_ld(P.Ww), b0 = P.Hz * odd_ld(P.Wz);
    const int nmax = a0 > b0 ? a0 : b0;
    cfloat* X = reinterpret_cast<cfloat*>(smem);
    cfloat* Wk = reinterpret_cast<cfloat*>(smem + align16((size_t)nmax * sizeof(cfloat)));
    cfloat* tw1 = reinterpret_cast<cfloat*>(smem + 2 * align16((size_t)nmax * sizeof(cfloat)));
    cfloat* tw2 = tw1 + N1;
    const int lmax = (P.Wh + P.Ww) > (P.Hz + P.Wz) ? (P.Wh + P.Ww) : (P.Hz + P.Wz);
    cfloat* ph1 = reinterpret_cast<cfloat*>(reinterpret_cast<unsigned char*>(tw1) + align16((size_t)lmax * 8));
    cfloat* ph2 = ph1 + N1;
    double* red = reinterpret_cast<double*>(reinterpret_cast<unsigned char*>(ph1) + align16((size_t)lmax * 8));
    const FastDiv dN2(N2), dN1(N1);

    const cfloat* src;
    long long ld;
    if (which) {
        const RawResult r = *rw;
        src = sec + (long long)(wc.secD + r.startX) * lds + (wc.secA + r.startY);
        ld = lds;
    } else {
        src = ref + (long long)wc.refD * ldr + wc.refA;
        ld = ldr;
    }
    block_fill_roots(tw1, N1);
    block_fill_roots(tw2, N2);
    // chip: (|z|, 0) when derampMethod == 0 (cuArraysCopyToBatchAbsWithOffset), complex otherwise
    if constexpr (GU == 0) {
        for (int t = threadIdx.x; t < n; t += blockDim.x) {
            const int i = (int)dN2.div(t), j = t - i * N2;
            cp_async_c(X + i * LD + j, src + (long long)i * ld + j);
        }
        cp_async_wait_all();
        if (P.deramp == 0) {  // each thread converts the samples it copied
            for (int t = threadIdx.x; t < n; t += blockDim.x) {
                const int i = (int)dN2.div(t), j = t - i * N2;
                X[i * LD + j] = cfloat{amp(X[i * LD + j]), 0.f};
            }
        }
    } else if constexpr (GU == 1) {
        for (int t = threadIdx.x; t < n; t += blockDim.x) {
            const int i = (int)dN2.div(t), j = t - i * N2;
            const cfloat z = ld_c(src + (long long)i * ld + j);
            X[i * LD + j] = P.deramp == 0 ? cfloat{amp(z), 0.f} : z;
        }
    } else {
        block_gather<GU, cfloat>(
            n,
            [&](int t) {
                const int i = (int)dN2.div(t), j = t - i * N2;
                return ld_c(src + (long long)i * ld + j);
            },
            [&](int t, cfloat z) {
                const int i = (int)dN2.div(t), j = t - i * N2;
                X[i * LD + j] = P.deramp == 0 ? cfloat{amp(z), 0.f} : z;
            });
    }
    __syncthreads();
    if (P.deramp == 1) {
        // cuDerampMethod1_kernel (cuDeramp.cu:67-114), quirks: the row-derived
        // phase multiplies the column index and vice versa; the product uses
        // the updated real part (float2.h operator*=).
        float yr = 0.f, yi = 0.f, xr = 0.f, xi = 0.f;  // per-thread partials, combined in double
        for (int t = threadIdx.x; t < n; t += blockDim.x) {
            const int i = (int)dN2.div(t), j = t - i * N2;
            const cfloat a = X[i * LD + j];
            if (j < N2 - 1) {
                const cfloat b = X[i * LD + j + 1];
                yr = fmaf(a.x, b.x, fmaf(a.y, b.y, yr));
                yi = fmaf(a.y, b.x, fmaf(-a.x, b.y, yi));
            }
            if (i < N1 - 1) {
                const cfloat b = X[(i + 1) * LD + j];
                xr = fmaf(a.x, b.x, fmaf(a.y, b.y, xr));
                xi = fmaf(a.y, b.x, fmaf(-a.x, b.y, xi));
            }
        }
        const double dyr = block_sum((double)yr, red);
        const double dyi = block_sum((double)yi, red);
        const double dxr = block_sum((double)xr, red);
        const double dxi = block_sum((double)xi, red);
        const float phaseY = atan2f((float)dyi, (float)dyr);
        const float phaseX = atan2f((float)dxi, (float)dxr);
        for (int t = threadIdx.x; t < n; t += blockDim.x) {
            const int row = (int)dN2.div(t), col = t - row * N2;
            const float ph = (float)col * phaseX + (float)row * phaseY;
            float s, c;
            sincosf(ph, &s, &c);
            cfloat z = X[row * LD + col];
            const float nr = z.x * c - z.y * s;
            const float ni = z.y * c + nr * s;
            X[row * LD + col] = {nr, ni};
        }
        __syncthreads();
    }
    const int raw = P.raw, outW = raw * N2;
    const int h1 = N1 / 2, h2 = N2 / 2;
    const float inv = 1.0f / ((float)N1 * (float)N2);
    float asum = 0.f;
    // For even lengths the spectral zero-padding keeps every input sample
    // exactly: plane (0,0) of the output is the chip itself.
    const bool identity00 = (N1 % 2 == 0) && (N2 % 2 == 0);
    if (identity00) {
        for (int t = threadIdx.x; t < n; t += blockDim.x) {
            const int p = (int)dN2.div(t), q = t - p * N2;
            const float m = amp(X[p * LD + q]);
            out[(size_t)(raw * p) * outW + raw * q] = m;
            asum += m;
        }
        __syncthreads();
    }
    // X~ = unnormalised inverse-sign DFT (cufftExecC2C INVERSE), digit-reversed
    block_fft_lines(true, fW, X, dN1, LD, 1, true, tw2, +1);
    block_fft_lines(true, fH, X, dN2, 1, LD, true, tw1, +1);

    for (int a = 0; a < raw; ++a) {
        for (int b = 0; b < raw; ++b) {
            if (identity00 && a == 0 && b == 0) continue;
            // one polyphase plane of the zero-padded spectrum (cuArraysPaddingMany):
            // per-axis factor e^{-2 pi i a f/(raw N)} for kept signed
            // frequencies f, zero for the middle index an odd length drops
            for (int t = threadIdx.x; t < N1 + N2; t += blockDim.x) {
                const bool first = t < N1;
                const int pos = first ? t : t - N1, NN = first ? N1 : N2, hh = first ? h1 : h2;
                const int f = fft_pos_to_freq(first ? fH : fW, pos);
                const int sf = f < hh ? f : (f >= NN - hh ? f - NN : INT32_MIN);
                cfloat e = {0.f, 0.f};
                if (sf != INT32_MIN) e = unit_root((long long)(first ? a : b) * sf, raw * NN, -1);
                if (first) ph1[pos] = cscale(e, inv);
                else ph2[pos] = e;
            }
            __syncthreads();
            for (int t = threadIdx.x; t < n; t += blockDim.x) {
                const int p1 = (int)dN2.div(t), p2 = t - p1 * N2;
                Wk[p1 * LD + p2] = cmul(X[p1 * LD + p2], cmul(ph1[p1], ph2[p2]));
            }
            __syncthreads();
            // FORWARD transform back to the sample grid of this plane
            block_fft_lines(false, fH, Wk, dN2, 1, LD, true, tw1, -1);
            block_fft_lines(false, fW, Wk, dN1, LD, 1, true, tw2, -1);
            for (int t = threadIdx.x; t < n; t += blockDim.x) {
                const int p = (int)dN2.div(t), q = t - p * N2;
                const float m = amp(Wk[p * LD + q]);
                out[(size_t)(raw * p + a) * outW + raw * q + b] = m;
                asum += m;
            }
            __syncthreads();
        }
    }
    if (which == 0) {
        const double s = block_sum((double)asum, red);
        if (threadIdx.x == 0) rw->refMean = (float)(s / (double)(raw * raw * n));
    }
}

#ifdef AMPCOR_PART_PLAIN
__global__ void __launch_bounds__(512) k_oversample(const __grid_constant__ WindowPlan P, const cfloat* __restrict__ ref, long long ldr,
                                                    const cfloat* __restrict__ sec, long long lds,
                                                    const WindowCoords* __restrict__ coords, int w0, int wend,
                                                    RawResult* __restrict__ res, float* __restrict__ osRef,
                                                    float* __restrict__ osSch) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int w = w0 + blockIdx.x;
    if (w >= wend) return;
    const int which = blockIdx.y;
    float* out = which ? osSch + (size_t)(w - w0) * P.osHz * P.osWz : osRef + (size_t)(w - w0) * P.osWh * P.osWw;
    os_body<0>(P, smem, which, ref, ldr, sec, lds, coords[w], &res[w], out);
}
#endif

// ---------------------------------------------------------------------------
// Separable oversampler for raw = 2 and even chip sides (the usual case).
// Spectral zero padding of an even length keeps every input sample and puts
// the half-sample shift of the signal between them, and the 2-D operation
// factors into a shift along the rows and one along the columns:
//   plane (0,0) = x,  (0,1) = R x,  (1,0) = C x,  (1,1) = R C x,
// with R x = IDFT_row(DFT+_row(x) e^{-i pi f/N2}) / N2 and C likewise along
// the columns (the reference computes the same numbers with a 2-D INVERSE
// transform, quadrant padding and a 2-D FORWARD transform of the 4x grid,
// cuOverSampler.cpp:72-78).  Plane (0,1) is built one block of rows at a time
// in a small buffer, so one chip tile plus that block fit twice per SM.
// ---------------------------------------------------------------------------
constexpr int kOs2Threads = 256;
constexpr int kOs2Rows = 32;

#ifdef AMPCOR_PART_PLAIN
size_t os2_smem_bytes(const WindowPlan& P) {
    const int a = P.Wh * odd_ld(P.Ww), b = P.Hz * odd_ld(P.Wz);
    const int n = a > b ? a : b;
    const int l = (P.Wh + P.Ww) > (P.Hz + P.Wz) ? (P.Wh + P.Ww) : (P.Hz + P.Wz);
    const int ldmax = odd_ld(P.Ww) > odd_ld(P.Wz) ? odd_ld(P.Ww) : odd_ld(P.Wz);
    return align16((size_t)n * sizeof(cfloat)) + align16((size_t)kOs2Rows * ldmax * sizeof(cfloat)) +
           2 * align16((size_t)l * sizeof(cfloat)) + 40 * sizeof(double);
}
#endif

// GU: chip loads in flight per thread, as raw_body (0: cp.async copies, used
// by every kernel)
template <int GU = 1>
__device__ __forceinline__ void os2_body(const WindowPlan& P, unsigned char* smem, int which,
                                         const cfloat* __restrict__ ref, long long ldr,
                                         const cfloat* __restrict__ sec, long long lds, const WindowCoords wc,
                                         RawResult* __restrict__ rw, float* __restrict__ out) {
    const int N1 = which ? P.Hz : P.Wh, N2 = which ? P.Wz : P.Ww;
    const FftPlan1D& fH = which ? P.fSchH : P.fRefH;
    const FftPlan1D& fW = which ? P.fSchW : P.fRefW;
    const int n = N1 * N2, LD = odd_ld(N2);
    const int a0 = P.Wh * odd_ld(P.Ww), b0 = P.Hz * odd_ld(P.Wz);
    const int nmax = a0 > b0 ? a0 : b0;
    const int ldmax = odd_ld(P.Ww) > odd_ld(P.Wz) ? odd_ld(P.Ww) : odd_ld(P.Wz);
    const int lmax = (P.Wh + P.Ww) > (P.Hz + P.Wz) ? (P.Wh + P.Ww) : (P.Hz + P.Wz);
    unsigned char* q = smem;
    cfloat* X = reinterpret_cast<cfloat*>(q);    q += align16((size_t)nmax * sizeof(cfloat));
    cfloat* Cb = reinterpret_cast<cfloat*>(q);   q += align16((size_t)kOs2Rows * ldmax * sizeof(cfloat));
    cfloat* tw1 = reinterpret_cast<cfloat*>(q);  // N1 then N2 roots
    cfloat* tw2 = tw1 + N1;                      q += align16((size_t)lmax * sizeof(cfloat));
    cfloat* ph1 = reinterpret_cast<cfloat*>(q);  // per digit-reversed position: e^{-i pi f/N}/N
    cfloat* ph2 = ph1 + N1;                      q += align16((size_t)lmax * sizeof(cfloat));
    double* red = reinterpret_cast<double*>(q);
    const FastDiv dN2(N2), dN1(N1), dRB(kOs2Rows);

    const cfloat* src;
    long long ld;
    if (which) {
        const RawResult r = *rw;
        src = sec + (long long)(wc.secD + r.startX) * lds + (wc.secA + r.startY);
        ld = lds;
    } else {
        src = ref + (long long)wc.refD * ldr + wc.refA;
        ld = ldr;
    }
    block_fill_roots(tw1, N1);
    block_fill_roots(tw2, N2);
    for (int t = threadIdx.x; t < N1 + N2; t += blockDim.x) {
        const bool first = t < N1;
        const int pos = first ? t : t - N1, NN = first ? N1 : N2;
        const int f = fft_pos_to_freq(first ? fH : fW, pos);
        const int sf = f < NN / 2 ? f : f - NN;
        (first ? ph1 : ph2)[pos] = cscale(unit_root((long long)sf, 2 * NN, -1), 1.0f / (float)NN);
    }
    if constexpr (GU == 0) {
        for (int t = threadIdx.x; t < n; t += blockDim.x) {
            const int i = (int)dN2.div(t), j = t - i * N2;
            cp_async_c(X + i * LD + j, src + (long long)i * ld + j);
        }
        cp_async_wait_all();
        if (P.deramp == 0) {  // each thread converts the samples it copied
            for (int t = threadIdx.x; t < n; t += blockDim.x) {
                const int i = (int)dN2.div(t), j = t - i * N2;
                X[i * LD + j] = cfloat{amp(X[i * LD + j]), 0.f};
            }
        }
    } else if constexpr (GU == 1) {
        for (int t = threadIdx.x; t < n; t += blockDim.x) {
            const int i = (int)dN2.div(t), j = t - i * N2;
            const cfloat z = ld_c(src + (long long)i * ld + j);
            X[i * LD + j] = P.deramp == 0 ? cfloat{amp(z), 0.f} : z;
        }
    } else {
        block_gather<GU, cfloat>(
            n,
            [&](int t) {
                const int i = (int)dN2.div(t), j = t - i * N2;
                return ld_c(src + (long long)i * ld + j);
            },
            [&](int t, cfloat z) {
                const int i = (int)dN2.div(t), j = t - i * N2;
                X[i * LD + j] = P.deramp == 0 ? cfloat{amp(z), 0.f} : z;
            });
    }
    __syncthreads();
    if (P.deramp == 1) {
        // cuDerampMethod1_kernel (cuDeramp.cu:67-114), with its quirks
        float yr = 0.f, yi = 0.f, xr = 0.f, xi = 0.f;
        for (int t = threadIdx.x; t < n; t += blockDim.x) {
            const int i = (int)dN2.div(t), j = t - i * N2;
            const cfloat a = X[i * LD + j];
            if (j < N2 - 1) {
                const cfloat b = X[i * LD + j + 1];
                yr = fmaf(a.x, b.x, fmaf(a.y, b.y, yr));
                yi = fmaf(a.y, b.x, fmaf(-a.x, b.y, yi));
            }
            if (i < N1 - 1) {
                const cfloat b = X[(i + 1) * LD + j];
                xr = fmaf(a.x, b.x, fmaf(a.y, b.y, xr));
                xi = fmaf(a.y, b.x, fmaf(-a.x, b.y, xi));
            }
        }
        const double dyr = block_sum((double)yr, red);
        const double dyi = block_sum((double)yi, red);
        const double dxr = block_sum((double)xr, red);
        const double dxi = block_sum((double)xi, red);
        const float phaseY = atan2f((float)dyi, (float)dyr);
        const float phaseX = atan2f((float)dxi, (float)dxr);
        for (int t = threadIdx.x; t < n; t += blockDim.x) {
            const int row = (int)dN2.div(t), col = t - row * N2;
            const float phv = (float)col * phaseX + (float)row * phaseY;
            float sn, cs;
            sincosf(phv, &sn, &cs);
            const cfloat z = X[row * LD + col];
            const float nr = z.x * cs - z.y * sn;
            const float ni = z.y * cs + nr * sn;
            X[row * LD + col] = {nr, ni};
        }
        __syncthreads();
    }
    const int outW = 2 * N2;
    float asum = 0.f;
    // plane (0,0): the samples themselves
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        const int p = (int)dN2.div(t), c = t - p * N2;
        const float m = amp(X[p * LD + c]);
        out[(size_t)(2 * p) * outW + 2 * c] = m;
        asum += m;
    }
    // plane (0,1): half-sample shift along the rows, one block of rows at a time
    for (int r0 = 0; r0 < N1; r0 += kOs2Rows) {
        const int rows = min(kOs2Rows, N1 - r0);
        const FastDiv dr(rows);
        __syncthreads();
        for (int t = threadIdx.x; t < rows * N2; t += blockDim.x) {
            const int i = (int)dN2.div(t), j = t - i * N2;
            Cb[i * LD + j] = X[(r0 + i) * LD + j];
        }
        __syncthreads();
        block_fft_lines(true, fW, Cb, dr, LD, 1, true, tw2, +1);
        for (int t = threadIdx.x; t < rows * N2; t += blockDim.x) {
            const int i = (int)dN2.div(t), j = t - i * N2;
            Cb[i * LD + j] = cmul(Cb[i * LD + j], ph2[j]);
        }
        __syncthreads();
        block_fft_lines(false, fW, Cb, dr, LD, 1, true, tw2, -1);
        for (int t = threadIdx.x; t < rows * N2; t += blockDim.x) {
            const int i = (int)dN2.div(t), j = t - i * N2;
            const float m = amp(Cb[i * LD + j]);
            out[(size_t)(2 * (r0 + i)) * outW + 2 * j + 1] = m;
            asum += m;
        }
    }
    __syncthreads();
    // plane (1,0): half-sample shift along the columns, in place
    block_fft_lines(true, fH, X, dN2, 1, LD, true, tw1, +1);
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        const int i = (int)dN2.div(t), j = t - i * N2;
        X[i * LD + j] = cmul(X[i * LD + j], ph1[i]);
    }
    __syncthreads();
    block_fft_lines(false, fH, X, dN2, 1, LD, true, tw1, -1);
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        const int p = (int)dN2.div(t), c = t - p * N2;
        const float m = amp(X[p * LD + c]);
        out[(size_t)(2 * p + 1) * outW + 2 * c] = m;
        asum += m;
    }
    __syncthreads();
    // plane (1,1): then along the rows, in place
    block_fft_lines(true, fW, X, dN1, LD, 1, true, tw2, +1);
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        const int i = (int)dN2.div(t), j = t - i * N2;
        X[i * LD + j] = cmul(X[i * LD + j], ph2[j]);
    }
    __syncthreads();
    block_fft_lines(false, fW, X, dN1, LD, 1, true, tw2, -1);
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        const int p = (int)dN2.div(t), c = t - p * N2;
        const float m = amp(X[p * LD + c]);
        out[(size_t)(2 * p + 1) * outW + 2 * c + 1] = m;
        asum += m;
    }
    if (which == 0) {
        const double sm = block_sum((double)asum, red);
        if (threadIdx.x == 0) rw->refMean = (float)(sm / (double)(4 * n));
    }
}

#ifdef AMPCOR_PART_PLAIN
__global__ void __launch_bounds__(kOs2Threads, 2) k_oversample2(const __grid_constant__ WindowPlan P,
                                                               const cfloat* __restrict__ ref, long long ldr,
                                                               const cfloat* __restrict__ sec, long long lds,
                                                               const WindowCoords* __restrict__ coords, int w0,
                                                               int wend, RawResult* __restrict__ res,
                                                               float* __restrict__ osRef, float* __restrict__ osSch) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int w = w0 + blockIdx.x;
    if (w >= wend) return;
    const int which = blockIdx.y;
    // the same chip of the window the CTA that follows on the SM will take
    // (two CTAs per SM; CTAs start in index order, the reference chips first)
    const int wn = w + 2 * sm_count();
    if (wn < wend) {
        const WindowCoords c = coords[wn];
        if (which) {
            const RawResult r = res[wn];
            prefetch_chip_l2(sec + (long long)(c.secD + r.startX) * lds + (c.secA + r.startY), lds, P.Hz, P.Wz);
        } else {
            prefetch_chip_l2(ref + (long long)c.refD * ldr + c.refA, ldr, P.Wh, P.Ww);
        }
    }
    float* out = which ? osSch + (size_t)(w - w0) * P.osHz * P.osWz : osRef + (size_t)(w - w0) * P.osWh * P.osWw;
    os2_body<0>(P, smem, which, ref, ldr, sec, lds, coords[w], &res[w], out);
}
#endif


// ---------------------------------------------------------------------------
// The same separable oversampler for chips too large for shared memory (a
// 256 x 256 window gives a 264 x 264 zoom-in chip, 550 KB).  The chip sits
// row-major in a global slot of the CTA (L2-resident); the row shifts run on
// groups of osGl rows and the column shift on groups of osGl columns, each
// staged through shared memory.  Per line the arithmetic is that of os2_body.
// ---------------------------------------------------------------------------
#ifdef AMPCOR_PART_PLAIN
size_t os2_l2_smem_bytes(const WindowPlan& P) {
    const int nmax = std::max(std::max(P.Wh, P.Ww), std::max(P.Hz, P.Wz));
    const int lmax = std::max(P.Wh + P.Ww, P.Hz + P.Wz);
    return align16((size_t)P.osGl * odd_ld(nmax) * sizeof(cfloat)) + 2 * align16((size_t)lmax * sizeof(cfloat)) +
           40 * sizeof(double);
}
#endif

#ifdef AMPCOR_PART_PLAIN
size_t os2_l2_slot_bytes(const WindowPlan& P) {
    const size_t a = (size_t)P.Wh * P.Ww, b = (size_t)P.Hz * P.Wz;
    return ((std::max(a, b) * sizeof(cfloat)) + 255) & ~(size_t)255;
}
#endif

__device__ __forceinline__ void os2_l2_body(const WindowPlan& P, unsigned char* smem, int which,
                                            const cfloat* __restrict__ ref, long long ldr,
                                            const cfloat* __restrict__ sec, long long lds, const WindowCoords wc,
                                            RawResult* __restrict__ rw, cfloat* __restrict__ X,
                                            float* __restrict__ out) {
    const int N1 = which ? P.Hz : P.Wh, N2 = which ? P.Wz : P.Ww;
    const FftPlan1D& fH = which ? P.fSchH : P.fRefH;
    const FftPlan1D& fW = which ? P.fSchW : P.fRefW;
    const int n = N1 * N2, G = P.osGl;
    const int nmax = max(max(P.Wh, P.Ww), max(P.Hz, P.Wz));
    const int lmax = max(P.Wh + P.Ww, P.Hz + P.Wz);
    const int LB = odd_ld(nmax);
    unsigned char* q = smem;
    cfloat* buf = reinterpret_cast<cfloat*>(q);  q += align16((size_t)G * LB * sizeof(cfloat));
    cfloat* tw1 = reinterpret_cast<cfloat*>(q);
    cfloat* tw2 = tw1 + N1;                      q += align16((size_t)lmax * sizeof(cfloat));
    cfloat* ph1 = reinterpret_cast<cfloat*>(q);
    cfloat* ph2 = ph1 + N1;                      q += align16((size_t)lmax * sizeof(cfloat));
    double* red = reinterpret_cast<double*>(q);
    const FastDiv dN2(N2), dN1(N1);

    const cfloat* src;
    long long ld;
    if (which) {
        const RawResult r = *rw;
        src = sec + (long long)(wc.secD + r.startX) * lds + (wc.secA + r.startY);
        ld = lds;
    } else {
        src = ref + (long long)wc.refD * ldr + wc.refA;
        ld = ldr;
    }
    block_fill_roots(tw1, N1);
    block_fill_roots(tw2, N2);
    for (int t = threadIdx.x; t < N1 + N2; t += blockDim.x) {
        const bool first = t < N1;
        const int pos = first ? t : t - N1, NN = first ? N1 : N2;
        const int f = fft_pos_to_freq(first ? fH : fW, pos);
        const int sf = f < NN / 2 ? f : f - NN;
        (first ? ph1 : ph2)[pos] = cscale(unit_root((long long)sf, 2 * NN, -1), 1.0f / (float)NN);
    }
    float phaseX = 0.f, phaseY = 0.f;
    if (P.deramp == 1) {
        float yr = 0.f, yi = 0.f, xr = 0.f, xi = 0.f;
        for (int t = threadIdx.x; t < n; t += blockDim.x) {
            const int i = (int)dN2.div(t), j = t - i * N2;
            const cfloat a = ld_c(src + (long long)i * ld + j);
            if (j < N2 - 1) {
                const cfloat b = ld_c(src + (long long)i * ld + j + 1);
                yr = fmaf(a.x, b.x, fmaf(a.y, b.y, yr));
                yi = fmaf(a.y, b.x, fmaf(-a.x, b.y, yi));
            }
            if (i < N1 - 1) {
                const cfloat b = ld_c(src + (long long)(i + 1) * ld + j);
                xr = fmaf(a.x, b.x, fmaf(a.y, b.y, xr));
                xi = fmaf(a.y, b.x, fmaf(-a.x, b.y, xi));
            }
        }
        const double dyr = block_sum((double)yr, red);
        const double dyi = block_sum((double)yi, red);
        const double dxr = block_sum((double)xr, red);
        const double dxi = block_sum((double)xi, red);
        phaseY = atan2f((float)dyi, (float)dyr);
        phaseX = atan2f((float)dxi, (float)dxr);
    }
    const int outW = 2 * N2;
    float asum = 0.f;
    // the (deramped) chip into the slot, plane (0,0)
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        const int i = (int)dN2.div(t), j = t - i * N2;
        const cfloat z = ld_c(src + (long long)i * ld + j);
        cfloat v;
        if (P.deramp == 0) {
            v = {amp(z), 0.f};
        } else {
            const float phv = (float)j * phaseX + (float)i * phaseY;
            float sn, cs;
            sincosf(phv, &sn, &cs);
            const float nr = z.x * cs - z.y * sn;
            v = {nr, z.y * cs + nr * sn};
        }
        X[t] = v;
        const float m = amp(v);
        out[(size_t)(2 * i) * outW + 2 * j] = m;
        asum += m;
    }
    __syncthreads();
    // rows of X (pass 0: plane (0,1)) and, after the column pass, of C X (pass 1: plane (1,1))
    auto row_pass = [&](int odd_row) {
        for (int r0 = 0; r0 < N1; r0 += G) {
            const int rows = min(G, N1 - r0);
            const FastDiv dr(rows);
            for (int t = threadIdx.x; t < rows * N2; t += blockDim.x) {
                const int i = (int)dN2.div(t), j = t - i * N2;
                buf[i * LB + j] = X[(size_t)(r0 + i) * N2 + j];
            }
            __syncthreads();
            block_fft_lines(true, fW, buf, dr, LB, 1, true, tw2, +1);
            for (int t = threadIdx.x; t < rows * N2; t += blockDim.x) {
                const int i = (int)dN2.div(t), j = t - i * N2;
                buf[i * LB + j] = cmul(buf[i * LB + j], ph2[j]);
            }
            __syncthreads();
            block_fft_lines(false, fW, buf, dr, LB, 1, true, tw2, -1);
            for (int t = threadIdx.x; t < rows * N2; t += blockDim.x) {
                const int i = (int)dN2.div(t), j = t - i * N2;
                const float m = amp(buf[i * LB + j]);
                out[(size_t)(2 * (r0 + i) + odd_row) * outW + 2 * j + 1] = m;
                asum += m;
            }
            __syncthreads();
        }
    };
    row_pass(0);
    // plane (1,0): column groups; C X goes back into the slot
    for (int c0 = 0; c0 < N2; c0 += G) {
        const int cols = min(G, N2 - c0);
        const FastDiv dc(cols);
        for (int t = threadIdx.x; t < cols * N1; t += blockDim.x) {
            const int i = (int)dc.div(t), k = t - i * cols;
            buf[k * LB + i] = X[(size_t)i * N2 + c0 + k];
        }
        __syncthreads();
        block_fft_lines(true, fH, buf, dc, LB, 1, true, tw1, +1);
        for (int t = threadIdx.x; t < cols * N1; t += blockDim.x) {
            const int k = (int)dN1.div(t), i = t - k * N1;
            buf[k * LB + i] = cmul(buf[k * LB + i], ph1[i]);
        }
        __syncthreads();
        block_fft_lines(false, fH, buf, dc, LB, 1, true, tw1, -1);
        for (int t = threadIdx.x; t < cols * N1; t += blockDim.x) {
            const int i = (int)dc.div(t), k = t - i * cols;
            const cfloat v = buf[k * LB + i];
            X[(size_t)i * N2 + c0 + k] = v;
            const float m = amp(v);
            out[(size_t)(2 * i + 1) * outW + 2 * (c0 + k)] = m;
            asum += m;
        }
        __syncthreads();
    }
    row_pass(1);
    if (which == 0) {
        const double sm = block_sum((double)asum, red);
        if (threadIdx.x == 0) rw->refMean = (float)(sm / (double)(4 * n));
    }
}

// Plain-path launch over 2 * (wend - w0) chips (window-major, reference
// first), one global slot per CTA.
#ifdef AMPCOR_PART_PLAIN
__global__ void __launch_bounds__(kOs2L2Threads) k_oversample2_l2(const __grid_constant__ WindowPlan P,
                                                               const cfloat* __restrict__ ref, long long ldr,
                                                               const cfloat* __restrict__ sec, long long lds,
                                                               const WindowCoords* __restrict__ coords, int w0,
                                                               int wend, RawResult* __restrict__ res,
                                                               float* __restrict__ osRef, float* __restrict__ osSch,
                                                               unsigned char* __restrict__ slots, size_t slot_bytes) {
    extern __shared__ __align__(16) unsigned char smem[];
    cfloat* X = reinterpret_cast<cfloat*>(slots + (size_t)blockIdx.x * slot_bytes);
    const int nitem = 2 * (wend - w0);
    for (int it = blockIdx.x; it < nitem; it += gridDim.x) {
        const int w = w0 + (it >> 1), which = it & 1;
        float* out = which ? osSch + (size_t)(w - w0) * P.osHz * P.osWz
                           : osRef + (size_t)(w - w0) * P.osWh * P.osWw;
        os2_l2_body(P, smem, which, ref, ldr, sec, lds, coords[w], &res[w], X, out);
        __syncthreads();
    }
}
#endif

#ifdef AMPCOR_PART_PLAIN
void launch_oversample(const WindowPlan& P, int nb, cudaStream_t st, const cfloat* ref, long long ldr,
                       const cfloat* sec, long long lds, const WindowCoords* coords, int w0, int wend,
                       RawResult* res, float* osRef, float* osSch) {
    if (os2_applies(P)) {
        const size_t sm = os2_smem_bytes(P);
        cudaFuncSetAttribute(k_oversample2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_oversample2<<<dim3(nb, 2), kOs2Threads, sm, st>>>(P, ref, ldr, sec, lds, coords, w0, wend, res, osRef,
                                                            osSch);
    } else {
        const size_t sm = os_smem_bytes(P);
        cudaFuncSetAttribute(k_oversample, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_oversample<<<dim3(nb, 2), 512, sm, st>>>(P, ref, ldr, sec, lds, coords, w0, wend, res, osRef, osSch);
    }
}
#endif

// ---------------------------------------------------------------------------
// Separable raw = 2 oversampler as dense contractions on the 5th-generation
// tensor cores (tcgen05), for chips whose sides round up to at most 80.
// The half-sample shift of a length-N line is a fixed N x N complex matrix
// S (S[j', j] = (1/N) sum_f e^{2 pi i f (j - j')/N} e^{-i pi sf/N}, the
// phase-ramped DFT pair of os2_body), so the three shifted planes are
//   (0,1) = X S_W^T,  (1,0) = S_H X,  (1,1) = (S_H X) S_W^T,
// each a real GEMM D = A B^T of M = 128 rows (chip rows, zero padded), in
// the real form [Xr | Xi] x [[Sr, -Si], [Si, Sr]].  Operands are bf16 in
// shared memory in the no-swizzle K-major core-matrix layout; with
// split-BF16 (osTc 1) A and B are each split into hi + lo and the product is
// hi*hi + hi*lo + lo*hi (about 16 significant bits), FP32 accumulation in
// tensor memory.  The shift tables (real form, core layout, hi then lo) are
// built on the host in FP64 per chip side.  One CTA of 256 threads per chip.
// ---------------------------------------------------------------------------
#ifdef AMPCOR_PART_PLAIN
// one GEMM: D (tmem, 128 x Nb fp32) = A (128 x K) B^T (Nb x K), issued by one thread
__device__ __forceinline__ void os_tc_mma(uint32_t tmem, const __nv_bfloat16* Ah, const __nv_bfloat16* Al,
                                          const __nv_bfloat16* Bh, const __nv_bfloat16* Bl, int K, int Nb,
                                          bool split, uint64_t* bar) {
    const uint32_t idesc = umma::idesc_bf16(128, Nb);
    const uint32_t sbo = 16 * K;
    for (int k0 = 0; k0 < K; k0 += 16) {
        const uint32_t koff = (uint32_t)(k0 / 8) * 128;
        const uint64_t ah = umma::make_desc(umma::smem_addr(Ah) + koff, 128, sbo);
        const uint64_t bh = umma::make_desc(umma::smem_addr(Bh) + koff, 128, sbo);
        umma::mma_bf16(tmem, ah, bh, idesc, k0 > 0);
        if (split) {
            const uint64_t al = umma::make_desc(umma::smem_addr(Al) + koff, 128, sbo);
            const uint64_t bl = umma::make_desc(umma::smem_addr(Bl) + koff, 128, sbo);
            umma::mma_bf16(tmem, ah, bl, idesc, true);
            umma::mma_bf16(tmem, al, bh, idesc, true);
        }
    }
    umma::commit(bar);
}

__device__ __forceinline__ void os_tc_put(__nv_bfloat16* hi, __nv_bfloat16* lo, int r, int k, int K, float v) {
    __nv_bfloat16 h, l;
    umma::split_bf16(v, h, l);
    const size_t o = umma::core_offset(r, k, K) / 2;
    hi[o] = h;
    lo[o] = l;
}

__global__ void __launch_bounds__(kOsTcThreads, 1) k_oversample_tc(const __grid_constant__ WindowPlan P,
                                                                   const cfloat* __restrict__ ref, long long ldr,
                                                                   const cfloat* __restrict__ sec, long long lds,
                                                                   const WindowCoords* __restrict__ coords, int w0,
                                                                   int wend, RawResult* __restrict__ res,
                                                                   float* __restrict__ osRef,
                                                                   float* __restrict__ osSch,
                                                                   const uint4* __restrict__ tabRow0,
                                                                   const uint4* __restrict__ tabCol0,
                                                                   const uint4* __restrict__ tabRow1,
                                                                   const uint4* __restrict__ tabCol1,
                                                                   int* __restrict__ err) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char* smem =
        reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~(uintptr_t)127);
    const int w = w0 + blockIdx.x;
    if (w >= wend) return;
    const int which = blockIdx.y;
    const WindowCoords wc = coords[w];
    RawResult* rw = &res[w];
    const int N1 = which ? P.Hz : P.Wh, N2 = which ? P.Wz : P.Ww;
    const int N1p = pad16(N1), N2p = pad16(N2), K1 = 2 * N1p, K2 = 2 * N2p;
    const int np = max(max(pad16(P.Wh), pad16(P.Ww)), max(pad16(P.Hz), pad16(P.Wz)));
    const int Kmax = 2 * np;
    const uint4* tabRow = which ? tabRow1 : tabRow0;  // shift along a row (length N2)
    const uint4* tabCol = which ? tabCol1 : tabCol0;  // shift along a column (length N1)
    float* out = which ? osSch + (size_t)(w - w0) * P.osHz * P.osWz : osRef + (size_t)(w - w0) * P.osWh * P.osWw;
    const int outW = 2 * N2, n = N1 * N2;
    const bool split = P.osTc == 1;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    __nv_bfloat16* Ah = reinterpret_cast<__nv_bfloat16*>(smem);  // A operand: 128 x Kmax, hi then lo
    __nv_bfloat16* Al = Ah + 128 * Kmax;
    __nv_bfloat16* Bh = Al + 128 * Kmax;                          // B operand: Kmax x Kmax, hi then lo
    double* red = reinterpret_cast<double*>(Bh + 2 * (size_t)Kmax * Kmax);
    uint64_t* bar = reinterpret_cast<uint64_t*>(red + 40);  // MMA completion
    uint64_t* tbar = bar + 1;                                  // shift-table copy completion
    uint32_t* tbase = reinterpret_cast<uint32_t*>(bar + 2);

    if (warp == 0) umma::tmem_alloc(tbase, 256);
    // the shift tables arrive by one bulk copy each (cp.async.bulk) while the
    // threads build the A operand
    auto fetch_table = [&](const uint4* tab, int Kt) {
        const uint32_t bytes = (uint32_t)(2 * (size_t)Kt * Kt * 2);
        tma::arrive_expect_tx(tbar, bytes);
        tma::load_bulk(Bh, tab, bytes, tbar);
    };
    if (tid == 0) {
        umma::mbar_init(bar, 1);
        umma::mbar_init(tbar, 1);
        tma::fence_barrier_init();
        fetch_table(tabRow, K2);
    }

    const cfloat* src;
    long long ld;
    if (which) {
        const RawResult r = *rw;
        src = sec + (long long)(wc.secD + r.startX) * lds + (wc.secA + r.startY);
        ld = lds;
    } else {
        src = ref + (long long)wc.refD * ldr + wc.refA;
        ld = ldr;
    }
    // deramp (cuDerampMethod1_kernel, cuDeramp.cu:67-114, with its quirks), as os2_body
    float phaseX = 0.f, phaseY = 0.f;
    const FastDiv dN2(N2);
    if (P.deramp == 1) {
        float yr = 0.f, yi = 0.f, xr = 0.f, xi = 0.f;
        for (int t = tid; t < n; t += blockDim.x) {
            const int i = (int)dN2.div(t), j = t - i * N2;
            const cfloat a = ld_c(src + (long long)i * ld + j);
            if (j < N2 - 1) {
                const cfloat b = ld_c(src + (long long)i * ld + j + 1);
                yr = fmaf(a.x, b.x, fmaf(a.y, b.y, yr));
                yi = fmaf(a.y, b.x, fmaf(-a.x, b.y, yi));
            }
            if (i < N1 - 1) {
                const cfloat b = ld_c(src + (long long)(i + 1) * ld + j);
                xr = fmaf(a.x, b.x, fmaf(a.y, b.y, xr));
                xi = fmaf(a.y, b.x, fmaf(-a.x, b.y, xi));
            }
        }
        const double dyr = block_sum((double)yr, red);
        const double dyi = block_sum((double)yi, red);
        const double dxr = block_sum((double)xr, red);
        const double dxi = block_sum((double)xi, red);
        phaseY = atan2f((float)dyi, (float)dyr);
        phaseX = atan2f((float)dxi, (float)dxr);
    }
    auto chip = [&](int i, int j) -> cfloat {
        const cfloat z = ld_c(src + (long long)i * ld + j);
        if (P.deramp == 0) return {amp(z), 0.f};
        const float phv = (float)j * phaseX + (float)i * phaseY;
        float sn, cs;
        sincosf(phv, &sn, &cs);
        const float nr = z.x * cs - z.y * sn;
        return {nr, z.y * cs + nr * sn};
    };
    // a shift table (Kt x Kt, hi then lo halves, core layout) into B
    auto to_async = [&]() {  // operand writes visible to the tensor core, TMEM reads done
        umma::fence_smem_async();
        umma::fence_before_sync();
        __syncthreads();
        umma::fence_after_sync();
    };
    bool ok = true;
    bool table_timeout = false;  // thread 0 only
    float asum = 0.f;

    // operand writes walk one core matrix per 32 lanes (8 rows x 4 columns):
    // conflict-free 2-byte stores
    auto core_walk = [](int t, int ncb, int& r, int& c) {
        const int rest = t >> 6, cb = rest % ncb, rg = rest / ncb;
        r = rg * 8 + (t & 7);
        c = cb * 8 + ((t >> 3) & 7);
    };
    // 1. A = [Xr | Xi] rows i (K2); B = row-shift table
    for (int t = tid; t < 128 * N2p; t += blockDim.x) {
        int i, j;
        core_walk(t, N2p / 8, i, j);
        cfloat v = {0.f, 0.f};
        if (i < N1 && j < N2) v = chip(i, j);
        os_tc_put(Ah, Al, i, j, K2, v.x);
        os_tc_put(Ah, Al, i, N2p + j, K2, v.y);
    }
    to_async();
    const uint32_t tmem = *tbase;
    if (tid == 0) {
        if (umma::mbar_wait(tbar, 0)) {
            os_tc_mma(tmem, Ah, Al, Bh, Bh + (size_t)K2 * K2, K2, K2, split, bar);
        } else {
            table_timeout = true;  // report; complete the MMA phase without issuing
            umma::commit(bar);
        }
    }
    if (!umma::mbar_wait(bar, 0)) ok = false;
    if (tid == 0) fetch_table(tabCol, K1);  // the last MMA read of B is done
    ok = __all_sync(FULLMASK, ok);  // warp-uniform: tcgen05.ld is a warp-collective
    umma::fence_after_sync();
    // epilogue 1: plane (0,1) = |X S_W^T|; warps 0-3 and 4-7 take alternate column chunks
    const int row = (warp & 3) * 32 + lane;
    const uint32_t lanes = (uint32_t)((warp & 3) * 32) << 16;
    // amplitudes staged in shared memory (the A operand is consumed), then
    // written row by row
    float* stage = reinterpret_cast<float*>(Ah);
    const int SL = N2 + 1;
    if (ok)
        for (int c0 = (warp >> 2) * 16; c0 < N2p; c0 += 32) {
            float re[16], im[16];
            umma::tmem_ld16(tmem + lanes + c0, re);
            umma::tmem_ld16(tmem + lanes + N2p + c0, im);
            if (row < N1)
                for (int q = 0; q < 16 && c0 + q < N2; ++q)
                    stage[row * SL + c0 + q] = sqrtf(re[q] * re[q] + im[q] * im[q]);
        }
    __syncthreads();
    for (int t = tid; t < n; t += blockDim.x) {
        const int i = (int)dN2.div(t), j = t - i * N2;
        const float m = stage[i * SL + j];
        out[(size_t)(2 * i) * outW + 2 * j + 1] = m;
        asum += m;
    }
    to_async();
    // 2. plane (0,0); A = [Xr^T | Xi^T] rows j (K1); B = column-shift table
    for (int t = tid; t < 128 * N1p; t += blockDim.x) {
        int j, i;
        core_walk(t, N1p / 8, j, i);
        cfloat v = {0.f, 0.f};
        if (i < N1 && j < N2) {
            v = chip(i, j);
            const float m = amp(v);
            out[(size_t)(2 * i) * outW + 2 * j] = m;
            asum += m;
        }
        os_tc_put(Ah, Al, j, i, K1, v.x);
        os_tc_put(Ah, Al, j, N1p + i, K1, v.y);
    }
    to_async();
    if (tid == 0) {
        if (umma::mbar_wait(tbar, 1)) {
            os_tc_mma(tmem, Ah, Al, Bh, Bh + (size_t)K1 * K1, K1, K1, split, bar);
        } else {
            table_timeout = true;
            umma::commit(bar);
        }
    }
    if (!umma::mbar_wait(bar, 1)) ok = false;
    if (tid == 0) fetch_table(tabRow, K2);
    ok = __all_sync(FULLMASK, ok);
    umma::fence_after_sync();
    // epilogue 2: plane (1,0) = |S_H X| from D = (S_H X)^T (rows j, columns i'); keep S_H X
    // for the last product in registers' worth of passes: first zero A, then write it
    {
        uint4* zh = reinterpret_cast<uint4*>(Ah);
        uint4* zl = reinterpret_cast<uint4*>(Al);
        const int nz = (int)(128 * (size_t)K2 * 2 / 16);
        for (int t = tid; t < nz; t += blockDim.x) {
            zh[t] = make_uint4(0u, 0u, 0u, 0u);
            zl[t] = make_uint4(0u, 0u, 0u, 0u);
        }
    }
    __syncthreads();
    if (ok)
        for (int c0 = (warp >> 2) * 16; c0 < N1p; c0 += 32) {
            float re[16], im[16];
            umma::tmem_ld16(tmem + lanes + c0, re);
            umma::tmem_ld16(tmem + lanes + N1p + c0, im);
            if (row < N2)
                for (int q = 0; q < 16 && c0 + q < N1; ++q) {
                    const int ip = c0 + q;
                    const float m = sqrtf(re[q] * re[q] + im[q] * im[q]);
                    out[(size_t)(2 * ip + 1) * outW + 2 * row] = m;
                    asum += m;
                    os_tc_put(Ah, Al, ip, row, K2, re[q]);
                    os_tc_put(Ah, Al, ip, N2p + row, K2, im[q]);
                }
        }
    to_async();
    // 3. plane (1,1) = |(S_H X) S_W^T|
    if (tid == 0) {
        if (umma::mbar_wait(tbar, 0)) {
            os_tc_mma(tmem, Ah, Al, Bh, Bh + (size_t)K2 * K2, K2, K2, split, bar);
        } else {
            table_timeout = true;
            umma::commit(bar);
        }
    }
    if (!umma::mbar_wait(bar, 0)) ok = false;
    ok = __all_sync(FULLMASK, ok);
    umma::fence_after_sync();
    if (ok)
        for (int c0 = (warp >> 2) * 16; c0 < N2p; c0 += 32) {
            float re[16], im[16];
            umma::tmem_ld16(tmem + lanes + c0, re);
            umma::tmem_ld16(tmem + lanes + N2p + c0, im);
            if (row < N1)
                for (int q = 0; q < 16 && c0 + q < N2; ++q)
                    stage[row * SL + c0 + q] = sqrtf(re[q] * re[q] + im[q] * im[q]);
        }
    __syncthreads();
    for (int t = tid; t < n; t += blockDim.x) {
        const int i = (int)dN2.div(t), j = t - i * N2;
        const float m = stage[i * SL + j];
        out[(size_t)(2 * i + 1) * outW + 2 * j + 1] = m;
        asum += m;
    }
    if ((!ok && lane == 0) || table_timeout) atomicExch(err, 1);
    if (table_timeout) umma::mbar_wait(tbar, 0);  // let a late table copy land (bounded)
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_free(tmem, 256);
    if (which == 0) {
        const double sm = block_sum((double)asum, red);
        if (tid == 0) rw->refMean = (float)(sm / (double)(4 * n));
    }
}
#endif

// ---------------------------------------------------------------------------
// oversampled correlation + normalisation, zp x zp lags
// ---------------------------------------------------------------------------
constexpr int kCosCols = 16;  // template columns per staged chunk

__host__ __device__ inline int pow2_ceil(int x) {
    int p = 1;
    while (p < x) p <<= 1;
    return p;
}

// nt: threads of the CTA that runs the body (one partial sum per thread and lag row)
#ifdef AMPCOR_PART_PLAIN
size_t corr_os_smem_bytes(const WindowPlan& P, int nt) {
    const int zp = P.zp;
    const size_t T = align16((size_t)P.osWh * kCosCols * 4);
    const size_t S = align16((size_t)P.osHz * (kCosCols + zp - 1) * 4);
    const size_t part = align16((size_t)nt * zp * 4);
    const size_t stage = T + S > part ? T + S : part;
    const size_t H = align16((size_t)P.osHz * zp * 8);
    return stage + H + align16((size_t)zp * zp * 4) + 40 * sizeof(double);
}
#endif

// Direct correlation of the oversampled chips for lags (u, v) < ZP x ZP.
// Lane layout: v = lane % VP, column phase jj = lane / VP (VP = pow2 >= ZP).
// For S row r every lane adds T[r-u][j] * S[r][j+v] for all u: T values of
// the last ZP template rows sit in a circular register window, so each step
// costs one S load, one broadcast T load and ZP FMAs.
template <int ZP>
__device__ __forceinline__ void corr_os_chunk(const float* __restrict__ Tc, const float* __restrict__ Sc, int tH,
                                              int sH, int cols, int ldS, float* acc) {
    constexpr int VP = ZP <= 8 ? 8 : (ZP <= 16 ? 16 : 32);
    constexpr int J = 32 / VP;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    const int v = lane % VP, jj = lane / VP;
    if (v >= ZP) return;
    const int rend = tH + ZP - 1;
    for (int g = warp; g * J < cols; g += nwarp) {
        const int j = g * J + jj;
        if (j >= cols) continue;
        float win[ZP];
#pragma unroll
        for (int k = 0; k < ZP; ++k) win[k] = 0.f;
        for (int r0 = 0; r0 < rend; r0 += ZP) {
#pragma unroll
            for (int k = 0; k < ZP; ++k) {
                const int r = r0 + k;
                win[k] = r < tH ? Tc[r * kCosCols + j] : 0.f;
                const float sv = r < sH ? Sc[r * ldS + j + v] : 0.f;
#pragma unroll
                for (int u = 0; u < ZP; ++u) acc[u] = fmaf(win[(k - u + ZP) % ZP], sv, acc[u]);
            }
        }
    }
}

// Oversampled correlation of one window from its amplitude chips T and S
// (global memory) into the zp x zp surface `sf`.
template <int ZP>
__device__ __forceinline__ void corr_os_body(const WindowPlan& P, unsigned char* smem, float mean,
                                             const float* __restrict__ T, const float* __restrict__ S,
                                             float* __restrict__ sf) {
    const int tW = P.osWw, tH = P.osWh, sW = P.osWz, sH = P.osHz;
    const int ldS = kCosCols + ZP - 1;
    float* Tc = reinterpret_cast<float*>(smem);
    float* Sc = reinterpret_cast<float*>(smem + align16((size_t)tH * kCosCols * 4));
    float* part = Tc;  // reused after the last chunk
    const size_t stageT = align16((size_t)tH * kCosCols * 4), stageS = align16((size_t)sH * ldS * 4);
    const size_t partB = align16((size_t)blockDim.x * ZP * 4);
    float2* H = reinterpret_cast<float2*>(smem + (stageT + stageS > partB ? stageT + stageS : partB));
    float* var = reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(H) + align16((size_t)sH * ZP * 8));
    double* red = reinterpret_cast<double*>(reinterpret_cast<unsigned char*>(var) + align16((size_t)ZP * ZP * 4));

    // exact box sums of the oversampled search amplitude: one warp per row
    // for the ZP horizontal lags, then one warp per lag column for the
    // vertical lags (warp_box_group)
    {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
        for (int r = warp; r < sH; r += nwarp) {
            const float* row = S + (size_t)r * sW;
            const float2 h = warp_box_group([&](int j) {
                const float a = row[j];  // coherent load: the persistent kernel writes S
                return make_float2(a, a * a);
            }, tW, 0, ZP);
            if (lane < ZP) H[r * ZP + lane] = h;
        }
        __syncthreads();
        const double invnd = 1.0 / (double)(tH * tW);
        for (int v = warp; v < ZP; v += nwarp) {
            const float2 b = warp_box_group([&](int i) { return H[i * ZP + v]; }, tH, 0, ZP);
            if (lane < ZP) var[lane * ZP + v] = var_fp64(b.x, b.y, invnd);
        }
    }

    float acc[ZP];
#pragma unroll
    for (int u = 0; u < ZP; ++u) acc[u] = 0.f;
    float r2 = 0.f;
    for (int j0 = 0; j0 < tW; j0 += kCosCols) {
        const int cols = min(kCosCols, tW - j0);
        __syncthreads();
        for (int t = threadIdx.x; t < tH * kCosCols; t += blockDim.x) {
            const int i = t / kCosCols, c = t - (t / kCosCols) * kCosCols;
            float val = 0.f;
            if (c < cols) {
                val = T[(size_t)i * tW + j0 + c] - mean;
                r2 = fmaf(val, val, r2);
            }
            Tc[t] = val;
        }
        for (int t = threadIdx.x; t < sH * ldS; t += blockDim.x) {
            const int i = t / ldS, c = t - (t / ldS) * ldS;
            Sc[t] = (j0 + c < sW) ? S[(size_t)i * sW + j0 + c] : 0.f;
        }
        __syncthreads();
        corr_os_chunk<ZP>(Tc, Sc, tH, sH, cols, ldS, acc);
    }
    const float R2 = (float)block_sum((double)r2, red);  // also orders the last chunk before reuse
#pragma unroll
    for (int u = 0; u < ZP; ++u) part[threadIdx.x * ZP + u] = acc[u];
    __syncthreads();
    constexpr int VP = ZP <= 8 ? 8 : (ZP <= 16 ? 16 : 32);
    for (int t = threadIdx.x; t < ZP * ZP; t += blockDim.x) {
        const int u = t / ZP, v = t - (t / ZP) * ZP;
        // sum the partials of every thread whose lane holds lag column v
        float c = 0.f;
        for (int th = v; th < (int)blockDim.x; th += VP) c += part[th * ZP + u];
        sf[t] = c / sqrtf(var[t] * R2 + FLT_EPSILON);
    }
}

#ifdef AMPCOR_PART_PLAIN
template <int ZP>
__global__ void __launch_bounds__(kCosThreads) k_corr_os_t(const __grid_constant__ WindowPlan P, int w0, int wend,
                                                           const RawResult* __restrict__ res,
                                                           const float* __restrict__ osRef,
                                                           const float* __restrict__ osSch,
                                                           float* __restrict__ surf) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int w = w0 + blockIdx.x;
    if (w >= wend) return;
    corr_os_body<ZP>(P, smem, res[w].refMean, osRef + (size_t)(w - w0) * P.osWh * P.osWw,
                     osSch + (size_t)(w - w0) * P.osHz * P.osWz, surf + (size_t)(w - w0) * ZP * ZP);
}
#endif

// The same correlation with the template and search columns staged by TMA
// (cp.async.bulk.tensor) into two shared-memory stages: the copies of chunk
// k+1 run while chunk k is correlated.  One CTA of 16 warps per SM.
constexpr int kCosTmaThreads = 512;
constexpr int kCosTmaCols = 32;  // template columns per staged chunk (16 for chips too tall for 32)

struct CosTmaGeom {
    int cols, tBoxRows, tBoxes, sBoxRows, sBoxes, sCols, stageBytes, txBytes;
};

__host__ __device__ inline size_t align128(size_t b) { return (b + 127) & ~(size_t)127; }

static CosTmaGeom cos_tma_geom(const WindowPlan& P, int cols = kCosTmaCols) {
    CosTmaGeom g;
    g.cols = cols;
    // boxes of at most 256 rows, row counts a multiple of 8 so that every box
    // (rows x 128-byte multiples) starts on a 128-byte boundary
    // the template stage also holds zp-1 zero rows below the template, so the
    // correlation loop runs over tH+zp-1 rows without bounds checks
    const int tRows = P.osWh + P.zp - 1;
    g.tBoxes = (tRows + 255) / 256;
    g.tBoxRows = ((tRows + g.tBoxes - 1) / g.tBoxes + 7) / 8 * 8;
    g.sBoxes = (P.osHz + 255) / 256;
    g.sBoxRows = ((P.osHz + g.sBoxes - 1) / g.sBoxes + 7) / 8 * 8;
    g.sCols = (cols + P.zp - 1 + 3) / 4 * 4;
    const int tb = g.tBoxes * g.tBoxRows * cols * 4, sb = g.sBoxes * g.sBoxRows * g.sCols * 4;
    g.txBytes = tb + sb;
    g.stageBytes = (int)(align128((size_t)tb) + align128((size_t)sb));
    return g;
}

// The row box sums H (osHz x zp float2) are consumed before the first chunk
// lands in the second stage, so they live there when they fit.
__host__ __device__ inline bool cos_tma_h_in_stage(const WindowPlan& P, const CosTmaGeom& g) {
    return align16((size_t)P.osHz * P.zp * 8) <= (size_t)g.stageBytes;
}

static size_t corr_os_tma_smem_bytes(const WindowPlan& P, int cols = kCosTmaCols) {
    const CosTmaGeom g = cos_tma_geom(P, cols);
    const size_t part = align16((size_t)kCosTmaThreads * P.zp * 4);
    return 128 + 2 * (size_t)g.stageBytes + (part > (size_t)g.stageBytes ? part - g.stageBytes : 0) +
           (cos_tma_h_in_stage(P, g) ? 0 : align16((size_t)P.osHz * P.zp * 8)) + align16((size_t)P.zp * P.zp * 4) +
           40 * sizeof(double) + 32;
}

// Columns per chunk of the TMA-staged correlation for this geometry: 32, or
// 16 when the double buffer of 32-column chunks does not fit; 0 if neither.
static int cos_tma_cols(const WindowPlan& P) {
    if (P.osWw % 4 || P.osWz % 4 || !corr_os_supported(P.zp)) return 0;
    for (int c : {32, 16}) {
        if (c == 16 && P.zp != 8 && P.zp != 16) break;  // 16-column instances exist for these lag counts
        const CosTmaGeom g = cos_tma_geom(P, c);
        if (g.tBoxRows <= 256 && g.sBoxRows <= 256 && corr_os_tma_smem_bytes(P, c) <= 232448) return c;
    }
    return 0;
}

#ifdef AMPCOR_PART_PLAIN
bool corr_os_tma_applies(const WindowPlan& P) { return cos_tma_cols(P) > 0; }
#endif

#ifdef AMPCOR_PART_PLAIN
template <int ZP, int COLS>
__global__ void __launch_bounds__(kCosTmaThreads, 1) k_corr_os_tma(const __grid_constant__ WindowPlan P,
                                                                  const __grid_constant__ CUtensorMap tmT,
                                                                  const __grid_constant__ CUtensorMap tmS,
                                                                  const CosTmaGeom g, int w0, int wend,
                                                                  const RawResult* __restrict__ res,
                                                                  const float* __restrict__ osSch,
                                                                  float* __restrict__ surf, int* __restrict__ err,
                                                                  long long sStride, long long fStride) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~(uintptr_t)127);
    const int w = w0 + blockIdx.x;
    if (w >= wend) return;
    const int z = w - w0;
    const int tW = P.osWw, tH = P.osWh, sW = P.osWz, sH = P.osHz;
    const float mean = res[w].refMean;
    const size_t part_b = align16((size_t)kCosTmaThreads * ZP * 4);
    unsigned char* stage[2] = {smem, smem + g.stageBytes};
    unsigned char* q = smem + 2 * (size_t)g.stageBytes + (part_b > (size_t)g.stageBytes ? part_b - g.stageBytes : 0);
    float2* H;
    if (cos_tma_h_in_stage(P, g)) {
        H = reinterpret_cast<float2*>(stage[1]);
    } else {
        H = reinterpret_cast<float2*>(q);
        q += align16((size_t)sH * ZP * 8);
    }
    float* var = reinterpret_cast<float*>(q);   q += align16((size_t)ZP * ZP * 4);
    double* red = reinterpret_cast<double*>(q); q += 40 * sizeof(double);
    uint64_t* bar = reinterpret_cast<uint64_t*>(q);
    float* part = reinterpret_cast<float*>(smem);  // reused after the last chunk
    const int nchunks = (tW + COLS - 1) / COLS;
    const size_t tOff = align128((size_t)g.tBoxes * g.tBoxRows * COLS * 4);

    auto issue = [&](int k) {
        unsigned char* st = stage[k & 1];
        umma::fence_smem_async();  // earlier generic reads of this stage before the async writes
        tma::arrive_expect_tx(&bar[k & 1], (uint32_t)g.txBytes);
        for (int b = 0; b < g.tBoxes; ++b)
            tma::load_3d(st + (size_t)b * g.tBoxRows * COLS * 4, &tmT, k * COLS, b * g.tBoxRows, z,
                         &bar[k & 1]);
        for (int b = 0; b < g.sBoxes; ++b)
            tma::load_3d(st + tOff + (size_t)b * g.sBoxRows * g.sCols * 4, &tmS, k * COLS, b * g.sBoxRows, z,
                         &bar[k & 1]);
    };
    if (threadIdx.x == 0) {
        umma::mbar_init(&bar[0], 1);
        umma::mbar_init(&bar[1], 1);
        tma::fence_barrier_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) issue(0);

    // exact box sums of the oversampled search amplitude (warp_box_group),
    // overlapping the first copy
    {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
        const float* S = osSch + (size_t)z * sStride;
        for (int r = warp; r < sH; r += nwarp) {
            const float* row = S + (size_t)r * sW;
            const float2 h = warp_box_group([&](int j) {
                const float a = __ldg(row + j);
                return make_float2(a, a * a);
            }, tW, 0, ZP);
            if (lane < ZP) H[r * ZP + lane] = h;
        }
        __syncthreads();
        const double invnd = 1.0 / (double)(tH * tW);
        for (int v = warp; v < ZP; v += nwarp) {
            const float2 b = warp_box_group([&](int i) { return H[i * ZP + v]; }, tH, 0, ZP);
            if (lane < ZP) var[lane * ZP + v] = var_fp64(b.x, b.y, invnd);
        }
    }
    __syncthreads();  // H (possibly in the second stage) is read before chunk 1 is issued into it

    constexpr int VP = ZP <= 8 ? 8 : (ZP <= 16 ? 16 : 32);
    constexpr int J = 32 / VP;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    const int v = lane % VP, jj = lane / VP;
    float acc[ZP];
#pragma unroll
    for (int u = 0; u < ZP; ++u) acc[u] = 0.f;
    float r2 = 0.f;
    // A wait that gives up stops the pipeline: no copy is issued after it,
    // and the copies already issued are drained in order below.
    int k_abort = -1, last_issued = 0;
    for (int k = 0; k < nchunks; ++k) {
        if (k + 1 < nchunks) {
            if (threadIdx.x == 0) issue(k + 1);
            last_issued = k + 1;
        }
        const bool landed = umma::mbar_wait(&bar[k & 1], (uint32_t)((k >> 1) & 1));
        const float* Tc = reinterpret_cast<const float*>(stage[k & 1]);
        const float* Sc = reinterpret_cast<const float*>(stage[k & 1] + tOff);
        const int cols = min(COLS, tW - k * COLS);
        // mean removal in place (cuArraysSubtractMean) and R2; rows past the
        // template and columns past the chip stay zero
        float* Tw = reinterpret_cast<float*>(stage[k & 1]);
        for (int t = threadIdx.x; t < tH * COLS; t += blockDim.x) {
            const int c = t % COLS;
            const float val = c < cols ? Tw[t] - mean : 0.f;
            Tw[t] = val;
            r2 = fmaf(val, val, r2);
        }
        __syncthreads();
        if (v < ZP) {
            // task = (column group, band of search rows r); fewer column
            // groups than warps (narrow chunks) split the rows into bands so
            // that every warp works.  acc[u] += t(r-u) s(r+v): a band
            // [rs, re) starting on a multiple of ZP first loads the ZP-1
            // template rows above it into the ring win[r % ZP].
            const int rend = tH + ZP - 1;  // < tBoxes*tBoxRows and <= sH - 1
            const int groups = (cols + J - 1) / J;
            const int bands = max(1, nwarp / groups);
            for (int task = warp; task < groups * bands; task += nwarp) {
                const int gi = task % groups, band = task / groups;
                const int j = gi * J + jj;
                if (j >= cols) continue;
                const int rs = (int)((long long)rend * band / bands) / ZP * ZP;
                const int re = band + 1 == bands ? rend : (int)((long long)rend * (band + 1) / bands) / ZP * ZP;
                const float* tcol = Tc + j;
                const float* scol = Sc + j + v;
                float win[ZP];
#pragma unroll
                for (int kk = 0; kk < ZP; ++kk) win[kk] = 0.f;
                if (rs > 0) {
#pragma unroll
                    for (int kk = 1; kk < ZP; ++kk) win[ZP - kk] = tcol[(rs - kk) * COLS];
                }
                int r0 = rs;
                for (; r0 + ZP <= re; r0 += ZP) {
#pragma unroll
                    for (int kk = 0; kk < ZP; ++kk) {
                        const int r = r0 + kk;
                        win[kk] = tcol[r * COLS];
                        const float sv = scol[r * g.sCols];
#pragma unroll
                        for (int u = 0; u < ZP; ++u) acc[u] = fmaf(win[(kk - u + ZP) % ZP], sv, acc[u]);
                    }
                }
#pragma unroll
                for (int kk = 0; kk < ZP; ++kk) {
                    const int r = r0 + kk;
                    if (r < re) {
                        win[kk] = tcol[r * COLS];
                        const float sv = scol[r * g.sCols];
#pragma unroll
                        for (int u = 0; u < ZP; ++u) acc[u] = fmaf(win[(kk - u + ZP) % ZP], sv, acc[u]);
                    }
                }
            }
        }
        // every thread is done with this stage before it is refilled; the
        // barrier's OR makes the give-up decision the same in every thread
        if (__syncthreads_or(!landed)) {
            k_abort = k;
            break;
        }
    }
    if (k_abort >= 0) {
        // a wait gave up: record it and let the copies issued from chunk
        // k_abort on land, each stage's phases in order (bounded), before the
        // stages are reused or the block exits
        if (threadIdx.x == 0) atomicExch(err, 1);
        for (int j = k_abort; j <= last_issued; ++j) umma::mbar_wait(&bar[j & 1], (uint32_t)((j >> 1) & 1));
        __syncthreads();
    }
    const float R2 = (float)block_sum((double)r2, red);
#pragma unroll
    for (int u = 0; u < ZP; ++u) part[threadIdx.x * ZP + u] = acc[u];
    __syncthreads();
    for (int t = threadIdx.x; t < ZP * ZP; t += blockDim.x) {
        const int u = t / ZP, vv = t - (t / ZP) * ZP;
        float c = 0.f;
        for (int th = vv; th < (int)blockDim.x; th += VP) c += part[th * ZP + u];
        surf[(size_t)z * fStride + t] = c / sqrtf(var[t] * R2 + FLT_EPSILON);
    }
}
#endif

// ---------------------------------------------------------------------------
// The oversampled correlation inside the persistent kernel, its chunks staged
// by contiguous bulk copies (cp.async.bulk, one per row segment, issued by one
// warp) into two shared-memory stages, so that the copy of chunk k+1 overlaps
// the correlation of chunk k.  The chips live in the CTA's own slot, so no
// tensor map is needed.  Same arithmetic as k_corr_os_tma.
// ---------------------------------------------------------------------------
struct CosBulkGeom {
    int cols, tRows, sCols, tBytes, stageBytes;
};

__host__ __device__ inline CosBulkGeom cos_bulk_geom(const WindowPlan& P, int cols) {
    CosBulkGeom g;
    g.cols = cols;
    g.tRows = P.osWh + P.zp - 1;  // zero rows below the template end the loop without bounds checks
    g.sCols = (cols + P.zp - 1 + 3) / 4 * 4;
    g.tBytes = (int)align128((size_t)g.tRows * cols * 4);
    g.stageBytes = g.tBytes + (int)align128((size_t)P.osHz * g.sCols * 4);
    return g;
}

#ifdef AMPCOR_PART_PLAIN
size_t corr_os_bulk_smem_bytes(const WindowPlan& P, int cols, int nt) {
    const CosBulkGeom g = cos_bulk_geom(P, cols);
    const size_t part = align16((size_t)nt * P.zp * 4);
    return std::max(2 * (size_t)g.stageBytes, part) + align16((size_t)P.osHz * P.zp * 8) +
           align16((size_t)P.zp * P.zp * 4) + 40 * sizeof(double) + 32;
}
#endif

#ifdef AMPCOR_PART_PLAIN
bool corr_os_bulk_applies(const WindowPlan& P) {
    return P.osWw % 4 == 0 && P.osWz % 4 == 0 && corr_os_supported(P.zp);
}
#endif

template <int ZP>
__device__ __forceinline__ void corr_os_bulk_body(const WindowPlan& P, unsigned char* smem, float mean,
                                                  const float* __restrict__ T, const float* __restrict__ S,
                                                  float* __restrict__ sf, int* __restrict__ err) {
    const CosBulkGeom g = cos_bulk_geom(P, P.cosCols);
    const int C = g.cols;
    const int tW = P.osWw, tH = P.osWh, sW = P.osWz, sH = P.osHz;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    const size_t part_b = align16((size_t)blockDim.x * ZP * 4);
    unsigned char* stage[2] = {smem, smem + g.stageBytes};
    unsigned char* q = smem + (2 * (size_t)g.stageBytes > part_b ? 2 * (size_t)g.stageBytes : part_b);
    float2* H = reinterpret_cast<float2*>(q);   q += align16((size_t)sH * ZP * 8);
    float* var = reinterpret_cast<float*>(q);   q += align16((size_t)ZP * ZP * 4);
    double* red = reinterpret_cast<double*>(q); q += 40 * sizeof(double);
    uint64_t* bar = reinterpret_cast<uint64_t*>(q);
    float* part = reinterpret_cast<float*>(smem);  // reused after the last chunk
    const int nchunks = (tW + C - 1) / C;

    for (int t = threadIdx.x; t < (g.tRows - tH) * C; t += blockDim.x) {
        reinterpret_cast<float*>(stage[0])[tH * C + t] = 0.f;
        reinterpret_cast<float*>(stage[1])[tH * C + t] = 0.f;
    }
    if (threadIdx.x == 0) {
        umma::mbar_init(&bar[0], 1);
        umma::mbar_init(&bar[1], 1);
        tma::fence_barrier_init();
    }
    tma::fence_global_async();  // the oversampler's slot writes before the bulk reads
    __syncthreads();

    auto issue = [&](int k) {  // by warp 0
        unsigned char* st = stage[k & 1];
        const int j0 = k * C, cols = min(C, tW - j0), scols = min(g.sCols, sW - j0);
        const uint32_t tb = (uint32_t)cols * 4, sb = (uint32_t)scols * 4;
        if (lane == 0) {
            umma::fence_smem_async();  // earlier generic accesses of this stage before the async writes
            tma::arrive_expect_tx(&bar[k & 1], (uint32_t)tH * tb + (uint32_t)sH * sb);
        }
        __syncwarp();
        for (int r = lane; r < tH; r += 32)
            tma::load_bulk(st + (size_t)r * C * 4, T + (size_t)r * tW + j0, tb, &bar[k & 1]);
        for (int r = lane; r < sH; r += 32)
            tma::load_bulk(st + g.tBytes + (size_t)r * g.sCols * 4, S + (size_t)r * sW + j0, sb, &bar[k & 1]);
    };
    if (warp == 0) issue(0);

    // exact box sums of the oversampled search amplitude, overlapping the first copy
    for (int r = warp; r < sH; r += nwarp) {
        const float* row = S + (size_t)r * sW;
        const float2 h = warp_box_group([&](int j) {
            const float a = row[j];
            return make_float2(a, a * a);
        }, tW, 0, ZP);
        if (lane < ZP) H[r * ZP + lane] = h;
    }
    __syncthreads();
    {
        const double invnd = 1.0 / (double)(tH * tW);
        for (int v = warp; v < ZP; v += nwarp) {
            const float2 b = warp_box_group([&](int i) { return H[i * ZP + v]; }, tH, 0, ZP);
            if (lane < ZP) var[lane * ZP + v] = var_fp64(b.x, b.y, invnd);
        }
    }

    constexpr int VP = ZP <= 8 ? 8 : (ZP <= 16 ? 16 : 32);
    constexpr int J = 32 / VP;
    const int v = lane % VP, jj = lane / VP;
    float acc[ZP];
#pragma unroll
    for (int u = 0; u < ZP; ++u) acc[u] = 0.f;
    float r2 = 0.f;
    // A wait that gives up stops the pipeline: no copy is issued after it,
    // and the copies already issued are drained in order below.
    int k_abort = -1, last_issued = 0;
    for (int k = 0; k < nchunks; ++k) {
        if (k + 1 < nchunks) {
            if (warp == 0) issue(k + 1);
            last_issued = k + 1;
        }
        const bool landed = umma::mbar_wait(&bar[k & 1], (uint32_t)((k >> 1) & 1));
        const float* Tc = reinterpret_cast<const float*>(stage[k & 1]);
        const float* Sc = reinterpret_cast<const float*>(stage[k & 1] + g.tBytes);
        const int cols = min(C, tW - k * C);
        float* Tw = reinterpret_cast<float*>(stage[k & 1]);
        for (int t = threadIdx.x; t < tH * C; t += blockDim.x) {
            const int c = t % C;
            const float val = c < cols ? Tw[t] - mean : 0.f;
            Tw[t] = val;
            r2 = fmaf(val, val, r2);
        }
        __syncthreads();
        if (v < ZP) {
            const int rend = tH + ZP - 1;
            for (int gi = warp; gi * J < cols; gi += nwarp) {
                const int j = gi * J + jj;
                if (j >= cols) continue;
                const float* tcol = Tc + j;
                const float* scol = Sc + j + v;
                float win[ZP];
#pragma unroll
                for (int kk = 0; kk < ZP; ++kk) win[kk] = 0.f;
                int r0 = 0;
                for (; r0 + ZP <= rend; r0 += ZP) {
#pragma unroll
                    for (int kk = 0; kk < ZP; ++kk) {
                        const int r = r0 + kk;
                        win[kk] = tcol[r * C];
                        const float sv = scol[r * g.sCols];
#pragma unroll
                        for (int u = 0; u < ZP; ++u) acc[u] = fmaf(win[(kk - u + ZP) % ZP], sv, acc[u]);
                    }
                }
#pragma unroll
                for (int kk = 0; kk < ZP; ++kk) {
                    const int r = r0 + kk;
                    if (r < rend) {
                        win[kk] = tcol[r * C];
                        const float sv = scol[r * g.sCols];
#pragma unroll
                        for (int u = 0; u < ZP; ++u) acc[u] = fmaf(win[(kk - u + ZP) % ZP], sv, acc[u]);
                    }
                }
            }
        }
        if (__syncthreads_or(!landed)) {  // same decision in every thread
            k_abort = k;
            break;
        }
    }
    if (k_abort >= 0) {
        if (threadIdx.x == 0) atomicExch(err, 1);
        for (int j = k_abort; j <= last_issued; ++j) umma::mbar_wait(&bar[j & 1], (uint32_t)((j >> 1) & 1));
        __syncthreads();
    }
    const float R2 = (float)block_sum((double)r2, red);
#pragma unroll
    for (int u = 0; u < ZP; ++u) part[threadIdx.x * ZP + u] = acc[u];
    __syncthreads();
    for (int t = threadIdx.x; t < ZP * ZP; t += blockDim.x) {
        const int u = t / ZP, vv = t - (t / ZP) * ZP;
        float c = 0.f;
        for (int th = vv; th < (int)blockDim.x; th += VP) c += part[th * ZP + u];
        sf[t] = c / sqrtf(var[t] * R2 + FLT_EPSILON);
    }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

// d2 chips of d1 rows x d0 floats, chip k at base + k * pitch2 floats
// (pitch2 = 0: packed, d0 * d1)
static bool encode_3d(CUtensorMap* m, const float* base, int d0, int d1, int d2, int box0, int box1,
                      size_t pitch2 = 0) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    if (pitch2 == 0) pitch2 = (size_t)d0 * d1;
    const cuuint64_t dims[3] = {(cuuint64_t)d0, (cuuint64_t)d1, (cuuint64_t)d2};
    const cuuint64_t strides[2] = {(cuuint64_t)d0 * 4, (cuuint64_t)pitch2 * 4};
    const cuuint32_t box[3] = {(cuuint32_t)box0, (cuuint32_t)box1, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Launch the TMA-staged correlation; false if it does not apply (the caller
// then uses the plain kernel).
#ifdef AMPCOR_PART_PLAIN
// Launch k_corr_os_tma<zp, cols> (the instances that exist); false otherwise.
static bool launch_cos_tma_kernel(const WindowPlan& P, int cols, int grid, size_t sm, cudaStream_t st,
                                  const CUtensorMap& tmT, const CUtensorMap& tmS, const CosTmaGeom& g, int w0,
                                  int wend, const RawResult* res, const float* osSch, float* surf, int* err,
                                  long long sStride, long long fStride) {
#define AMPCOR_COST_CASE(Z, C)                                                                                \
    if (P.zp == Z && cols == C) {                                                                             \
        cudaFuncSetAttribute(k_corr_os_tma<Z, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);      \
        k_corr_os_tma<Z, C><<<grid, kCosTmaThreads, sm, st>>>(P, tmT, tmS, g, w0, wend, res, osSch, surf, err, \
                                                               sStride, fStride);                             \
        return true;                                                                                          \
    }
    AMPCOR_COST_CASE(8, 32)
    AMPCOR_COST_CASE(12, 32)
    AMPCOR_COST_CASE(16, 32)
    AMPCOR_COST_CASE(20, 32)
    AMPCOR_COST_CASE(24, 32)
    AMPCOR_COST_CASE(32, 32)
    AMPCOR_COST_CASE(8, 16)
    AMPCOR_COST_CASE(16, 16)
#undef AMPCOR_COST_CASE
    return false;
}

bool launch_corr_os_tma(const WindowPlan& P, int nb, cudaStream_t st, int w0, int wend, const RawResult* res,
                        const float* osRef, const float* osSch, float* surf, int* err) {
    const int cols = cos_tma_cols(P);
    if (!cols) return false;
    const CosTmaGeom g = cos_tma_geom(P, cols);
    CUtensorMap tmT, tmS;
    if (!encode_3d(&tmT, osRef, P.osWw, P.osWh, nb, cols, g.tBoxRows)) return false;
    if (!encode_3d(&tmS, osSch, P.osWz, P.osHz, nb, g.sCols, g.sBoxRows)) return false;
    const size_t sm = corr_os_tma_smem_bytes(P, cols);
    return launch_cos_tma_kernel(P, cols, nb, sm, st, tmT, tmS, g, w0, wend, res, osSch, surf, err,
                                 (long long)P.osHz * P.osWz, (long long)P.zp * P.zp);
}
#endif

#ifdef AMPCOR_PART_PLAIN
void launch_corr_os(const WindowPlan& P, int nb, cudaStream_t st, int w0, int wend, const RawResult* res,
                    const float* osRef, const float* osSch, float* surf) {
    const size_t sm = corr_os_smem_bytes(P);
    switch (P.zp) {
#define AMPCOR_COS_CASE(Z)                                                                            \
    case Z:                                                                                           \
        cudaFuncSetAttribute(k_corr_os_t<Z>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);   \
        k_corr_os_t<Z><<<nb, kCosThreads, sm, st>>>(P, w0, wend, res, osRef, osSch, surf);             \
        break;
        AMPCOR_COS_CASE(2)
        AMPCOR_COS_CASE(4)
        AMPCOR_COS_CASE(6)
        AMPCOR_COS_CASE(8)
        AMPCOR_COS_CASE(10)
        AMPCOR_COS_CASE(12)
        AMPCOR_COS_CASE(14)
        AMPCOR_COS_CASE(16)
        AMPCOR_COS_CASE(20)
        AMPCOR_COS_CASE(24)
        AMPCOR_COS_CASE(28)
        AMPCOR_COS_CASE(32)
#undef AMPCOR_COS_CASE
        default: break;
    }
}
#endif

// Oversampled correlation for any kept surface side zp (the register-blocked
// kernels above cover the even sides up to 32 except 18, 22, 26 and 30):
// one CTA per window, one thread per lag at a time, every sum read straight
// from the chips (L1/L2).  The same normalisation as the other kernels:
// c / sqrt((S2 - S1^2/n) R2 + FLT_EPSILON) with the reference chip mean
// removed (cuAmpcorChunk.cpp:148-161).
#ifdef AMPCOR_PART_PLAIN
__global__ void __launch_bounds__(256) k_corr_os_direct(const __grid_constant__ WindowPlan P, int w0, int wend,
                                                        const RawResult* __restrict__ res,
                                                        const float* __restrict__ osRef,
                                                        const float* __restrict__ osSch, float* __restrict__ surf) {
    __shared__ double red[40];
    const int w = w0 + blockIdx.x;
    if (w >= wend) return;
    const int z = w - w0, zp = P.zp, tH = P.osWh, tW = P.osWw, sW = P.osWz;
    const float* T = osRef + (size_t)z * tH * tW;
    const float* S = osSch + (size_t)z * P.osHz * sW;
    const float mean = res[w].refMean;
    float r2 = 0.f;
    for (int t = threadIdx.x; t < tH * tW; t += blockDim.x) {
        const float v = T[t] - mean;
        r2 = fmaf(v, v, r2);
    }
    const float R2 = (float)block_sum((double)r2, red);
    const double invnd = 1.0 / (double)(tH * tW);
    for (int lag = threadIdx.x; lag < zp * zp; lag += blockDim.x) {
        const int u = lag / zp, v = lag - (lag / zp) * zp;
        float c = 0.f, s1 = 0.f, s2 = 0.f;
        for (int i = 0; i < tH; ++i) {
            const float* tr = T + (size_t)i * tW;
            const float* sr = S + (size_t)(i + u) * sW + v;
            for (int j = 0; j < tW; ++j) {
                const float sv = __ldg(sr + j);
                c = fmaf(__ldg(tr + j) - mean, sv, c);
                s1 += sv;
                s2 = fmaf(sv, sv, s2);
            }
        }
        surf[(size_t)z * zp * zp + lag] = c / sqrtf(var_fp64(s1, s2, invnd) * R2 + FLT_EPSILON);
    }
}
#endif

// ---------------------------------------------------------------------------
// The oversampled correlation on the 5th-generation tensor cores (tcgen05),
// for kept surfaces of up to 16 x 16 lags.  The surface is
//   C[u][v] = sum_i sum_j T[i][j] S[i+u][j+v]
// (T: oversampled reference amplitude minus its mean, S: oversampled search
// amplitude).  For each group of 8 template rows i0 .. i0+7 one pass over
// the search columns c accumulates
//   D[(q, p)][n] += sum_c T[i0+p][c-(15-q)] S[i0+n][c]      (M = 128, N = 32)
// in tensor memory, so that C[u][15-q] = sum over all groups and p of
// D[(q, p)][p+u].  A is the template held MN-major: the 8 rows of a core
// matrix are 8 consecutive columns of T and the 16 bytes of a row hold the
// group's 8 template rows, so the 16 lag shifts q are 16-byte steps of the
// descriptor's M-group stride over one copy of T (no shifted copies).  B is
// the search chip K-major (rows n are search rows).  With split-BF16 both
// operands are split into bf16 hi + lo and D accumulates hi*hi + hi*lo +
// lo*hi in FP32.  Template and search rows stream through two shared-memory
// buffers in bands of 8*cosTcBg template rows: the threads convert band b+1
// while the tensor core consumes band b.  Box sums and normalisation are the
// FP32 kernels' (exact float box sums, the variance subtraction in FP64).
// ---------------------------------------------------------------------------
constexpr int kCosTcConv = 512;                 // converting threads (sixteen warps)
constexpr int kCosTcThreads = kCosTcConv + 32;  // + the warp that issues copies and MMAs

struct CosTcGeom {
    int G;     // 8-row template groups (template rows rounded up to 8)
    int BG;    // groups per band
    int nb;    // bands
    int sWp;   // search columns rounded up to 16: the K extent
    int nC;    // columns of the template copy: sWp + 16 (15 zero columns on the left)
    int SR;    // search rows per band: 8 BG + 24 (N = 32 rows from each group's first row)
    int ttB;   // bytes of one template part (hi or lo) of a band
    int ssB;   // bytes of one search part of a band
    int bufB;  // bytes of one operand buffer: template then search, hi then lo
    int fTB;   // bytes of a float stage's template rows (8 BG rows)
    int fB;    // bytes of one float stage: template rows, then SR search rows
    int hB;    // bytes of one band's row box sums: (8 BG + 16) rows x zp float2
};

__host__ __device__ inline CosTcGeom cos_tc_geom(const WindowPlan& P, int bg) {
    CosTcGeom g;
    const int parts = P.cosTc == 2 ? 1 : 2;
    g.G = (P.osWh + 7) / 8;
    g.BG = bg;
    g.nb = (g.G + bg - 1) / bg;
    g.sWp = (P.osWz + 15) / 16 * 16;
    g.nC = g.sWp + 16;
    g.SR = 8 * bg + 24;
    g.ttB = bg * g.nC * 16;
    g.ssB = (g.sWp / 8) * g.SR * 16;
    g.bufB = parts * (g.ttB + g.ssB);
    g.fTB = (int)align128((size_t)8 * bg * P.osWw * 4);
    g.fB = g.fTB + (int)align128((size_t)g.SR * P.osWz * 4);
    g.hB = (int)align16((size_t)(8 * bg + 16) * P.zp * 8);
    return g;
}

// two operand buffers (which the 128 x 33 accumulator staging reuses after
// the last band), two float stages, three box-sum buffers, then the tail
__host__ __device__ inline size_t cos_tc_ops_bytes(const CosTcGeom& g) {
    const size_t a = (size_t)2 * g.bufB, b = (size_t)128 * 33 * 4;
    return a > b ? a : b;
}

__host__ __device__ inline size_t corr_os_tc_smem_bytes(const WindowPlan& P, int bg) {
    const CosTcGeom g = cos_tc_geom(P, bg);
    return 128 + cos_tc_ops_bytes(g) + 2 * (size_t)g.fB + 3 * (size_t)g.hB + align16((size_t)P.zp * P.zp * 4) +
           align16((size_t)P.zp * P.zp * 8) + 40 * sizeof(double) + 128;
}

// Template groups per band for this geometry: the largest of 4, 2, 1 that
// fits; 0 if the tensor-core correlation does not apply (more than 16 x 16
// lags, or chip rows that are not whole 16-byte units, which the bulk copies
// need).
#ifdef AMPCOR_PART_PLAIN
int cos_tc_band_groups(const WindowPlan& P) {
    if (P.zp > kCosTcMaxZp || P.zp < 1) return 0;
    if (P.osWw % 4 || P.osWz % 4 || ((long long)P.osWh * P.osWw) % 4 || ((long long)P.osHz * P.osWz) % 4) return 0;
    for (int bg : {4, 2, 1})
        if (corr_os_tc_smem_bytes(P, bg) <= 232448) return bg;
    return 0;
}
#endif

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// 8 floats -> 16 bytes of bf16 hi (and lo when `split`)
__device__ __forceinline__ void split8(const float* x, bool split, uint4& hi, uint4& lo) {
    uint32_t h[4], l[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const __nv_bfloat162 hh = __floats2bfloat162_rn(x[2 * k], x[2 * k + 1]);
        h[k] = *reinterpret_cast<const uint32_t*>(&hh);
        if (split) {
            const float2 f = __bfloat1622float2(hh);
            l[k] = pack_bf16x2(x[2 * k] - f.x, x[2 * k + 1] - f.y);
        } else {
            l[k] = 0u;
        }
    }
    hi = make_uint4(h[0], h[1], h[2], h[3]);
    lo = make_uint4(l[0], l[1], l[2], l[3]);
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(umma::smem_addr(bar)) : "memory");
}

// Row box sums H[v] = sum_{j < tW} x[v + j] (S, S^2) for the lags v < G <= 16,
// two rows per warp (lanes 0-15 the first, 16-31 the second): a core shared
// by every lag, x[G-1 .. tW-1], plus a head x[v .. G-2] (suffix scan) and a
// tail x[tW .. tW+v-1] (exclusive prefix scan).  Sums of non-negative terms
// only, as warp_box_group.
__device__ __forceinline__ float2 halfwarp_box(const float* __restrict__ x, int tW, int G, bool valid) {
    const int hl = threadIdx.x & 15;
    float c1 = 0.f, c2 = 0.f;
    if (valid)
        for (int j = G - 1 + hl; j < tW; j += 16) {
            const float a = x[j];
            c1 += a;
            c2 = fmaf(a, a, c2);
        }
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) {
        c1 += __shfl_xor_sync(FULLMASK, c1, o, 16);
        c2 += __shfl_xor_sync(FULLMASK, c2, o, 16);
    }
    const bool in = valid && hl < G - 1;
    const float a = in ? x[hl] : 0.f, b = in ? x[tW + hl] : 0.f;
    float h1 = a, h2 = a * a, t1 = b, t2 = b * b;
#pragma unroll
    for (int o = 1; o < 16; o <<= 1) {  // inclusive suffix scan of the head, prefix scan of the tail
        const float p1 = __shfl_down_sync(FULLMASK, h1, o, 16), p2 = __shfl_down_sync(FULLMASK, h2, o, 16);
        const float q1 = __shfl_up_sync(FULLMASK, t1, o, 16), q2 = __shfl_up_sync(FULLMASK, t2, o, 16);
        if (hl + o < 16) { h1 += p1; h2 += p2; }
        if (hl >= o) { t1 += q1; t2 += q2; }
    }
    float e1 = __shfl_up_sync(FULLMASK, t1, 1, 16), e2 = __shfl_up_sync(FULLMASK, t2, 1, 16);
    if (hl == 0) { e1 = 0.f; e2 = 0.f; }
    return make_float2(c1 + (h1 + e1), c2 + (h2 + e2));
}

// Warp roles: warps 0-15 compute the row box sums of each band and convert
// it into operands, and warp 0 also folds each band's row box sums into the
// per-lag sums once the whole band is in; warp 16 waits for a band's
// operands, issues the copy of the band two ahead into the float stage just
// read and issues the band's MMAs (lane 0).  The tensor core's instruction rate
// (an M = 128, K = 16 MMA costs the same whatever N) bounds the kernel, so
// the issuing warp does nothing else.  Barriers: fetched[s]
// (float stage s landed), converted[o] (operand buffer o filled, float stage
// o read, box sums written), mmadone[o] (the MMAs reading buffer o
// completed).  Buffer reuse: operand buffer and float stage b & 1 and
// box-sum buffer b % 3 serve band b; a band waits for the MMAs of band b - 2,
// which follow warp 0's arrival for band b - 2, which follows its folding of
// band b - 3.  Every wait is bounded and warp-uniform; a warp whose wait
// gives up stops, the other side's waits then give up in turn, and copies
// and MMAs already issued are drained before the block exits.
// `tmem`: 32 tensor-memory columns the caller allocated for the CTA (a CTA
// allocates once: tcgen05.alloc gives up the permit to allocate again).
__device__ __forceinline__ void corr_os_tc_body(const WindowPlan& P, unsigned char* smem, uint32_t tmem, float mean,
                                                const float* __restrict__ T, const float* __restrict__ S,
                                                float* __restrict__ sf, int* __restrict__ err) {
    const CosTcGeom g = cos_tc_geom(P, P.cosTcBg);
    const int zp = P.zp, tW = P.osWw, tH = P.osWh, sW = P.osWz, sH = P.osHz;
    const bool split = P.cosTc != 2;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int NW = kCosTcConv / 32;
    const bool conv = tid < kCosTcConv;
    unsigned char* ops = smem;
    unsigned char* q = smem + cos_tc_ops_bytes(g);
    unsigned char* fst = q;                     q += 2 * (size_t)g.fB;
    float2* Hbuf = reinterpret_cast<float2*>(q); q += 3 * (size_t)g.hB;
    float* var = reinterpret_cast<float*>(q);   q += align16((size_t)zp * zp * 4);
    float2* lagacc = reinterpret_cast<float2*>(q); q += align16((size_t)zp * zp * 8);  // S1, S2 per lag
    double* red = reinterpret_cast<double*>(q); q += 40 * sizeof(double);
    uint64_t* fetched = reinterpret_cast<uint64_t*>(q);
    uint64_t* mmadone = fetched + 2;
    uint64_t* converted = fetched + 4;
    int* abortf = reinterpret_cast<int*>(fetched + 6);
    int* lastc = abortf + 1;  // last band whose MMAs were committed
    int* lastf = abortf + 2;  // last band whose copy was issued
    float* Dsm = reinterpret_cast<float*>(ops);  // accumulator rows, after the last band

    // rows of band b into float stage b & 1: template [8 BG b, +8 BG), search [8 BG b, +SR)
    auto fetch = [&](int b) {
        const int r0 = 8 * g.BG * b;
        const int tr = min(8 * g.BG, tH - r0), sr = min(g.SR, sH - r0);
        const uint32_t tb = (uint32_t)tr * tW * 4, sb = (uint32_t)sr * sW * 4;
        unsigned char* st = fst + (size_t)(b & 1) * g.fB;
        tma::arrive_expect_tx(&fetched[b & 1], tb + sb);
        tma::load_bulk(st, T + (size_t)r0 * tW, tb, &fetched[b & 1]);
        tma::load_bulk(st + g.fTB, S + (size_t)r0 * sW, sb, &fetched[b & 1]);
        *lastf = b;
    };
    if (tid == 0) {
        for (int i = 0; i < 2; ++i) {
            umma::mbar_init(&fetched[i], 1);
            umma::mbar_init(&mmadone[i], 1);
            umma::mbar_init(&converted[i], kCosTcConv);  // every converting thread arrives
        }
        *abortf = 0;
        *lastc = -1;
        *lastf = -1;
        tma::fence_barrier_init();
        for (int b = 0; b < min(2, g.nb); ++b) fetch(b);
    }
    for (int t = tid; t < zp * zp; t += blockDim.x) lagacc[t] = make_float2(0.f, 0.f);
    umma::fence_before_sync();
    __syncthreads();  // barriers initialised
    umma::fence_after_sync();
    const uint32_t idesc = umma::idesc_bf16(128, 32) | umma::kIdescAMnMajor;

    // the MMAs of band b (one thread): 8-row groups x 16-column K steps;
    // descriptors step by address offsets (16-byte units in the low field;
    // shared-memory addresses stay below 2^18)
    auto issue = [&](int b) {
        const uint32_t base = umma::smem_addr(ops + (size_t)(b & 1) * g.bufB);
        const uint64_t dth = umma::make_desc(base, 128, 16);
        const uint64_t dsh = umma::make_desc(base + (split ? 2 : 1) * g.ttB, g.SR * 16, 128);
        const uint64_t dtl = dth + (uint64_t)(g.ttB >> 4), dsl = dsh + (uint64_t)(g.ssB >> 4);
        const int gl_n = min(g.BG, g.G - b * g.BG);
        const int nk = g.sWp / 16;
        for (int gl = 0; gl < gl_n; ++gl) {
            const uint64_t a0 = (uint64_t)(gl * g.nC), b0 = (uint64_t)(gl * 8);
            for (int k = 0; k < nk; ++k) {
                const uint64_t ao = a0 + (uint64_t)(16 * k), bo = b0 + (uint64_t)(2 * g.SR * k);
                umma::mma_bf16(tmem, dth + ao, dsh + bo, idesc, (b | gl | k) != 0);
                if (split) {
                    umma::mma_bf16(tmem, dth + ao, dsl + bo, idesc, true);
                    umma::mma_bf16(tmem, dtl + ao, dsh + bo, idesc, true);
                }
            }
        }
        umma::commit(&mmadone[b & 1]);
        *lastc = b;
    };
    // fold band b's row box sums into the lag sums: lane v owns lag column v,
    // rows add in order; lag (u, v) takes rows u .. u + tH - 1, every lag the
    // rows [zp - 1, tH)
    auto fold = [&](int b, const float2* Hb, int r0, int rnew) {
        const int v = lane;
        const int fa = max(r0, zp - 1), fe = min(r0 + rnew, tH);
        float f1 = 0.f, f2 = 0.f;
        for (int r = fa; r < fe; ++r) {
            const float2 h = Hb[(r - r0) * zp + v];
            f1 += h.x;
            f2 += h.y;
        }
        for (int u = 0; u < zp; ++u) {
            float2 s = lagacc[u * zp + v];
            const int pa = max(r0, u), pe = min(r0 + rnew, u + tH);
            for (int r = pa; r < min(pe, fa); ++r) {
                const float2 h = Hb[(r - r0) * zp + v];
                s.x += h.x;
                s.y += h.y;
            }
            if (fa < fe) {
                s.x += f1;
                s.y += f2;
            }
            for (int r = max(pa, max(fe, fa)); r < pe; ++r) {
                const float2 h = Hb[(r - r0) * zp + v];
                s.x += h.x;
                s.y += h.y;
            }
            lagacc[u * zp + v] = s;
        }
    };

    float r2 = 0.f;
    if (!conv) {
        for (int b = 0; b < g.nb; ++b) {
            bool ok = true;
            if (lane == 0) ok = umma::mbar_wait_sleep(&converted[b & 1], (uint32_t)((b >> 1) & 1), 128);
            if (!__shfl_sync(FULLMASK, (int)ok, 0)) {
                if (lane == 0) atomicExch(abortf, 1);
                break;
            }
            umma::fence_after_sync();
            if (lane == 0) {
                if (b + 2 < g.nb) fetch(b + 2);  // stage b & 1 is read: refill it with band b + 2
                issue(b);
            }
            __syncwarp();
        }
    } else {
    // warp 0: once every converter has arrived for band fb, fold its row box sums
    auto fold_band = [&](int fb) -> bool {
        const bool in = umma::mbar_wait(&converted[fb & 1], (uint32_t)((fb >> 1) & 1));
        if (!__all_sync(FULLMASK, in)) {
            if (lane == 0) atomicExch(abortf, 1);
            return false;
        }
        if (lane < zp) {
            const int r0 = 8 * g.BG * fb;
            const int rnew = (fb == g.nb - 1) ? sH - r0 : min(8 * g.BG, sH - r0);
            fold(fb, reinterpret_cast<const float2*>(reinterpret_cast<const unsigned char*>(Hbuf) +
                                                     (size_t)(fb % 3) * g.hB),
                 r0, rnew);
        }
        __syncwarp();
        return true;
    };
    const FastDiv dtW((uint32_t)tW);
    const int ncg = g.sWp / 8;
    const int nB = 8 * g.BG, ovl = g.SR - nB;
    const FastDiv dnB((uint32_t)nB), dSR((uint32_t)g.SR);
    for (int b = 0; b < g.nb; ++b) {
        bool ok = umma::mbar_wait(&fetched[b & 1], (uint32_t)((b >> 1) & 1));
        // operand buffer b & 1 last served band b - 2
        if (ok && b >= 2) ok = umma::mbar_wait(&mmadone[b & 1], (uint32_t)(((b - 2) >> 1) & 1));
        if (!__all_sync(FULLMASK, ok)) {
            if (lane == 0) atomicExch(abortf, 1);
            break;
        }
        if (warp == 0 && b > 0 && !fold_band(b - 1)) break;
        const float* Tst = reinterpret_cast<const float*>(fst + (size_t)(b & 1) * g.fB);
        const float* Sst = reinterpret_cast<const float*>(fst + (size_t)(b & 1) * g.fB + g.fTB);
        float2* Hb = reinterpret_cast<float2*>(reinterpret_cast<unsigned char*>(Hbuf) + (size_t)(b % 3) * g.hB);
        const int r0 = 8 * g.BG * b;
        const int rnew = (b == g.nb - 1) ? sH - r0 : min(8 * g.BG, sH - r0);  // search rows first seen here
        // row box sums of those rows (two rows per warp)
        for (int r2w = 2 * warp; r2w < rnew; r2w += 2 * NW) {
            const int r = r2w + (lane >> 4);
            const bool valid = r < rnew;
            const float2 h = halfwarp_box(Sst + (size_t)(valid ? r : 0) * sW, tW, zp, valid);
            if (valid && (lane & 15) < zp) Hb[r * zp + (lane & 15)] = h;
        }
        // template operand [group][column c + 15][8 rows], bf16 hi (then lo);
        // the 15 zero columns on each side are written in the first use of
        // each buffer of the window
        unsigned char* B0 = ops + (size_t)(b & 1) * g.bufB;
        uint4* tth = reinterpret_cast<uint4*>(B0);
        uint4* ttl = reinterpret_cast<uint4*>(B0 + g.ttB);
        const int gl_n = min(g.BG, g.G - b * g.BG);
        if (b < 2) {
            const int npad = g.nC - tW;
            for (int t = tid; t < g.BG * npad; t += kCosTcConv) {
                const int gl = t / npad, j = t - gl * npad;
                const int c1 = j < 15 ? j : tW + j;
                tth[gl * g.nC + c1] = make_uint4(0u, 0u, 0u, 0u);
                if (split) ttl[gl * g.nC + c1] = make_uint4(0u, 0u, 0u, 0u);
            }
        }
        for (int t = tid; t < gl_n * tW; t += kCosTcConv) {
            const int gl = (int)dtW.div((uint32_t)t), c = t - gl * tW;
            const int rr = r0 + 8 * gl;
            const float* col = Tst + (size_t)(8 * gl) * tW + c;
            float x[8];
#pragma unroll
            for (int p = 0; p < 8; ++p) {
                const float val = rr + p < tH ? col[p * tW] - mean : 0.f;
                r2 = fmaf(val, val, r2);
                x[p] = val;
            }
            uint4 hi, lo;
            split8(x, split, hi, lo);
            tth[gl * g.nC + c + 15] = hi;
            if (split) ttl[gl * g.nC + c + 15] = lo;
        }
        // search operand [8-column group][row][8 columns]: the SR - 8 BG rows
        // a band shares with the next are converted once and copied into
        // the next band's buffer.  Rows [SR - 8 BG, SR) of every band are
        // converted by the same thread (item order below), which also copies
        // them on: a copy reads only what its own thread wrote, and no thread
        // overwrites a row another may still be copying.
        unsigned char* SB = B0 + (split ? 2 : 1) * (size_t)g.ttB;
        uint4* ssh = reinterpret_cast<uint4*>(SB);
        uint4* ssl = reinterpret_cast<uint4*>(SB + g.ssB);
        auto conv_row = [&](int cg, int r) {
            float x[8];
            if (r0 + r < sH) {
                const float4 a = *reinterpret_cast<const float4*>(Sst + r * sW + cg * 8);
                const float4 c = *reinterpret_cast<const float4*>(Sst + r * sW + cg * 8 + 4);
                x[0] = a.x; x[1] = a.y; x[2] = a.z; x[3] = a.w; x[4] = c.x; x[5] = c.y; x[6] = c.z; x[7] = c.w;
                if (cg * 8 + 8 > sW) {
#pragma unroll
                    for (int e = 0; e < 8; ++e)
                        if (cg * 8 + e >= sW) x[e] = 0.f;
                }
            } else {
#pragma unroll
                for (int e = 0; e < 8; ++e) x[e] = 0.f;
            }
            uint4 hi, lo;
            split8(x, split, hi, lo);
            ssh[cg * g.SR + r] = hi;
            if (split) ssl[cg * g.SR + r] = lo;
        };
        if (nB < ovl) {  // bands too short to pass rows on: convert every row
            for (int t = tid; t < ncg * g.SR; t += kCosTcConv) {
                const int cg = (int)dSR.div((uint32_t)t);
                conv_row(cg, t - cg * g.SR);
            }
        } else {
            if (b == 0)
                for (int t = tid; t < ncg * ovl; t += kCosTcConv) {
                    const int cg = t / ovl;
                    conv_row(cg, t - cg * ovl);
                }
            const uint4* psh = reinterpret_cast<const uint4*>(
                ops + (size_t)((b - 1) & 1) * g.bufB + (split ? 2 : 1) * (size_t)g.ttB);
            const uint4* psl = psh + g.ssB / 16;
            for (int t = tid; t < ncg * nB; t += kCosTcConv) {
                const int cg = (int)dnB.div((uint32_t)t), r = ovl + (t - cg * nB);
                if (b > 0 && r >= nB) {
                    const int o = cg * g.SR + r;
                    ssh[o - nB] = psh[o];
                    if (split) ssl[o - nB] = psl[o];
                }
                conv_row(cg, r);
            }
        }
        // operand writes ordered before the tensor core's reads; box sums
        // and stage reads before the fold and the next copy into the stage
        umma::fence_smem_async();
        mbar_arrive(&converted[b & 1]);
        if (warp == 0 && b == g.nb - 1) fold_band(b);
    }
    }
    __syncthreads();  // every warp done with every band (or stopped)
    if (tid == 0) {
        // drain (bounded): the MMAs (the last commit covers all) and the copies
        // issued but perhaps not consumed
        const int c = *lastc, f = *lastf;
        if (c >= 0) umma::mbar_wait(&mmadone[c & 1], (uint32_t)((c >> 1) & 1));
        for (int k = max(0, f - 1); k <= f; ++k) umma::mbar_wait(&fetched[k & 1], (uint32_t)((k >> 1) & 1));
    }
    for (int t = tid; t < zp * zp; t += blockDim.x) {
        const float2 s = lagacc[t];
        var[t] = var_fp64(s.x, s.y, 1.0 / (double)(tH * tW));
    }
    __syncthreads();
    bool ok = *abortf == 0 && *lastc == g.nb - 1;
    if (ok && warp < 4) {
        // the accumulator: MMAs complete in order, so the last band's commit covers every band
        const int b = g.nb - 1;
        const bool done = umma::mbar_wait(&mmadone[b & 1], (uint32_t)((b >> 1) & 1));
        if (__all_sync(FULLMASK, done)) {
            umma::fence_after_sync();
            float v[32];
            const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16);
            umma::tmem_ld16(ta, v);
            umma::tmem_ld16(ta + 16, v + 16);
            const int m = warp * 32 + lane;
#pragma unroll
            for (int n = 0; n < 32; ++n) Dsm[m * 33 + n] = v[n];
        } else if (lane == 0) {
            atomicExch(abortf, 1);
        }
    }
    const float R2 = (float)block_sum((double)r2, red);  // also orders the staging writes
    ok = *abortf == 0 && *lastc == g.nb - 1;
    for (int t = tid; t < zp * zp; t += blockDim.x) {
        const int u = t / zp, v = t - (t / zp) * zp;
        float c = 0.f;
#pragma unroll
        for (int p = 0; p < 8; ++p) c += Dsm[((15 - v) * 8 + p) * 33 + p + u];
        sf[t] = ok ? c / sqrtf(var[t] * R2 + FLT_EPSILON) : 0.f;
    }
    if (!ok && tid == 0) atomicExch(err, 1);
    umma::fence_before_sync();
    __syncthreads();  // accumulator reads done before the CTA's next window or its TMEM release
}

#ifdef AMPCOR_PART_PLAIN
__global__ void __launch_bounds__(kCosTcThreads, 1) k_corr_os_tc(const __grid_constant__ WindowPlan P, int w0,
                                                                 int wend, const RawResult* __restrict__ res,
                                                                 const float* __restrict__ osRef,
                                                                 const float* __restrict__ osSch,
                                                                 float* __restrict__ surf, int* __restrict__ err,
                                                                 long long tStride, long long sStride,
                                                                 long long fStride) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char* smem =
        reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~(uintptr_t)127);
    __shared__ uint32_t tbase;
    const int w = w0 + blockIdx.x;
    if (w >= wend) return;
    const int z = w - w0;
    if (threadIdx.x < 32) umma::tmem_alloc(&tbase, 32);
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    corr_os_tc_body(P, smem, tbase, res[w].refMean, osRef + (size_t)z * tStride, osSch + (size_t)z * sStride,
                    surf + (size_t)z * fStride, err);
    if (threadIdx.x < 32) umma::tmem_free(tbase, 32);
}

bool launch_corr_os_tc(const WindowPlan& P, int nb, cudaStream_t st, int w0, int wend, const RawResult* res,
                       const float* osRef, const float* osSch, float* surf, int* err, long long tStride,
                       long long sStride, long long fStride) {
    if (!P.cosTc || !P.cosTcBg || P.zp > kCosTcMaxZp) return false;
    const size_t sm = corr_os_tc_smem_bytes(P, P.cosTcBg);
    cudaFuncSetAttribute(k_corr_os_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_corr_os_tc<<<nb, kCosTcThreads, sm, st>>>(P, w0, wend, res, osRef, osSch, surf, err, tStride, sStride,
                                                fStride);
    return true;
}
#endif

#ifdef AMPCOR_PART_PLAIN
void launch_corr_os_best(const WindowPlan& P, int nb, cudaStream_t st, int w0, int wend, const RawResult* res,
                         const float* osRef, const float* osSch, float* surf, int* err) {
    if (launch_corr_os_tc(P, nb, st, w0, wend, res, osRef, osSch, surf, err, (long long)P.osWh * P.osWw,
                          (long long)P.osHz * P.osWz, (long long)P.zp * P.zp))
        return;
    if (!corr_os_supported(P.zp)) {
        k_corr_os_direct<<<nb, 256, 0, st>>>(P, w0, wend, res, osRef, osSch, surf);
        return;
    }
    if (!launch_corr_os_tma(P, nb, st, w0, wend, res, osRef, osSch, surf, err))
        launch_corr_os(P, nb, st, w0, wend, res, osRef, osSch, surf);
}
#endif

#ifdef AMPCOR_PART_PLAIN
bool corr_os_supported(int zp) {
    switch (zp) {
        case 2: case 4: case 6: case 8: case 10: case 12: case 14: case 16: case 20: case 24: case 28: case 32:
            return true;
        default:
            return false;
    }
}
#endif

// ---------------------------------------------------------------------------
// Correlation-surface zoom.  The reference oversamples the zp x zp surface to
// M x M = (zoom*ovs)^2 by spectral zero padding and scans every point
// (cuOverSampler.cpp:141-148, cuAmpcorChunk.cpp:194).  Here the same
// trigonometric interpolant y(m,n) = Re sum X[c1][c2] e^{-2pi i (f1 m + f2 n)/M}
// is evaluated on a coarse grid of step s, and only the cells that can hold
// the maximum are evaluated at every point: |dy/dm| <= Lm and |dy/dn| <= Ln with
// Lm = 2pi/M sum |X| |f1| (likewise Ln), so no point of a cell exceeds the
// largest corner by more than (Lm + Ln) s/2; and since the bilinear
// interpolant of the corners peaks at a corner and is within
// s^2/8 (|y_mm| + |y_nn|) of y, nor by more than s^2/8 (2pi/M)^2 sum |X|
// (f1^2 + f2^2), the tighter of the two near a smooth peak.  A margin of
// 1e-5 sum|X| covers float32 evaluation error, so the arg-max (with the
// reference's tie order) is the one a full scan finds.
// ---------------------------------------------------------------------------

// nt: threads of the CTA that runs the body (one scratch block per warp)
#ifdef AMPCOR_PART_PLAIN
size_t zoom_smem_bytes(const WindowPlan& P, int nt) {
    if (P.method == 1) {
        const int n = 4 * P.ovs + 1;
        return align16((size_t)P.zp * P.zp * 4) + 4 * align16((size_t)n * kSincLen * 4) + 80 * 8 + 16;
    }
    const int Z = P.zoom, Zc = 2 * (Z / 2), Mc = P.M / P.zs, s1 = P.zs + 1;
    const int nw = nt / 32;
    return align16((size_t)Z * Z * 4) + align16((size_t)Zc * Zc * 8) + align16((size_t)Z * Z * 8) +
           align16((size_t)Z * 8) + 2 * align16((size_t)Mc * Zc * 8) + align16((size_t)s1 * Zc * 8) +
           2 * align16((size_t)Mc * Mc * 4) + align16((size_t)nw * 3 * s1 * Zc * 8) + 80 * 8 + 16;
}
#endif

// Outputs of one window once the arg-max (bv, bi) of its zoomed surface is
// known: cuSubPixelOffset_kernel (cuOffset.cu:137-146), the gross-offset merge
// (cuAmpcorController.cpp:145-150) and the raw-stage SNR and covariance.
__device__ __forceinline__ void zoom_write(const WindowPlan& P, const RawResult& r, const WindowCoords& wc, float bv,
                                           int bi, int merge_gross, float2* __restrict__ off_w,
                                           float* __restrict__ snr_w, float* __restrict__ cov_w,
                                           int* __restrict__ diag_w) {
    if (threadIdx.x != 0) return;
    const int M = P.M;
    if (bi < 0) bi = 0;
    const int mx = bi / M, my = bi - (bi / M) * M;
    float ox = __fmaf_rn(P.osratio, (float)mx, (float)r.startX) - (float)P.hsD;
    float oy = __fmaf_rn(P.osratio, (float)my, (float)r.startY) - (float)P.hsA;
    if (merge_gross) {
        ox += (float)(wc.secD - wc.refD + P.hsD);
        oy += (float)(wc.secA - wc.refA + P.hsA);
    }
    *off_w = make_float2(ox, oy);
    *snr_w = r.snr;
    cov_w[0] = r.covxx;
    cov_w[1] = r.covyy;
    cov_w[2] = r.covxy;
    if (diag_w) {
        diag_w[0] = r.locX; diag_w[1] = r.locY;
        diag_w[2] = r.startX; diag_w[3] = r.startY;
        diag_w[4] = mx; diag_w[5] = my;
        diag_w[6] = __float_as_int(r.maxval);
        diag_w[7] = __float_as_int(bv);
    }
}

// Coefficient k of the reference's Hamming-weighted sinc kernel
// (cuSincOverSampler.cu:40-63 with the constants of cuSincOverSampler.h:30-45:
// beta 0.75, relative length 6, 4096 phases, pedestal 0), evaluated with the
// same float operations in the same order.
__device__ __forceinline__ float sinc_coef(int k) {
    const float pi = 3.14159265359f;
    const float soff = ((float)(kSincLen * kSincPhases) - 1.0f) / 2.0f;
    const float wa = (float)k - soff;
    const float wgt = (1.0f - 0.5f) + 0.5f * cosf(pi * wa * (1.0f / soff));
    const float sarg = wa * 0.75f * (1.0f / (float)kSincPhases) * pi;
    const float fct = sarg != 0.0f ? sinf(sarg) / sarg : 1.0f;
    return fct * wgt;
}

// Sinc oversampling of the zp x zp surface and the arg-max of the M x M
// result (corrSurfaceOverSamplingMethod = 1, cuSincOverSamplerR2R::execute,
// cuSincOverSampler.cu:168-195 and kernel :83-160; arg-max of
// cuAmpcorChunk.cpp:194).  The reference zeroes the M x M output, then
// interpolates only the (4 ovs + 1)^2 points around the centre moved by the
// zoom-start shift times ovs*raw (wrapping once past M), each a weighted
// 8 x 8 sum over the surface with wrapped indices (the wrap past the end of
// a row subtracts the row length, as there) divided by the sum of the
// weights.  The arg-max therefore runs over those points and the zeros
// elsewhere; the zeros are only scanned when no interpolated value is
// positive.
__device__ inline void sinc_zoom_argmax(const WindowPlan& P, unsigned char* smem, const RawResult& r,
                                 const float* __restrict__ sf, float& bv_out, int& bi_out) {
    const int zp = P.zp, M = P.M, ovs = P.ovs, n = 4 * ovs + 1;
    const int start = M / 2 - 2 * ovs, factor = ovs * P.raw;
    unsigned char* q = smem;
    float* x = reinterpret_cast<float*>(q);    q += align16((size_t)zp * zp * 4);
    float* cx = reinterpret_cast<float*>(q);   q += align16((size_t)n * kSincLen * 4);
    int* ix = reinterpret_cast<int*>(q);       q += align16((size_t)n * kSincLen * 4);
    float* cy = reinterpret_cast<float*>(q);   q += align16((size_t)n * kSincLen * 4);
    int* iy = reinterpret_cast<int*>(q);       q += align16((size_t)n * kSincLen * 4);
    float* redv = reinterpret_cast<float*>(q);
    int* redi = reinterpret_cast<int*>(redv + 40);
    for (int t = threadIdx.x; t < zp * zp; t += blockDim.x) x[t] = sf[t];
    // per output row (and column): its 8 input rows and their coefficients
    for (int t = threadIdx.x; t < 2 * n; t += blockDim.x) {
        const bool col = t >= n;
        const int i = col ? t - n : t;
        int o = i + start + (col ? r.shiftY : r.shiftX) * factor;
        if (o >= M) o -= M;
        const float ro = __fdiv_rn((float)o, (float)ovs);
        const int io = (int)ro;
        const int frac = (int)((ro - (float)io) * (float)kSincPhases);
        float* c = col ? cy : cx;
        int* id = col ? iy : ix;
        for (int k = 0; k < kSincLen; ++k) {
            int in = io - k + kSincLen / 2;
            if (in < 0) in += zp;
            if (in >= zp) in -= zp;
            c[i * kSincLen + k] = sinc_coef(k * kSincPhases + frac);
            id[i * kSincLen + k] = in;
        }
    }
    __syncthreads();
    float bv = -INFINITY;
    int bi = -1;
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
        const int a = t / n, b = t - (t / n) * n;
        float acc = 0.0f, wsum = 0.0f;
        for (int k = 0; k < kSincLen; ++k) {
            const float c1 = cx[a * kSincLen + k];
            const float* row = x + ix[a * kSincLen + k] * zp;
            for (int l = 0; l < kSincLen; ++l) {
                const float w = c1 * cy[b * kSincLen + l];
                wsum += w;
                acc += row[iy[b * kSincLen + l]] * w;
            }
        }
        const float y = acc / wsum;
        int ox = a + start + r.shiftX * factor, oy = b + start + r.shiftY * factor;
        if (ox >= M) ox -= M;
        if (oy >= M) oy -= M;
        const int idx = ox * M + oy;
        if (y >= bv && (y > bv || better(y, idx, bv, bi))) { bv = y; bi = idx; }
    }
    block_argmax(bv, bi, redv, redi);
    if (!(bv > 0.0f)) {
        // the zeros outside the interpolated points take part in the arg-max
        const int x0 = start + r.shiftX * factor, y0 = start + r.shiftY * factor;
        float zv = -INFINITY;
        int zi = -1;
        for (int t = threadIdx.x; t < M * M; t += blockDim.x) {
            const int a = t / M, b = t - (t / M) * M;
            int da = a - x0, db = b - y0;
            if (da < 0) da += M;
            if (db < 0) db += M;
            if (da < n && db < n) continue;
            if (better(0.0f, t, zv, zi)) { zv = 0.0f; zi = t; }
        }
        block_argmax(zv, zi, redv, redi);
        if (zi >= 0 && better(0.0f, zi, bv, bi)) { bv = 0.0f; bi = zi; }
    }
    bv_out = bv;
    bi_out = bi;
}

// Surface zoom, arg-max and outputs of one window; `r` holds its raw-stage
// results and `sf` its zp x zp oversampled surface.
__device__ __forceinline__ void zoom_body(const WindowPlan& P, unsigned char* smem, const RawResult r,
                                          const WindowCoords wc, const float* __restrict__ sf, int merge_gross,
                                          float2* __restrict__ off_w, float* __restrict__ snr_w,
                                          float* __restrict__ cov_w, int* __restrict__ diag_w) {
    if (P.method == 1) {
        float bv;
        int bi;
        sinc_zoom_argmax(P, smem, r, sf, bv, bi);
        zoom_write(P, r, wc, bv, bi, merge_gross, off_w, snr_w, cov_w, diag_w);
        return;
    }
    const int Z = P.zoom, zp = P.zp, M = P.M, h = Z / 2, Zc = 2 * h, s = P.zs, Mc = M / s, s1 = s + 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    unsigned char* q = smem;
    float* x = reinterpret_cast<float*>(q);            q += align16((size_t)Z * Z * 4);
    cfloat* Xc = reinterpret_cast<cfloat*>(q);         q += align16((size_t)Zc * Zc * 8);
    cfloat* A = reinterpret_cast<cfloat*>(q);          q += align16((size_t)Z * Z * 8);
    cfloat* rz = reinterpret_cast<cfloat*>(q);         q += align16((size_t)Z * 8);
    cfloat* EcT = reinterpret_cast<cfloat*>(q);        q += align16((size_t)Mc * Zc * 8);  // [c][a]
    cfloat* Pc = reinterpret_cast<cfloat*>(q);         q += align16((size_t)Mc * Zc * 8);
    cfloat* Ef = reinterpret_cast<cfloat*>(q);         q += align16((size_t)s1 * Zc * 8);
    float* Yc = reinterpret_cast<float*>(q);           q += align16((size_t)Mc * Mc * 4);
    int* cand = reinterpret_cast<int*>(q);             q += align16((size_t)Mc * Mc * 4);
    cfloat* wsc = reinterpret_cast<cfloat*>(q);        q += align16((size_t)nw * 3 * s1 * Zc * 8);
    double* red = reinterpret_cast<double*>(q);
    float* redv = reinterpret_cast<float*>(red + 40);
    int* redi = reinterpret_cast<int*>(redv + 40);
    int* ncand = redi + 40;

    // zero-padded zp x zp surface (cuArraysCopyPadded) and its inverse-sign DFT
    for (int t = threadIdx.x; t < Z * Z; t += blockDim.x) {
        const int i = t / Z, j = t - (t / Z) * Z;
        x[t] = (i < zp && j < zp) ? sf[i * zp + j] : 0.f;
    }
    for (int t = threadIdx.x; t < Z; t += blockDim.x) rz[t] = unit_root(t, Z, +1);
    if (threadIdx.x == 0) *ncand = 0;
    __syncthreads();
    for (int t = threadIdx.x; t < Z * Z; t += blockDim.x) {
        const int i = t / Z, k = t - (t / Z) * Z;
        cfloat acc = {0.f, 0.f};
        int e = 0;
        for (int j = 0; j < Z; ++j) {
            acc = cadd(acc, cscale(rz[e], x[i * Z + j]));
            e += k;
            if (e >= Z) e -= Z;
        }
        A[t] = acc;
    }
    __syncthreads();
    // compact spectrum over the kept signed frequencies f(c) = c < h ? c : c - Zc,
    // scaled by 1/Z^2 (cuArraysPaddingMany), plus the derivative bounds
    const float inv = 1.0f / ((float)Z * (float)Z);
    float labs = 0.f, lmf = 0.f, lnf = 0.f, lqf = 0.f;
    for (int t = threadIdx.x; t < Zc * Zc; t += blockDim.x) {
        const int c1 = t / Zc, c2 = t - (t / Zc) * Zc;
        const int k1 = c1 < h ? c1 : c1 - Zc + Z, k2 = c2 < h ? c2 : c2 - Zc + Z;
        cfloat acc = {0.f, 0.f};
        int e = 0;
        for (int i = 0; i < Z; ++i) {
            acc = cadd(acc, cmul(A[i * Z + k2], rz[e]));
            e += k1;
            if (e >= Z) e -= Z;
        }
        acc = cscale(acc, inv);
        Xc[t] = acc;
        const float a = sqrtf(acc.x * acc.x + acc.y * acc.y);
        const float f1 = (float)(c1 < h ? c1 : c1 - Zc), f2 = (float)(c2 < h ? c2 : c2 - Zc);
        labs += a;
        lmf += a * fabsf(f1);
        lnf += a * fabsf(f2);
        lqf += a * (f1 * f1 + f2 * f2);
    }
    const double sabs = block_sum((double)labs, red);
    const double slm = block_sum((double)lmf, red);
    const double sln = block_sum((double)lnf, red);
    const double slq = block_sum((double)lqf, red);
    // Bound of the surface inside a coarse cell of side s (fine-grid steps of
    // 2 pi / M radians per unit frequency) above the largest of its corners:
    // first order, the Lipschitz constant times the distance to the nearest
    // corner, pi s / M * sum |X| (|f1| + |f2|); second order, the bilinear
    // interpolant of the corners (its maximum is a corner) is within
    // s^2 / 8 (|g_xx| + |g_yy|) <= s^2 / 8 (2 pi / M)^2 sum |X| (f1^2 + f2^2)
    // of the surface.  Both hold; the smaller prunes more cells.  1e-5 of the
    // spectrum's l1 norm covers float32 rounding of the evaluated points.
    const double kPi = 3.14159265358979323846;
    const double m1 = (slm + sln) * kPi / M * s;
    const double m2 = (double)s * s / 8.0 * (2.0 * kPi / M) * (2.0 * kPi / M) * slq;
    const float margin = (float)((m1 < m2 ? m1 : m2) + 1e-5 * sabs);

    // twiddles of the coarse grid (column-major: neighbouring lanes read
    // neighbouring coarse columns) and of the offsets inside a cell
    for (int t = threadIdx.x; t < Mc * Zc; t += blockDim.x) {
        const int c = t / Mc, a = t - (t / Mc) * Mc;
        EcT[t] = unit_root((long long)(c < h ? c : c - Zc) * a * s, M, -1);
    }
    for (int t = threadIdx.x; t < s1 * Zc; t += blockDim.x) {
        const int j = t / Zc, c = t - (t / Zc) * Zc;
        Ef[t] = unit_root((long long)(c < h ? c : c - Zc) * j, M, -1);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < Mc * Zc; t += blockDim.x) {
        const int a = t / Zc, c2 = t - (t / Zc) * Zc;
        cfloat acc = {0.f, 0.f};
        for (int c1 = 0; c1 < Zc; ++c1) acc = cadd(acc, cmul(Xc[c1 * Zc + c2], EcT[c1 * Mc + a]));
        Pc[t] = acc;
    }
    __syncthreads();
    // coarse grid
    float bv = -INFINITY;
    int bi = -1;
    for (int t = threadIdx.x; t < Mc * Mc; t += blockDim.x) {
        const int a = t / Mc, b = t - (t / Mc) * Mc;
        const cfloat* pr = Pc + a * Zc;
        float y = 0.f;
        for (int c = 0; c < Zc; ++c) {
            const cfloat e = EcT[c * Mc + b];
            y = fmaf(pr[c].x, e.x, y);
            y = fmaf(-pr[c].y, e.y, y);
        }
        Yc[t] = y;
        const int idx = (a * s) * M + b * s;
        if (y >= bv && (y > bv || better(y, idx, bv, bi))) { bv = y; bi = idx; }
    }
    block_argmax(bv, bi, redv, redi);  // also publishes Yc
    const float best = bv;
    // cells whose bound reaches the coarse maximum
    for (int t = threadIdx.x; t < Mc * Mc; t += blockDim.x) {
        const int a = t / Mc, b = t - (t / Mc) * Mc;
        const int a1 = a + 1 < Mc ? a + 1 : 0, b1 = b + 1 < Mc ? b + 1 : 0;
        const float ub = fmaxf(fmaxf(Yc[t], Yc[a1 * Mc + b]), fmaxf(Yc[a * Mc + b1], Yc[a1 * Mc + b1])) + margin;
        if (ub >= best || isnan(ub)) cand[atomicAdd(ncand, 1)] = t;
    }
    __syncthreads();
    const int nc = *ncand;
    // every point of the candidate cells, one warp per cell
    cfloat* Erow = wsc + (size_t)warp * 3 * s1 * Zc;
    cfloat* Ecol = Erow + s1 * Zc;
    cfloat* Prow = Ecol + s1 * Zc;
    for (int ci = warp; ci < nc; ci += nw) {
        const int cell = cand[ci];
        const int a = cell / Mc, b = cell - (cell / Mc) * Mc;
        // per-cell tables, column-major ([c][offset]) for conflict-free reads
        for (int t = lane; t < s1 * Zc; t += 32) {
            const int c = t / s1, j = t - (t / s1) * s1;
            Erow[t] = cmul(EcT[c * Mc + a], Ef[j * Zc + c]);
            Ecol[t] = cmul(EcT[c * Mc + b], Ef[j * Zc + c]);
        }
        __syncwarp();
        for (int t = lane; t < s1 * Zc; t += 32) {
            const int i = t / Zc, c2 = t - (t / Zc) * Zc;
            cfloat acc = {0.f, 0.f};
            for (int c1 = 0; c1 < Zc; ++c1) acc = cadd(acc, cmul(Xc[c1 * Zc + c2], Erow[c1 * s1 + i]));
            Prow[c2 * s1 + i] = acc;
        }
        __syncwarp();
        for (int t = lane; t < s1 * s1; t += 32) {
            const int i = t / s1, j = t - (t / s1) * s1;
            float y = 0.f;
            for (int c = 0; c < Zc; ++c) {
                const cfloat pv = Prow[c * s1 + i], ev = Ecol[c * s1 + j];
                y = fmaf(pv.x, ev.x, y);
                y = fmaf(-pv.y, ev.y, y);
            }
            int m = a * s + i, n = b * s + j;
            if (m >= M) m -= M;
            if (n >= M) n -= M;
            const int idx = m * M + n;
            if (y >= bv && (y > bv || better(y, idx, bv, bi))) { bv = y; bi = idx; }
        }
        __syncwarp();
    }
    block_argmax(bv, bi, redv, redi);
    zoom_write(P, r, wc, bv, bi, merge_gross, off_w, snr_w, cov_w, diag_w);
}

#ifdef AMPCOR_PART_PLAIN
__global__ void __launch_bounds__(kZoomThreads) k_zoom(const __grid_constant__ WindowPlan P, int w0, int wend,
                                                       const RawResult* __restrict__ res,
                                                       const WindowCoords* __restrict__ coords,
                                                       const float* __restrict__ surf, int merge_gross,
                                                       float2* __restrict__ offset, float* __restrict__ snr,
                                                       float* __restrict__ cov, int* __restrict__ diag) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int w = w0 + blockIdx.x;
    if (w >= wend) return;
    zoom_body(P, smem, res[w], coords[w], surf + (size_t)(w - w0) * P.zp * P.zp, merge_gross, offset + w, snr + w,
              cov + 3 * (size_t)w, diag ? diag + 8 * (size_t)w : nullptr);
}
#endif


// ---------------------------------------------------------------------------
// Persistent batched kernel.  Windows of many jobs, each with its own
// geometry, come from one global work queue (an atomic counter over a list
// ordered by decreasing cost); a CTA runs all four stages of a window and
// keeps the intermediates (box-sum scratch, oversampled chips, oversampled
// surface, raw results) in its own scratch slot, small enough to stay in L2.
// ---------------------------------------------------------------------------
#ifdef AMPCOR_PART_PLAIN
size_t batch_smem_bytes(const WindowPlan& P, int nt) {
    size_t m = P.rawL2 ? raw_l2_smem_bytes(P) : raw_smem_bytes(P);
    m = std::max(m, P.osL2 ? os2_l2_smem_bytes(P) : os2_applies(P) ? os2_smem_bytes(P) : os_smem_bytes(P));
    m = std::max(m, P.cosCols ? corr_os_bulk_smem_bytes(P, P.cosCols, nt) : corr_os_smem_bytes(P, nt));
    m = std::max(m, zoom_smem_bytes(P, nt));
    return m;
}
#endif

// Move the raw tile, then the oversampler chips, to L2-staged slots until
// every stage body fits `limit` bytes of shared memory in a CTA of nt
// threads.  Returns false if even that does not fit.
#ifdef AMPCOR_PART_PLAIN
bool fit_plan_smem(WindowPlan& P, int nt, size_t limit) {
    if (batch_smem_bytes(P, nt) <= limit) return true;
    if (!P.rawL2) {
        P.rawL2 = 1;
        P.rawGl = 32;
        while (P.rawGl > 2 && raw_l2_smem_bytes(P) > limit) P.rawGl -= 2;
        if (batch_smem_bytes(P, nt) <= limit) return true;
    }
    if (!P.osL2 && os2_applies(P)) {
        P.osL2 = 1;
        P.osGl = 32;
        while (P.osGl > 2 && os2_l2_smem_bytes(P) > limit) P.osGl -= 2;
    }
    return batch_smem_bytes(P, nt) <= limit;
}
#endif

// Stage the oversampled correlation by bulk copies when its double buffer
// fits `limit` bytes of shared memory (32-column chunks, else 16).
#ifdef AMPCOR_PART_PLAIN
void plan_enable_bulk_corr(WindowPlan& P, int nt, size_t limit) {
    P.cosCols = 0;
    if (!corr_os_bulk_applies(P)) return;
    for (int c : {32, 16}) {
        P.cosCols = c;
        if (batch_smem_bytes(P, nt) <= limit) return;
    }
    P.cosCols = 0;
}
#endif

#ifdef AMPCOR_PART_PLAIN
SlotLayout batch_slot_layout(const WindowPlan* plans, int n) {
    size_t v = 0, t = 0, o = 0, r = 0, s2 = 0, f = 0;
    for (int i = 0; i < n; ++i) {
        const WindowPlan& P = plans[i];
        if (P.osL2) o = std::max(o, os2_l2_slot_bytes(P));
        if (P.rawL2)
            t = std::max(t, raw_l2_slot_bytes(P));
        else
            v = std::max(v, (size_t)P.NX * P.Ws * sizeof(float2));
        r = std::max(r, (size_t)P.osWh * P.osWw * sizeof(float));
        s2 = std::max(s2, (size_t)P.osHz * P.osWz * sizeof(float));
        f = std::max(f, (size_t)P.zp * P.zp * sizeof(float));
    }
    SlotLayout L;
    size_t off = 0;
    auto take = [&](size_t b) { size_t o = off; off += (b + 255) & ~(size_t)255; return o; };
    L.vbox = take(v);
    L.rawl2 = take(t);
    L.osl2 = take(o);
    L.osRef = take(r);
    L.osSch = take(s2);
    L.surf = take(f);
    L.res = take(sizeof(RawResult));
    L.bytes = off;
    return L;
}
#endif

#ifdef AMPCOR_PART_PERSIST
template <int NT, int MINB, bool BULK>
__global__ void __launch_bounds__(NT, MINB) k_persist(const BatchJob* __restrict__ jobs, const int2* __restrict__ items,
                                                   int nitems, int* __restrict__ next,
                                                   unsigned char* __restrict__ scratch, const SlotLayout L) {
    int* err = next + 1;  // device error word: a bounded wait gave up
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ WindowPlan Ps;
    __shared__ int it_s;
    unsigned char* slot = scratch + (size_t)blockIdx.x * L.bytes;
    float2* V = reinterpret_cast<float2*>(slot + L.vbox);
    float* oR = reinterpret_cast<float*>(slot + L.osRef);
    float* oS = reinterpret_cast<float*>(slot + L.osSch);
    float* sf = reinterpret_cast<float*>(slot + L.surf);
    RawResult* rw = reinterpret_cast<RawResult*>(slot + L.res);
    for (;;) {
        if (threadIdx.x == 0) it_s = atomicAdd(next, 1);
        __syncthreads();
        const int it = it_s;
        if (it >= nitems) break;
        const int2 wi = items[it];
        const BatchJob* J = jobs + wi.x;
        {
            const int* src = reinterpret_cast<const int*>(&J->P);
            int* dst = reinterpret_cast<int*>(&Ps);
            for (int k = threadIdx.x; k < (int)(sizeof(WindowPlan) / sizeof(int)); k += blockDim.x) dst[k] = src[k];
        }
        __syncthreads();
        const WindowCoords wc = J->coords[wi.y];
        if (Ps.rawL2)
            raw_l2_body(Ps, smem, J->ref, J->ldr, J->sec, J->lds, wc, slot + L.rawl2, rw);
        else
            raw_body<0>(Ps, smem, J->ref, J->ldr, J->sec, J->lds, wc, V, rw);
        __syncthreads();
        if (Ps.osL2) {
            cfloat* X = reinterpret_cast<cfloat*>(slot + L.osl2);
            os2_l2_body(Ps, smem, 0, J->ref, J->ldr, J->sec, J->lds, wc, rw, X, oR);
            __syncthreads();
            os2_l2_body(Ps, smem, 1, J->ref, J->ldr, J->sec, J->lds, wc, rw, X, oS);
        } else if (os2_applies(Ps)) {
            os2_body<0>(Ps, smem, 0, J->ref, J->ldr, J->sec, J->lds, wc, rw, oR);
            __syncthreads();
            os2_body<0>(Ps, smem, 1, J->ref, J->ldr, J->sec, J->lds, wc, rw, oS);
        } else {
            os_body<0>(Ps, smem, 0, J->ref, J->ldr, J->sec, J->lds, wc, rw, oR);
            __syncthreads();
            os_body<0>(Ps, smem, 1, J->ref, J->ldr, J->sec, J->lds, wc, rw, oS);
        }
        __syncthreads();
        const float mean = rw->refMean;
        switch (Ps.zp) {
#define AMPCOR_PERSIST_COS(Z)                                           \
    case Z:                                                             \
        if (BULK && Ps.cosCols)                                         \
            corr_os_bulk_body<Z>(Ps, smem, mean, oR, oS, sf, err);      \
        else                                                            \
            corr_os_body<Z>(Ps, smem, mean, oR, oS, sf);                \
        break;
            AMPCOR_PERSIST_COS(2)
            AMPCOR_PERSIST_COS(4)
            AMPCOR_PERSIST_COS(6)
            AMPCOR_PERSIST_COS(8)
            AMPCOR_PERSIST_COS(10)
            AMPCOR_PERSIST_COS(12)
            AMPCOR_PERSIST_COS(14)
            AMPCOR_PERSIST_COS(16)
            AMPCOR_PERSIST_COS(20)
            AMPCOR_PERSIST_COS(24)
            AMPCOR_PERSIST_COS(28)
            AMPCOR_PERSIST_COS(32)
#undef AMPCOR_PERSIST_COS
            default: break;
        }
        __syncthreads();
        zoom_body(Ps, smem, *rw, wc, sf, J->merge, J->offset + wi.y, J->snr + wi.y, J->cov + 3 * (size_t)wi.y,
                  nullptr);
        __syncthreads();
    }
}
#endif

// Launch shapes: 512 threads x 1 CTA per SM, 256 x 1 (more registers per
// thread), 256 x 2 (registers capped at 128 so two CTAs fit).  Each shape is
// compiled in its own translation unit (AMPCOR_PERSIST_SHAPE 0, 1, 2).
#ifdef AMPCOR_PART_PERSIST
#if AMPCOR_PERSIST_SHAPE == 0
#define AMPCOR_PNT 512
#define AMPCOR_PMINB 1
#define AMPCOR_PLAUNCH launch_persist_512x1
#define AMPCOR_POCC persist_occupancy_512x1
#elif AMPCOR_PERSIST_SHAPE == 1
#define AMPCOR_PNT 256
#define AMPCOR_PMINB 1
#define AMPCOR_PLAUNCH launch_persist_256x1
#define AMPCOR_POCC persist_occupancy_256x1
#else
#define AMPCOR_PNT 256
#define AMPCOR_PMINB 2
#define AMPCOR_PLAUNCH launch_persist_256x2
#define AMPCOR_POCC persist_occupancy_256x2
#endif
cudaError_t AMPCOR_PLAUNCH(int grid, size_t smem, cudaStream_t st, const BatchJob* jobs, const int2* items,
                           int nitems, int* next, unsigned char* scratch, const SlotLayout& L) {
    const void* f = (const void*)k_persist<AMPCOR_PNT, AMPCOR_PMINB, false>;
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_persist<AMPCOR_PNT, AMPCOR_PMINB, false><<<grid, AMPCOR_PNT, smem, st>>>(jobs, items, nitems, next, scratch, L);
    return cudaGetLastError();
}

int AMPCOR_POCC(size_t smem) {
    int n = 0;
    const void* f = (const void*)k_persist<AMPCOR_PNT, AMPCOR_PMINB, false>;
    if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f, AMPCOR_PNT, smem) != cudaSuccess) return 0;
    return n;
}
#endif

#ifdef AMPCOR_PART_PLAIN
cudaError_t launch_persist(int nt, int per_sm, int grid, size_t smem, cudaStream_t st, const BatchJob* jobs,
                           const int2* items, int nitems, int* next, unsigned char* scratch, const SlotLayout& L) {
    if (nt == 256 && per_sm >= 2) return launch_persist_256x2(grid, smem, st, jobs, items, nitems, next, scratch, L);
    if (nt == 256) return launch_persist_256x1(grid, smem, st, jobs, items, nitems, next, scratch, L);
    return launch_persist_512x1(grid, smem, st, jobs, items, nitems, next, scratch, L);
}

int persist_blocks_per_sm(int nt, int per_sm, size_t smem) {
    if (nt == 256 && per_sm >= 2) return persist_occupancy_256x2(smem);
    if (nt == 256) return persist_occupancy_256x1(smem);
    return persist_occupancy_512x1(smem);
}
#endif

// ---------------------------------------------------------------------------
// Batched chain: the four stages as four persistent kernels over a wave of
// (job, window) items, each with its own launch shape (the plain chain's
// thread counts and occupancy).  A wave spans at most kWavePlans distinct
// jobs, whose plans travel in the launch parameters (constant bank, like the
// plain kernels' plan: no shared-memory copy that the transforms' stores
// would force the compiler to reload).  The intermediates of a wave (raw
// results, oversampled chips, surfaces) live in a wave workspace, the
// L2-staged tiles in per-CTA slots.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int wave_slot(const WavePlans& WP, int job) {
    int s = 0;
    for (int k = 1; k < WP.count; ++k)
        if (WP.job[k] == job) s = k;
    return s;
}

// Every wave is homogeneous in its code path (raw tile placement, oversampler
// body, oversampled lag count, bulk-copied correlation): the kernels are
// instantiated per path, so each carries only its own body and register
// allocation, as the plain kernels do.
#ifdef AMPCOR_PART_WAVE
template <int L2>
__global__ void __launch_bounds__(kWaveRawThreads) k_wave_raw(const __grid_constant__ WavePlans WP,
                                                              const BatchJob* __restrict__ jobs,
                                                              const int2* __restrict__ items, int i0, int n,
                                                              const WaveLayout W) {
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned char* slot = W.slots + (size_t)blockIdx.x * W.slotBytes;
    for (int b = blockIdx.x; b < n; b += gridDim.x) {
        const int2 wi = items[i0 + b];
        const BatchJob* J = jobs + wi.x;
        const WindowPlan& P = WP.P[wave_slot(WP, wi.x)];
        const WindowCoords wc = J->coords[wi.y];
        if (b + gridDim.x < n) {  // this CTA's next window
            const int2 wj = items[i0 + b + gridDim.x];
            const BatchJob* Jn = jobs + wj.x;
            const WindowPlan& Pn = WP.P[wave_slot(WP, wj.x)];
            const WindowCoords c = Jn->coords[wj.y];
            prefetch_chip_l2(Jn->ref + (long long)c.refD * Jn->ldr + c.refA, Jn->ldr, Pn.Wh, Pn.Ww);
            prefetch_chip_l2(Jn->sec + (long long)c.secD * Jn->lds + c.secA, Jn->lds, Pn.Hs, Pn.Ws);
        }
        if (L2)
            raw_l2_body(P, smem, J->ref, J->ldr, J->sec, J->lds, wc, slot + W.L.rawl2, &W.res[b]);
        else
            raw_body<0>(P, smem, J->ref, J->ldr, J->sec, J->lds, wc, reinterpret_cast<float2*>(slot + W.L.vbox),
                     &W.res[b]);
        __syncthreads();
    }
}
#endif

// V: 0 separable raw=2 oversampler, 1 its L2-staged form, 2 any raw factor
#ifdef AMPCOR_PART_WAVE
template <int V>
__global__ void __launch_bounds__(kWaveOsThreads, 2) k_wave_os(const __grid_constant__ WavePlans WP,
                                                               const BatchJob* __restrict__ jobs,
                                                               const int2* __restrict__ items, int i0, int n,
                                                               const WaveLayout W) {
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned char* slot = W.slots + (size_t)blockIdx.x * W.slotBytes;
    for (int t = blockIdx.x; t < 2 * n; t += gridDim.x) {
        const int b = t >> 1, which = t & 1;
        const int2 wi = items[i0 + b];
        const BatchJob* J = jobs + wi.x;
        const WindowPlan& P = WP.P[wave_slot(WP, wi.x)];
        const WindowCoords wc = J->coords[wi.y];
        // the chip this CTA takes next, or (one CTA per chip, two per SM,
        // starting in index order) the CTA that follows it on the SM
        const int tn = gridDim.x >= 2 * n ? t + 2 * sm_count() : t + gridDim.x;
        if (tn < 2 * n) {
            const int bn = tn >> 1;
            const int2 wj = items[i0 + bn];
            const BatchJob* Jn = jobs + wj.x;
            const WindowPlan& Pn = WP.P[wave_slot(WP, wj.x)];
            const WindowCoords c = Jn->coords[wj.y];
            if (tn & 1) {
                const RawResult r = W.res[bn];
                prefetch_chip_l2(Jn->sec + (long long)(c.secD + r.startX) * Jn->lds + (c.secA + r.startY), Jn->lds,
                                 Pn.Hz, Pn.Wz);
            } else {
                prefetch_chip_l2(Jn->ref + (long long)c.refD * Jn->ldr + c.refA, Jn->ldr, Pn.Wh, Pn.Ww);
            }
        }
        float* out = which ? W.osSch + (size_t)b * W.osSchStride : W.osRef + (size_t)b * W.osRefStride;
        if (V == 1)
            os2_l2_body(P, smem, which, J->ref, J->ldr, J->sec, J->lds, wc, &W.res[b],
                        reinterpret_cast<cfloat*>(slot + W.L.osl2), out);
        else if (V == 0)
            os2_body<0>(P, smem, which, J->ref, J->ldr, J->sec, J->lds, wc, &W.res[b], out);
        else
            os_body<0>(P, smem, which, J->ref, J->ldr, J->sec, J->lds, wc, &W.res[b], out);
        __syncthreads();
    }
}
#endif

#ifdef AMPCOR_PART_WAVE
template <int ZP, bool BULK>
__global__ void __launch_bounds__(kWaveCosThreads) k_wave_cos(const __grid_constant__ WavePlans WP,
                                                              const int2* __restrict__ items, int i0, int n,
                                                              const WaveLayout W, int* __restrict__ err) {
    extern __shared__ __align__(16) unsigned char smem[];
    for (int b = blockIdx.x; b < n; b += gridDim.x) {
        const int2 wi = items[i0 + b];
        const WindowPlan& P = WP.P[wave_slot(WP, wi.x)];
        const float mean = W.res[b].refMean;
        const float* oR = W.osRef + (size_t)b * W.osRefStride;
        const float* oS = W.osSch + (size_t)b * W.osSchStride;
        float* sf = W.surf + (size_t)b * W.surfStride;
        if (BULK)
            corr_os_bulk_body<ZP>(P, smem, mean, oR, oS, sf, err);
        else
            corr_os_body<ZP>(P, smem, mean, oR, oS, sf);
        __syncthreads();
    }
}
#endif

// the tensor-core oversampled correlation over a wave of mixed geometry
#ifdef AMPCOR_PART_WAVE
__global__ void __launch_bounds__(kCosTcThreads, 1) k_wave_cos_tc(const __grid_constant__ WavePlans WP,
                                                                  const int2* __restrict__ items, int i0, int n,
                                                                  const WaveLayout W, int* __restrict__ err) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char* smem =
        reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~(uintptr_t)127);
    __shared__ uint32_t tbase;
    if (blockIdx.x >= n) return;
    if (threadIdx.x < 32) umma::tmem_alloc(&tbase, 32);  // once per CTA, for all its windows
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    for (int b = blockIdx.x; b < n; b += gridDim.x) {
        const int2 wi = items[i0 + b];
        const WindowPlan& P = WP.P[wave_slot(WP, wi.x)];
        corr_os_tc_body(P, smem, tbase, W.res[b].refMean, W.osRef + (size_t)b * W.osRefStride,
                        W.osSch + (size_t)b * W.osSchStride, W.surf + (size_t)b * W.surfStride, err);
        __syncthreads();
    }
    if (threadIdx.x < 32) umma::tmem_free(tbase, 32);
}
#endif

#ifdef AMPCOR_PART_WAVE
__global__ void __launch_bounds__(kWaveZoomThreads, 2) k_wave_zoom(const __grid_constant__ WavePlans WP,
                                                                   const BatchJob* __restrict__ jobs,
                                                                   const int2* __restrict__ items, int i0, int n,
                                                                   const WaveLayout W) {
    extern __shared__ __align__(16) unsigned char smem[];
    for (int b = blockIdx.x; b < n; b += gridDim.x) {
        const int2 wi = items[i0 + b];
        const BatchJob* J = jobs + wi.x;
        const WindowPlan& P = WP.P[wave_slot(WP, wi.x)];
        const WindowCoords wc = J->coords[wi.y];
        zoom_body(P, smem, W.res[b], wc, W.surf + (size_t)b * W.surfStride, J->merge, J->offset + wi.y,
                  J->snr + wi.y, J->cov + 3 * (size_t)wi.y, nullptr);
        __syncthreads();
    }
}
#endif

// Code path of a plan in the chain: (raw L2, oversampler body, lag count,
// bulk-copied correlation); waves never mix paths.
#ifdef AMPCOR_PART_WAVE
int wave_path_key(const WindowPlan& P) {
    const int osv = P.osL2 ? 1 : os2_applies(P) ? 0 : 2;
    return (P.rawL2 ? 1 : 0) | (osv << 1) | (P.zp << 3) | ((P.cosCols ? 1 : 0) << 10) | (P.cosTc << 11);
}
#endif

static constexpr bool bulk_zp(int zp) { return zp == 8 || zp == 12 || zp == 16 || zp == 20 || zp == 24 || zp == 32; }

#ifdef AMPCOR_PART_WAVE
static const void* wave_fn(int stage, const WindowPlan& P) {
    switch (stage) {
        case 0: return P.rawL2 ? (const void*)k_wave_raw<1> : (const void*)k_wave_raw<0>;
        case 1: return P.osL2 ? (const void*)k_wave_os<1>
                              : os2_applies(P) ? (const void*)k_wave_os<0> : (const void*)k_wave_os<2>;
        case 2:
            if (P.cosTc) return (const void*)k_wave_cos_tc;
            switch (P.zp) {
#define AMPCOR_WAVE_COS_FN(Z) \
    case Z: return (P.cosCols && bulk_zp(Z)) ? (const void*)k_wave_cos<Z, bulk_zp(Z)> : (const void*)k_wave_cos<Z, false>;
                AMPCOR_WAVE_COS_FN(2)
                AMPCOR_WAVE_COS_FN(4)
                AMPCOR_WAVE_COS_FN(6)
                AMPCOR_WAVE_COS_FN(8)
                AMPCOR_WAVE_COS_FN(10)
                AMPCOR_WAVE_COS_FN(12)
                AMPCOR_WAVE_COS_FN(14)
                AMPCOR_WAVE_COS_FN(16)
                AMPCOR_WAVE_COS_FN(20)
                AMPCOR_WAVE_COS_FN(24)
                AMPCOR_WAVE_COS_FN(28)
                AMPCOR_WAVE_COS_FN(32)
#undef AMPCOR_WAVE_COS_FN
                default: return nullptr;
            }
        default: return (const void*)k_wave_zoom;
    }
}
#endif

// Shared memory of one chain stage for a plan (the stage's own body only).
#ifdef AMPCOR_PART_WAVE
size_t wave_stage_smem(const WindowPlan& P, int stage) {
    switch (stage) {
        case 0: return P.rawL2 ? raw_l2_smem_bytes(P) : raw_smem_bytes(P);
        case 1: return P.osL2 ? os2_l2_smem_bytes(P) : os2_applies(P) ? os2_smem_bytes(P) : os_smem_bytes(P);
        case 2: return P.cosTc     ? corr_os_tc_smem_bytes(P, P.cosTcBg)
                       : P.cosCols ? corr_os_bulk_smem_bytes(P, P.cosCols, kWaveCosThreads)
                                   : corr_os_smem_bytes(P, kWaveCosThreads);
        default: return zoom_smem_bytes(P, kWaveZoomThreads);
    }
}
#endif

#ifdef AMPCOR_PART_WAVE
static int wave_threads(int stage, const WindowPlan& P) {
    const int nt[4] = {kWaveRawThreads, kWaveOsThreads, P.cosTc ? kCosTcThreads : kWaveCosThreads,
                       kWaveZoomThreads};
    return nt[stage];
}
#endif

#ifdef AMPCOR_PART_WAVE
int wave_blocks_per_sm(int stage, const WindowPlan& P, size_t smem) {
    int n = 0;
    const void* f = wave_fn(stage, P);
    if (!f) return 0;
    if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f, wave_threads(stage, P), smem) != cudaSuccess)
        return 0;
    return n;
}
#endif

// The chain's oversampled correlation of a single-geometry wave through the
// TMA-staged kernel (tensor maps over the wave workspace); false if it does
// not apply.
#ifdef AMPCOR_PART_PLAIN
bool launch_wave_cos_tma(const WindowPlan& P, int n, cudaStream_t st, const WaveLayout& W, int* err) {
    if (launch_corr_os_tc(P, n, st, 0, n, W.res, W.osRef, W.osSch, W.surf, err, (long long)W.osRefStride,
                          (long long)W.osSchStride, (long long)W.surfStride))
        return true;
    const int cols = cos_tma_cols(P);
    if (!cols) return false;
    if ((W.osRefStride * 4) % 16 || (W.osSchStride * 4) % 16) return false;
    const CosTmaGeom g = cos_tma_geom(P, cols);
    CUtensorMap tmT, tmS;
    if (!encode_3d(&tmT, W.osRef, P.osWw, P.osWh, n, cols, g.tBoxRows, W.osRefStride)) return false;
    if (!encode_3d(&tmS, W.osSch, P.osWz, P.osHz, n, g.sCols, g.sBoxRows, W.osSchStride)) return false;
    const size_t sm = corr_os_tma_smem_bytes(P, cols);
    return launch_cos_tma_kernel(P, cols, n, sm, st, tmT, tmS, g, 0, n, W.res, W.osSch, W.surf, err,
                                 (long long)W.osSchStride, (long long)W.surfStride);
}
#endif

// P: any plan of the wave (all share its code path).
#ifdef AMPCOR_PART_WAVE
cudaError_t launch_wave_stage(int stage, int grid, size_t smem, cudaStream_t st, const WavePlans& WP,
                              const BatchJob* jobs, const int2* items, int i0, int n, const WaveLayout& W,
                              int* err) {
    const WindowPlan& P = WP.P[0];
    const void* f = wave_fn(stage, P);
    if (!f) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    switch (stage) {
        case 0:
            if (P.rawL2) k_wave_raw<1><<<grid, kWaveRawThreads, smem, st>>>(WP, jobs, items, i0, n, W);
            else k_wave_raw<0><<<grid, kWaveRawThreads, smem, st>>>(WP, jobs, items, i0, n, W);
            break;
        case 1:
            if (P.osL2) k_wave_os<1><<<grid, kWaveOsThreads, smem, st>>>(WP, jobs, items, i0, n, W);
            else if (os2_applies(P)) k_wave_os<0><<<grid, kWaveOsThreads, smem, st>>>(WP, jobs, items, i0, n, W);
            else k_wave_os<2><<<grid, kWaveOsThreads, smem, st>>>(WP, jobs, items, i0, n, W);
            break;
        case 2: {
            void* args[] = {(void*)&WP, (void*)&items, (void*)&i0, (void*)&n, (void*)&W, (void*)&err};
            e = cudaLaunchKernel(f, dim3(grid), dim3(wave_threads(2, P)), args, smem, st);
            if (e != cudaSuccess) return e;
            break;
        }
        default: k_wave_zoom<<<grid, kWaveZoomThreads, smem, st>>>(WP, jobs, items, i0, n, W); break;
    }
    return cudaGetLastError();
}
#endif

// ---------------------------------------------------------------------------
// Host planning of the batched chain: cut a (job, window) work list into
// waves (homogeneous code path, at most kWavePlans jobs, intermediates within
// `budget`), with per stage the shared memory of the largest body and the
// grid that fills the GPU at that occupancy.
// ---------------------------------------------------------------------------
#ifdef AMPCOR_PART_WAVE
size_t ChainPlan::bytes() const {
    const size_t res_b = ((size_t)nmax * sizeof(RawResult) + 255) & ~(size_t)255;
    return res_b + (size_t)nmax * (osr + oss + sf) * sizeof(float) + (size_t)maxGrid01 * slotBytes;
}
#endif

#ifdef AMPCOR_PART_WAVE
bool plan_chain(const std::vector<WindowPlan>& plans, const std::vector<int2>& items, int sms, size_t budget,
                ChainPlan* out, std::string* err, bool by_geometry) {
    ChainPlan& C = *out;
    size_t v = 0, t = 0, o = 0;
    C.osr = C.oss = C.sf = 0;
    for (const WindowPlan& P : plans) {
        C.osr = std::max(C.osr, (size_t)P.osWh * P.osWw);
        C.oss = std::max(C.oss, (size_t)P.osHz * P.osWz);
        C.sf = std::max(C.sf, (size_t)P.zp * P.zp);
        if (P.rawL2)
            t = std::max(t, raw_l2_slot_bytes(P));
        else
            v = std::max(v, (size_t)P.NX * P.Ws * sizeof(float2));
        if (P.osL2) o = std::max(o, os2_l2_slot_bytes(P));
    }
    auto r64 = [](size_t f) { return (f + 63) & ~(size_t)63; };  // 256-byte aligned item strides
    C.osr = r64(C.osr);
    C.oss = r64(C.oss);
    C.sf = r64(C.sf);
    const size_t per_item = (C.osr + C.oss + C.sf) * sizeof(float) + sizeof(RawResult);
    const int nw = (int)std::max<size_t>((size_t)sms * 4, std::min<size_t>(items.size(), budget / per_item));
    C.waves.clear();
    C.maxGrid01 = 1;
    C.nmax = 0;
    std::vector<char> seen(plans.size(), 0);
    for (int i0 = 0; i0 < (int)items.size();) {
        ChainWave w{};
        w.i0 = i0;
        w.plans.count = 0;
        std::fill(seen.begin(), seen.end(), 0);
        int i = i0;
        for (; i < (int)items.size() && i - i0 < nw; ++i) {
            const int j = items[i].x;
            if (seen[j]) continue;
            // a new job opens a new wave when the wave is full of plans or
            // the job's code path differs
            if (w.plans.count == kWavePlans ||
                (w.plans.count > 0 && wave_path_key(plans[j]) != wave_path_key(w.plans.P[0])))
                break;
            if (by_geometry && w.plans.count > 0) {
                const WindowPlan &A = w.plans.P[0], &B = plans[j];
                if (A.osWh != B.osWh || A.osWw != B.osWw || A.osHz != B.osHz || A.osWz != B.osWz) break;
            }
            seen[j] = 1;
            w.plans.job[w.plans.count] = j;
            w.plans.P[w.plans.count] = plans[j];
            w.plans.count += 1;
            for (int s = 0; s < 4; ++s) w.smem[s] = std::max(w.smem[s], wave_stage_smem(plans[j], s));
        }
        w.n = i - i0;
        i0 = i;
        w.single_geometry = true;
        for (int k = 1; k < w.plans.count; ++k) {
            const WindowPlan &A = w.plans.P[0], &B = w.plans.P[k];
            if (A.osWh != B.osWh || A.osWw != B.osWw || A.osHz != B.osHz || A.osWz != B.osWz || A.zp != B.zp)
                w.single_geometry = false;
        }
        for (int s = 0; s < 4; ++s) {
            const int occ = w.smem[s] <= 232448 ? wave_blocks_per_sm(s, w.plans.P[0], w.smem[s]) : 0;
            if (occ < 1) {
                if (err) *err = "chain stage " + std::to_string(s) + " does not fit (" + std::to_string(w.smem[s]) +
                                " bytes of shared memory)";
                return false;
            }
            const int work = s == 1 ? 2 * w.n : w.n;
            // the oversampler without an L2 slot takes one CTA per chip, as
            // the plain chain does (no per-CTA state to keep resident)
            w.grid[s] = (s == 1 && !w.plans.P[0].osL2) ? work : std::max(1, std::min(work, sms * occ));
        }
        C.maxGrid01 = std::max(C.maxGrid01, std::max(w.grid[0], w.plans.P[0].osL2 ? w.grid[1] : 0));
        C.nmax = std::max(C.nmax, w.n);
        C.waves.push_back(w);
    }
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t q = off; off += (bytes + 255) & ~(size_t)255; return q; };
    C.L = SlotLayout{};
    C.L.vbox = take(v);
    C.L.rawl2 = take(t);
    C.L.osl2 = take(o);
    C.L.bytes = off;
    C.slotBytes = std::max<size_t>(C.L.bytes, 256);
    return true;
}
#endif

#ifdef AMPCOR_PART_WAVE
void chain_layout(const ChainPlan& C, unsigned char* base, WaveLayout* out) {
    WaveLayout& W = *out;
    const size_t res_b = ((size_t)C.nmax * sizeof(RawResult) + 255) & ~(size_t)255;
    unsigned char* q = base;
    W.res = reinterpret_cast<RawResult*>(q);
    q += res_b;
    W.osRef = reinterpret_cast<float*>(q);
    q += (size_t)C.nmax * C.osr * sizeof(float);
    W.osSch = reinterpret_cast<float*>(q);
    q += (size_t)C.nmax * C.oss * sizeof(float);
    W.surf = reinterpret_cast<float*>(q);
    q += (size_t)C.nmax * C.sf * sizeof(float);
    W.slots = q;
    W.osRefStride = C.osr;
    W.osSchStride = C.oss;
    W.surfStride = C.sf;
    W.slotBytes = C.slotBytes;
    W.L = C.L;
}
#endif

#ifdef AMPCOR_PART_WAVE
cudaError_t launch_chain(const ChainPlan& C, const WaveLayout& W, const BatchJob* jobs, const int2* items,
                         cudaStream_t st, int* err, const ChainTimer* timer) {
    for (const ChainWave& w : C.waves)
        for (int s = 0; s < 4; ++s) {
            if (timer) {
                const cudaError_t e = timer->begin(s, st);
                if (e != cudaSuccess) return e;
            }
            // a wave of one geometry correlates its oversampled chips with the
            // TMA-staged kernel, as the plain chain does
            if (!(s == 2 && w.single_geometry && launch_wave_cos_tma(w.plans.P[0], w.n, st, W, err))) {
                const cudaError_t e =
                    launch_wave_stage(s, w.grid[s], w.smem[s], st, w.plans, jobs, items, w.i0, w.n, W, err);
                if (e != cudaSuccess) return e;
            }
            if (timer) {
                const cudaError_t e = timer->end(s, st);
                if (e != cudaSuccess) return e;
            }
        }
    return cudaSuccess;
}
#endif

}  // namespace ampcor
