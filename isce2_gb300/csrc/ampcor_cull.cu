// Offset-field post-processing on the device: outlier culling of an offset
// field (ISCE2's Offoutliers, components/isceobj/Util/offoutliers), the
// offset-polynomial fit (stdproc/offsetpoly) and the nearest-neighbour
// decimation of full-resolution rasters onto the offset
// grid (contrib/PyCuAmpcor/examples/cuDenseOffsets.py:400-460,
// prepareGeometry through GDAL's Translate).
//
// Culling, as offoutliers.F:53-127 defines it:
//   1. optional SNR pre-cull (Offoutliers.py:268-276 through
//      OffsetField.cull, isceobj/Location/Offset.py:364-378: an offset is
//      kept unless its SNR is below the threshold);
//   2. two weighted straight-line fits, across shift against across location
//      and down shift against down location (svdfit, offoutliers.F:165-215:
//      basis (1, location), weights 1/sig, singular values below 1e-6 of the
//      largest dropped, the minimum-norm solution otherwise);
//   3. slope and intercept stored as REAL*4, the perpendicular distance of
//      every point to its line in Fortran's mixed REAL*4 / REAL*8 arithmetic
//      (offoutliers.F:97-118), kept where both distances are within
//      `distance`, indices in input order.
//
// Layout: five FP64 arrays (locations, shifts, sigmas) and one FP32 SNR
// array of n points, read twice (the fit sums, then the distances) and a
// one-byte flag array; every block owns one contiguous chunk, so the kept
// indices come out in input order without a sort.  The fit sums are FP64
// normal equations of the 2-column design matrix; their 2 x 2
// eigen-decomposition gives the singular values the reference thresholds.
// Reductions run in a fixed order (per-block trees, then blocks in order),
// so results are identical run to run.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <string>

#include "ampcor_gb.h"

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxBlocks = 1024;
constexpr int kSums = 9;

thread_local std::string g_field_err;

int field_fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_field_err = buf;
    return code;
}

__device__ __forceinline__ bool snr_kept(const float* snr, double thr, int64_t i) {
    return snr == nullptr || !((double)snr[i] < thr);
}

// the block's contiguous chunk [b0, b1)
__device__ __forceinline__ void chunk_of(int64_t n, int64_t chunk, int64_t& b0, int64_t& b1) {
    b0 = (int64_t)blockIdx.x * chunk;
    b1 = b0 + chunk < n ? b0 + chunk : n;
}

// Per-block FP64 sums of the two fits' normal equations: U rows (w, w x),
// right side w z, w = 1 / sig (offoutliers.F:166-174).  s[0] = sum w^2
// (shared), across: s[1] = sum w^2 x, s[2] = sum w^2 x^2, s[3] = sum w^2 z,
// s[4] = sum w^2 x z; down: s[5..8] the same.
__global__ void __launch_bounds__(kThreads) k_cull_sums(const double* __restrict__ xa, const double* __restrict__ za,
                                                        const double* __restrict__ xd, const double* __restrict__ zd,
                                                        const double* __restrict__ sig, const float* __restrict__ snr,
                                                        double thr, int64_t n, int64_t chunk,
                                                        double* __restrict__ part) {
    double s[kSums];
#pragma unroll
    for (int k = 0; k < kSums; ++k) s[k] = 0.0;
    int64_t b0, b1;
    chunk_of(n, chunk, b0, b1);
    for (int64_t i = b0 + threadIdx.x; i < b1; i += kThreads) {
        if (!snr_kept(snr, thr, i)) continue;
        const double w = sig ? 1.0 / sig[i] : 1.0;
        const double ua = w * xa[i], ba = za[i] * w, ud = w * xd[i], bd = zd[i] * w;
        s[0] += w * w;
        s[1] += w * ua;
        s[2] += ua * ua;
        s[3] += w * ba;
        s[4] += ua * ba;
        s[5] += w * ud;
        s[6] += ud * ud;
        s[7] += w * bd;
        s[8] += ud * bd;
    }
    __shared__ double red[kWarps][kSums];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < kSums; ++k) {
        double v = s[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < kSums) {
        double v = 0.0;
        for (int w = 0; w < kWarps; ++w) v += red[w][threadIdx.x];
        part[(size_t)blockIdx.x * kSums + threadIdx.x] = v;
    }
}

// Least-squares line z = c0 + c1 x from the normal matrix [a b; b c] = U^T U
// and right side (r0, r1) = U^T z: the singular values of U are the square
// roots of the eigenvalues; one below tol times the largest is dropped
// (offoutliers.F:190-199, tol the REAL*4 constant 1e-6), which leaves the
// minimum-norm solution along the leading eigenvector.
__device__ void solve_line(double a, double b, double c, double r0, double r1, double* coef) {
    const double tol = (double)1e-6f;
    const double h = 0.5 * (a - c), m = 0.5 * (a + c);
    const double lmax = m + sqrt(h * h + b * b);
    if (!(lmax > 0.0)) {  // no points with weight: svbksb skips every zero singular value
        coef[0] = 0.0;
        coef[1] = 0.0;
        return;
    }
    const double det = a * c - b * b;
    const double lmin = det > 0.0 ? det / lmax : 0.0;
    if (sqrt(lmin) >= tol * sqrt(lmax)) {
        coef[0] = (c * r0 - b * r1) / det;
        coef[1] = (a * r1 - b * r0) / det;
        return;
    }
    // eigenvector of lmax: (lmax - c, b) or (b, lmax - a), the longer one
    double v0, v1;
    if (fabs(lmax - c) >= fabs(lmax - a)) {
        v0 = lmax - c;
        v1 = b;
    } else {
        v0 = b;
        v1 = lmax - a;
    }
    const double nv = sqrt(v0 * v0 + v1 * v1);
    v0 /= nv;
    v1 /= nv;
    const double p = (v0 * r0 + v1 * r1) / lmax;
    coef[0] = v0 * p;
    coef[1] = v1 * p;
}

// one thread: add the block sums in block order, fit both lines, store the
// REAL*4 slope / intercept pairs (offoutliers.F:67-68,84-85)
__global__ void k_cull_fit(const double* __restrict__ part, int nb, float* __restrict__ fit32,
                           double* __restrict__ fit64, float* __restrict__ avg_across, float* __restrict__ avg_down) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s[kSums];
    for (int k = 0; k < kSums; ++k) s[k] = 0.0;
    for (int b = 0; b < nb; ++b)
        for (int k = 0; k < kSums; ++k) s[k] += part[(size_t)b * kSums + k];
    double ca[2], cd[2];
    solve_line(s[0], s[1], s[2], s[3], s[4], ca);
    solve_line(s[0], s[5], s[6], s[7], s[8], cd);
    fit32[0] = (float)ca[0];  // cac
    fit32[1] = (float)ca[1];  // slpac
    fit32[2] = (float)cd[0];  // cdn
    fit32[3] = (float)cd[1];  // slpdn
    if (fit64) {
        fit64[0] = ca[0];
        fit64[1] = ca[1];
        fit64[2] = cd[0];
        fit64[3] = cd[1];
    }
    if (avg_across) *avg_across = fit32[0];
    if (avg_down) *avg_down = fit32[2];
}

// Perpendicular distance of (loc, shift) to shift = slp loc + c as
// offoutliers.F:98-103 evaluates it: REAL*4 slope, intercept, foot point x
// and y; real*8 locations, shifts and the mixed-mode intermediates; the
// distance rounded to REAL*4.  Every operation is rounded on its own (no
// fused multiply-adds), as the reference's x86-64 build computes it.
__device__ __forceinline__ float line_distance(double loc, double shift, float slp, float c) {
    const float p1 = __fmul_rn(slp, c);                                              // slp*c       REAL*4
    const double t = __dadd_rn(__dadd_rn(loc, -(double)p1), __dmul_rn((double)slp, shift));  // loc - p1 + slp*shift
    const float den = __fadd_rn(1.0f, __fmul_rn(slp, slp));                          // 1 + slp**2  REAL*4
    const float x = __double2float_rn(__ddiv_rn(t, (double)den));
    const float y = __fadd_rn(__fmul_rn(slp, x), c);
    const double dx = __dadd_rn((double)x, -loc), dy = __dadd_rn((double)y, -shift);
    return __double2float_rn(__dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy))));
}

__global__ void __launch_bounds__(kThreads) k_cull_flags(const double* __restrict__ xa, const double* __restrict__ za,
                                                         const double* __restrict__ xd, const double* __restrict__ zd,
                                                         const float* __restrict__ snr, double thr, float distance,
                                                         const float* __restrict__ fit32, int64_t n, int64_t chunk,
                                                         uint8_t* __restrict__ flags, int* __restrict__ bcount) {
    const float cac = fit32[0], slpac = fit32[1], cdn = fit32[2], slpdn = fit32[3];
    int64_t b0, b1;
    chunk_of(n, chunk, b0, b1);
    int cnt = 0;
    for (int64_t i = b0 + threadIdx.x; i < b1; i += kThreads) {
        bool keep = snr_kept(snr, thr, i);
        if (keep) {
            const float dac = line_distance(xa[i], za[i], slpac, cac);
            const float ddn = line_distance(xd[i], zd[i], slpdn, cdn);
            keep = dac <= distance && ddn <= distance;
        }
        flags[i] = keep ? 1 : 0;
        cnt += keep ? 1 : 0;
    }
    __shared__ int red[kWarps];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < kWarps; ++w) t += red[w];
        bcount[blockIdx.x] = t;
    }
}

// exclusive offsets of the blocks' kept counts, and the total (one thread)
__global__ void k_cull_offsets(const int* __restrict__ bcount, int nb, int* __restrict__ boff,
                               int32_t* __restrict__ count_out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int t = 0;
    for (int b = 0; b < nb; ++b) {
        boff[b] = t;
        t += bcount[b];
    }
    *count_out = t;
}

// kept indices in input order: tiles of kThreads consecutive points, each
// placed by a block-wide exclusive scan of the flags
__global__ void __launch_bounds__(kThreads) k_cull_scatter(const uint8_t* __restrict__ flags, int64_t n, int64_t chunk,
                                                           const int* __restrict__ boff,
                                                           int32_t* __restrict__ index_out) {
    __shared__ int wsum[kWarps];
    int64_t b0, b1;
    chunk_of(n, chunk, b0, b1);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int base = boff[blockIdx.x];
    for (int64_t t0 = b0; t0 < b1; t0 += kThreads) {
        const int64_t i = t0 + threadIdx.x;
        const bool f = i < b1 && flags[i] != 0;
        const unsigned m = __ballot_sync(0xffffffffu, f);
        if (lane == 0) wsum[warp] = __popc(m);
        __syncthreads();
        int before = 0, total = 0;
        for (int w = 0; w < kWarps; ++w) {
            if (w < warp) before += wsum[w];
            total += wsum[w];
        }
        if (f) index_out[base + before + __popc(m & ((1u << lane) - 1u))] = (int32_t)i;
        base += total;
        __syncthreads();  // wsum reused by the next tile
    }
}

// dst[i][j] = src[y0 + i*ystep + ystep/2][x0 + j*xstep + xstep/2], zero
// outside the source (GDAL's nearest-neighbour sampling of a source window
// of rows*ystep x cols*xstep onto rows x cols takes the pixel under each
// output pixel's centre; noData = 0)
template <typename T>
__global__ void k_decimate(const T* __restrict__ src, int64_t src_rows, int64_t src_cols, int64_t src_ld, int64_t y0,
                           int64_t x0, int64_t ystep, int64_t xstep, T* __restrict__ dst, int64_t rows,
                           int64_t cols) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= cols) return;
    const int64_t sx = x0 + j * xstep + xstep / 2;
    for (int64_t i = (int64_t)blockIdx.y * blockDim.y + threadIdx.y; i < rows; i += (int64_t)gridDim.y * blockDim.y) {
        const int64_t sy = y0 + i * ystep + ystep / 2;
        T v = T(0);
        if (sy >= 0 && sy < src_rows && sx >= 0 && sx < src_cols) v = src[sy * src_ld + sx];
        dst[i * cols + j] = v;
    }
}

// ---------------------------------------------------------------------------
// Offset polynomial (stdproc/offsetpoly: offsetpoly.f90:53-84 with svdfit,
// resampLib/src/svd.f:1-40, and poly_funcs.f90): the weighted least-squares
// fit of an offset as the first `ma` of 1, x, y, x y, x^2, y^2, x y^2, x^2 y,
// x^3, y^3 (x = across location, y = down location), weights 1 / (1 + 1/snr),
// singular values of the design matrix below 1e-12 of the largest dropped.
//
// The design matrix U (n x ma) of unscaled locations is far too ill
// conditioned for normal equations (x^3 reaches 1e12), so the device works
// in centred, scaled locations xs = (x - x0) / Lx, ys = (y - y0) / Ly:
// U = U_s A with A the exact change of polynomial basis.  The FP64 Gram
// matrix G = U_s^T U_s of the scaled basis is well conditioned; its Jacobi
// eigen-decomposition G = Q L Q^T gives U_s = P S with P orthonormal and
// S = L^(1/2) Q^T, so U = P (S A): the singular values of U are those of the
// ma x ma matrix M = S A (one-sided Jacobi), and the truncated minimum-norm
// solution is sum_j V_j (W_j . c) / s_j with c = P^T b = L^(-1/2) Q^T U_s^T b.
// ---------------------------------------------------------------------------
constexpr int kPolyMax = 10;
constexpr int kPolyThreads = 128;
__constant__ int kPolyExp[kPolyMax][2] = {{0, 0}, {1, 0}, {0, 1}, {1, 1}, {2, 0},
                                          {0, 2}, {1, 2}, {2, 1}, {3, 0}, {0, 3}};

// the basis functions at (x, y), evaluated as poly_funcs does
template <int MA>
__device__ __forceinline__ void poly_basis(double x, double y, double* p) {
    const double xy = x * y;
    const double v[kPolyMax] = {1.0, x, y, xy, x * x, y * y, xy * y, xy * x, x * (x * x), y * (y * y)};
#pragma unroll
    for (int k = 0; k < MA; ++k) p[k] = v[k];
}

// per-block sums for the centring: sum w^2, w^2 x, w^2 y, w^2 x^2, w^2 y^2
__global__ void __launch_bounds__(kThreads) k_poly_moments(const double* __restrict__ x, const double* __restrict__ y,
                                                           const double* __restrict__ snr, int64_t n, int64_t chunk,
                                                           double* __restrict__ part, double* __restrict__ w2out) {
    double s[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    int64_t b0, b1;
    chunk_of(n, chunk, b0, b1);
    for (int64_t i = b0 + threadIdx.x; i < b1; i += kThreads) {
        const double w = 1.0 / (1.0 + 1.0 / snr[i]);  // offsetpoly.f90:58, rows scaled by 1/sig
        const double w2 = w * w;
        w2out[i] = w2;
        s[0] += w2;
        s[1] += w2 * x[i];
        s[2] += w2 * y[i];
        s[3] += w2 * x[i] * x[i];
        s[4] += w2 * y[i] * y[i];
    }
    __shared__ double red[kWarps][5];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        double v = s[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < 5) {
        double v = 0.0;
        for (int w = 0; w < kWarps; ++w) v += red[w][threadIdx.x];
        part[(size_t)blockIdx.x * 5 + threadIdx.x] = v;
    }
}

// one thread: centre x0, y0 (weighted means) and scales Lx, Ly (weighted
// standard deviations; 1 where the spread is zero)
__global__ void k_poly_centre(const double* __restrict__ part, int nb, double* __restrict__ ctr) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int b = 0; b < nb; ++b)
        for (int k = 0; k < 5; ++k) s[k] += part[(size_t)b * 5 + k];
    const double x0 = s[0] > 0.0 ? s[1] / s[0] : 0.0, y0 = s[0] > 0.0 ? s[2] / s[0] : 0.0;
    const double vx = s[0] > 0.0 ? s[3] / s[0] - x0 * x0 : 0.0, vy = s[0] > 0.0 ? s[4] / s[0] - y0 * y0 : 0.0;
    const double lx = vx > 0.0 ? sqrt(vx) : 0.0, ly = vy > 0.0 ? sqrt(vy) : 0.0;
    ctr[0] = x0;
    ctr[1] = lx > 0.0 ? lx : 1.0;
    ctr[2] = y0;
    ctr[3] = ly > 0.0 ? ly : 1.0;
}

// per-block FP64 sums of the scaled Gram matrix (upper triangle, row-major)
// and of U_s^T b; w2 the squared row weights of the first pass
template <int MA>
__global__ void __launch_bounds__(kPolyThreads) k_poly_gram(const double* __restrict__ x, const double* __restrict__ y,
                                                            const double* __restrict__ z,
                                                            const double* __restrict__ w2v,
                                                            const double* __restrict__ ctr, int64_t n, int64_t chunk,
                                                            double* __restrict__ part) {
    constexpr int NG = MA * (MA + 1) / 2, NS = NG + MA;
    double acc[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) acc[k] = 0.0;
    const double x0 = ctr[0], ix = 1.0 / ctr[1], y0 = ctr[2], iy = 1.0 / ctr[3];
    int64_t b0, b1;
    chunk_of(n, chunk, b0, b1);
    for (int64_t i = b0 + threadIdx.x; i < b1; i += kPolyThreads) {
        const double w2 = w2v[i];
        double p[MA];
        poly_basis<MA>((x[i] - x0) * ix, (y[i] - y0) * iy, p);
        int t = 0;
#pragma unroll
        for (int a = 0; a < MA; ++a) {
            const double wa = w2 * p[a];
#pragma unroll
            for (int b = a; b < MA; ++b) acc[t++] += wa * p[b];
        }
        const double wz = w2 * z[i];
#pragma unroll
        for (int a = 0; a < MA; ++a) acc[NG + a] += wz * p[a];
    }
    constexpr int kW = kPolyThreads / 32;
    __shared__ double red[kW][NS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        double v = acc[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][k] = v;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < NS; k += kPolyThreads) {
        double v = 0.0;
        for (int w = 0; w < kW; ++w) v += red[w][k];
        part[(size_t)blockIdx.x * NS + k] = v;
    }
}

__device__ __forceinline__ double jacobi_t(double zeta) {
    // the smaller root of t^2 + 2 zeta t - 1 = 0, sign of zeta
    const double az = fabs(zeta);
    const double r = az > 1.0 ? az * sqrt(1.0 + (1.0 / az) * (1.0 / az)) : sqrt(1.0 + az * az);
    return (zeta >= 0.0 ? 1.0 : -1.0) / (az + r);
}

__device__ __forceinline__ double warp_sum0(double v) {
    // butterfly sum, then lane 0's value everywhere (lanes may round differently)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return __shfl_sync(0xffffffffu, v, 0);
}

// One warp: Jacobi eigen-decomposition of G, M = S A, one-sided Jacobi SVD
// of M, truncated minimum-norm coefficients of the unscaled basis.  Lane r
// owns row r of every matrix; rotation parameters are computed by every
// lane from the same shared values and sums are lane 0's, so every branch
// is warp-uniform.
__global__ void __launch_bounds__(32) k_poly_solve(const double* __restrict__ part, int nb, int ma,
                                                   const double* __restrict__ ctr, double* __restrict__ coef,
                                                   int32_t* __restrict__ rank) {
    constexpr int P = kPolyMax + 1;  // padded row pitch
    __shared__ double G[kPolyMax][P], Q[kPolyMax][P], S[kPolyMax][P], A[kPolyMax][P], M[kPolyMax][P],
        V[kPolyMax][P];
    __shared__ double tot[kPolyMax * (kPolyMax + 1) / 2 + kPolyMax], h[kPolyMax], cv[kPolyMax];
    const int lane = threadIdx.x;
    const bool row = lane < ma;
    const int NG = ma * (ma + 1) / 2, NS = NG + ma;
    for (int e = lane; e < NS; e += 32) {  // block sums in block order
        double v = 0.0;
        for (int blk = 0; blk < nb; ++blk) v += part[(size_t)blk * NS + e];
        tot[e] = v;
    }
    __syncwarp();
    if (row) {
        // row `lane` of the upper triangle starts at lane*ma - lane*(lane-1)/2
        const int base = lane * ma - lane * (lane - 1) / 2;
        for (int b = lane; b < ma; ++b) G[lane][b] = tot[base + (b - lane)];
        h[lane] = tot[NG + lane];
        for (int b = 0; b < ma; ++b) Q[lane][b] = lane == b ? 1.0 : 0.0;
    }
    __syncwarp();
    if (row)
        for (int b = 0; b < lane; ++b) G[lane][b] = G[b][lane];
    __syncwarp();
    // cyclic Jacobi: G <- J^T G J, the annihilated element set to zero
    for (int sweep = 0; sweep < 60; ++sweep) {
        double off = 0.0, dia = 0.0;
        if (row) {
            dia = G[lane][lane] * G[lane][lane];
            for (int q = lane + 1; q < ma; ++q) off += G[lane][q] * G[lane][q];
        }
        off = warp_sum0(off);
        dia = warp_sum0(dia);
        if (off == 0.0 || off <= 1e-30 * dia) break;
        for (int p = 0; p < ma; ++p)
            for (int q = p + 1; q < ma; ++q) {
                const double gpq = G[p][q];
                if (gpq == 0.0) continue;
                const double t = jacobi_t((G[q][q] - G[p][p]) / (2.0 * gpq));
                const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                __syncwarp();  // every lane has read G[p][q], G[p][p], G[q][q]
                if (row) {
                    const double gp = G[lane][p], gq = G[lane][q];
                    G[lane][p] = c * gp - s * gq;
                    G[lane][q] = s * gp + c * gq;
                    const double qp = Q[lane][p], qq = Q[lane][q];
                    Q[lane][p] = c * qp - s * qq;
                    Q[lane][q] = s * qp + c * qq;
                }
                __syncwarp();
                if (row) {
                    const double gp = G[p][lane], gq = G[q][lane];
                    G[p][lane] = c * gp - s * gq;
                    G[q][lane] = s * gp + c * gq;
                }
                __syncwarp();
                if (lane == 0) {
                    G[p][q] = 0.0;
                    G[q][p] = 0.0;
                }
                __syncwarp();
            }
    }
    // S = L^(1/2) Q^T (rows of non-positive eigenvalues zero), c = L^(-1/2) Q^T h;
    // A[j][k]: coefficient of xs^a' ys^b' (term j) in x^a y^b (term k)
    const double x0 = ctr[0], lx = ctr[1], y0 = ctr[2], ly = ctr[3];
    if (row) {
        const int k = lane;
        const double l = G[k][k];
        double qh = 0.0;
        for (int a = 0; a < ma; ++a) qh += Q[a][k] * h[a];
        const double sk = l > 0.0 ? sqrt(l) : 0.0;
        cv[k] = sk > 0.0 ? qh / sk : 0.0;
        for (int a = 0; a < ma; ++a) S[k][a] = sk * Q[a][k];
        const int j = lane, a1 = kPolyExp[j][0], b1 = kPolyExp[j][1];
        const double binom[4][4] = {{1, 0, 0, 0}, {1, 1, 0, 0}, {1, 2, 1, 0}, {1, 3, 3, 1}};
        for (int kk = 0; kk < ma; ++kk) {
            const int a = kPolyExp[kk][0], b = kPolyExp[kk][1];
            double ajk = 0.0;
            if (a1 <= a && b1 <= b) {
                ajk = binom[a][a1] * binom[b][b1];
                for (int e = 0; e < a - a1; ++e) ajk *= x0;
                for (int e = 0; e < a1; ++e) ajk *= lx;
                for (int e = 0; e < b - b1; ++e) ajk *= y0;
                for (int e = 0; e < b1; ++e) ajk *= ly;
            }
            A[j][kk] = ajk;
        }
    }
    __syncwarp();
    if (row) {
        const int r = lane;
        for (int k = 0; k < ma; ++k) {
            double m = 0.0;
            for (int j = 0; j < ma; ++j) m += S[r][j] * A[j][k];
            M[r][k] = m;
            V[r][k] = r == k ? 1.0 : 0.0;
        }
    }
    __syncwarp();
    // one-sided Jacobi: rotate column pairs of M (and V) until orthogonal;
    // columns below 1e-30 of the largest (dropped by the truncation in any
    // case) are left alone.  Lane r touches only row r of M and V.
    for (int sweep = 0; sweep < 60; ++sweep) {
        bool rotated = false;
        double amax = 0.0;
        for (int j = 0; j < ma; ++j) amax = fmax(amax, warp_sum0(row ? M[lane][j] * M[lane][j] : 0.0));
        for (int p = 0; p < ma; ++p)
            for (int q = p + 1; q < ma; ++q) {
                const double mp = row ? M[lane][p] : 0.0, mq = row ? M[lane][q] : 0.0;
                const double al = warp_sum0(mp * mp), be = warp_sum0(mq * mq), ga = warp_sum0(mp * mq);
                if (ga == 0.0 || fabs(ga) <= 1e-14 * sqrt(al * be) || fmin(al, be) <= 1e-60 * amax) continue;
                rotated = true;
                const double t = jacobi_t((be - al) / (2.0 * ga));
                const double c = 1.0 / sqrt(1.0 + t * t), s = c * t;
                if (row) {
                    M[lane][p] = c * mp - s * mq;
                    M[lane][q] = s * mp + c * mq;
                    const double vp = V[lane][p], vq = V[lane][q];
                    V[lane][p] = c * vp - s * vq;
                    V[lane][q] = s * vp + c * vq;
                }
            }
        if (!rotated) break;
    }
    double smax = 0.0, sv[kPolyMax];
    for (int j = 0; j < ma; ++j) {
        sv[j] = sqrt(warp_sum0(row ? M[lane][j] * M[lane][j] : 0.0));
        smax = fmax(smax, sv[j]);
    }
    const double thresh = (double)1e-12f * smax;  // svd.f:3,17-26
    int kept = 0;
    double out = 0.0;  // coefficient `lane`
    for (int j = 0; j < ma; ++j) {
        if (!(sv[j] >= thresh) || sv[j] == 0.0) continue;
        ++kept;
        const double wc = warp_sum0(row ? M[lane][j] * cv[lane] : 0.0);
        const double f = wc / (sv[j] * sv[j]);
        if (row) out += V[lane][j] * f;
    }
    if (row) coef[lane] = out;
    if (lane == 0 && rank) *rank = kept;
}

template <int MA>
void launch_poly_gram(int nb, cudaStream_t st, const double* x, const double* y, const double* z, const double* w2,
                      const double* ctr, int64_t n, int64_t chunk, double* part) {
    k_poly_gram<MA><<<nb, kPolyThreads, 0, st>>>(x, y, z, w2, ctr, n, chunk, part);
}

#define FIELD_CUDA(call)                                                                            \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess) return field_fail(AMPCOR_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

}  // namespace

extern "C" {

int ampcor_offoutliers(const double* loc_across, const double* off_across, const double* loc_down,
                       const double* off_down, const double* sig, const float* snr, double snr_threshold,
                       float distance, int64_t n, int32_t* index_out, int32_t* count_out, float* average_across,
                       float* average_down, double* fit_out, void* stream) {
    g_field_err.clear();
    if (n <= 0) return field_fail(AMPCOR_ERR_ARG, "no offsets to cull (n = %lld)", (long long)n);
    if (n > INT32_MAX) return field_fail(AMPCOR_ERR_ARG, "too many offsets (%lld)", (long long)n);
    if (!loc_across || !off_across || !loc_down || !off_down || !index_out || !count_out)
        return field_fail(AMPCOR_ERR_ARG, "null array");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int nb = (int)std::min<int64_t>(kMaxBlocks, (n + kThreads - 1) / kThreads);
    const int64_t chunk = ((n + nb - 1) / nb + kThreads - 1) / kThreads * kThreads;
    // workspace: block sums, fit, block counts and offsets, flags
    const size_t o_fit = (size_t)nb * kSums * sizeof(double);
    const size_t o_cnt = o_fit + 16;
    const size_t o_off = o_cnt + (size_t)nb * sizeof(int);
    const size_t o_flg = o_off + (size_t)nb * sizeof(int);
    const size_t bytes = o_flg + (size_t)n;
    unsigned char* ws = nullptr;
    FIELD_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&ws), bytes, st));
    double* part = reinterpret_cast<double*>(ws);
    float* fit32 = reinterpret_cast<float*>(ws + o_fit);
    int* bcount = reinterpret_cast<int*>(ws + o_cnt);
    int* boff = reinterpret_cast<int*>(ws + o_off);
    uint8_t* flags = ws + o_flg;
    k_cull_sums<<<nb, kThreads, 0, st>>>(loc_across, off_across, loc_down, off_down, sig, snr, snr_threshold, n,
                                          chunk, part);
    k_cull_fit<<<1, 32, 0, st>>>(part, nb, fit32, fit_out, average_across, average_down);
    k_cull_flags<<<nb, kThreads, 0, st>>>(loc_across, off_across, loc_down, off_down, snr, snr_threshold, distance,
                                           fit32, n, chunk, flags, bcount);
    k_cull_offsets<<<1, 32, 0, st>>>(bcount, nb, boff, count_out);
    k_cull_scatter<<<nb, kThreads, 0, st>>>(flags, n, chunk, boff, index_out);
    const cudaError_t le = cudaGetLastError();
    FIELD_CUDA(cudaFreeAsync(ws, st));
    if (le != cudaSuccess) return field_fail(AMPCOR_ERR_CUDA, "culling launch: %s", cudaGetErrorString(le));
    return AMPCOR_OK;
}

int ampcor_decimate(const void* src, int64_t src_rows, int64_t src_cols, int64_t src_ld, int32_t elem_bytes,
                    int64_t y0, int64_t x0, int64_t ystep, int64_t xstep, void* dst, int64_t rows, int64_t cols,
                    void* stream) {
    g_field_err.clear();
    if (!src || !dst) return field_fail(AMPCOR_ERR_ARG, "null array");
    if (rows <= 0 || cols <= 0 || src_rows <= 0 || src_cols <= 0 || src_ld < src_cols || ystep <= 0 || xstep <= 0)
        return field_fail(AMPCOR_ERR_ARG, "bad sizes (%lld x %lld from %lld x %lld, ld %lld, steps %lld %lld)",
                          (long long)rows, (long long)cols, (long long)src_rows, (long long)src_cols,
                          (long long)src_ld, (long long)ystep, (long long)xstep);
    if ((cols + 31) / 32 > INT32_MAX) return field_fail(AMPCOR_ERR_ARG, "too many columns (%lld)", (long long)cols);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const dim3 blk(32, 8);
    const dim3 grd((unsigned)((cols + 31) / 32), (unsigned)std::min<int64_t>((rows + 7) / 8, 4096));
    switch (elem_bytes) {
        case 1:
            k_decimate<uint8_t><<<grd, blk, 0, st>>>(static_cast<const uint8_t*>(src), src_rows, src_cols, src_ld, y0,
                                                     x0, ystep, xstep, static_cast<uint8_t*>(dst), rows, cols);
            break;
        case 2:
            k_decimate<uint16_t><<<grd, blk, 0, st>>>(static_cast<const uint16_t*>(src), src_rows, src_cols, src_ld,
                                                      y0, x0, ystep, xstep, static_cast<uint16_t*>(dst), rows, cols);
            break;
        case 4:
            k_decimate<uint32_t><<<grd, blk, 0, st>>>(static_cast<const uint32_t*>(src), src_rows, src_cols, src_ld,
                                                      y0, x0, ystep, xstep, static_cast<uint32_t*>(dst), rows, cols);
            break;
        case 8:
            k_decimate<unsigned long long><<<grd, blk, 0, st>>>(static_cast<const unsigned long long*>(src), src_rows,
                                                                src_cols, src_ld, y0, x0, ystep, xstep,
                                                                static_cast<unsigned long long*>(dst), rows, cols);
            break;
        default:
            return field_fail(AMPCOR_ERR_ARG, "element size %d is not 1, 2, 4 or 8 bytes", (int)elem_bytes);
    }
    FIELD_CUDA(cudaGetLastError());
    return AMPCOR_OK;
}

int ampcor_offsetpoly(const double* loc_across, const double* loc_down, const double* offset, const double* snr,
                      int64_t n, int32_t ncoef, double* coef_out, int32_t* rank_out, void* stream) {
    g_field_err.clear();
    if (n <= 0) return field_fail(AMPCOR_ERR_ARG, "no offsets to fit (n = %lld)", (long long)n);
    if (ncoef < 1 || ncoef > kPolyMax)
        return field_fail(AMPCOR_ERR_ARG, "number of fit coefficients %d is not 1 to %d", (int)ncoef, kPolyMax);
    if (!loc_across || !loc_down || !offset || !snr || !coef_out) return field_fail(AMPCOR_ERR_ARG, "null array");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int nb = (int)std::min<int64_t>(kMaxBlocks, (n + kThreads - 1) / kThreads);
    const int64_t chunk = ((n + nb - 1) / nb + kThreads - 1) / kThreads * kThreads;
    const int ns = ncoef * (ncoef + 1) / 2 + ncoef;
    const size_t o_ctr = (size_t)nb * 5 * sizeof(double);
    const size_t o_gram = o_ctr + 4 * sizeof(double);
    const size_t o_w2 = o_gram + (size_t)nb * ns * sizeof(double);
    const size_t bytes = o_w2 + (size_t)n * sizeof(double);
    unsigned char* ws = nullptr;
    FIELD_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&ws), bytes, st));
    double* part1 = reinterpret_cast<double*>(ws);
    double* ctr = reinterpret_cast<double*>(ws + o_ctr);
    double* part2 = reinterpret_cast<double*>(ws + o_gram);
    double* w2 = reinterpret_cast<double*>(ws + o_w2);
    k_poly_moments<<<nb, kThreads, 0, st>>>(loc_across, loc_down, snr, n, chunk, part1, w2);
    k_poly_centre<<<1, 32, 0, st>>>(part1, nb, ctr);
    switch (ncoef) {
        case 1: launch_poly_gram<1>(nb, st, loc_across, loc_down, offset, w2, ctr, n, chunk, part2); break;
        case 2: launch_poly_gram<2>(nb, st, loc_across, loc_down, offset, w2, ctr, n, chunk, part2); break;
        case 3: launch_poly_gram<3>(nb, st, loc_across, loc_down, offset, w2, ctr, n, chunk, part2); break;
        case 4: launch_poly_gram<4>(nb, st, loc_across, loc_down, offset, w2, ctr, n, chunk, part2); break;
        case 5: launch_poly_gram<5>(nb, st, loc_across, loc_down, offset, w2, ctr, n, chunk, part2); break;
        case 6: launch_poly_gram<6>(nb, st, loc_across, loc_down, offset, w2, ctr, n, chunk, part2); break;
        case 7: launch_poly_gram<7>(nb, st, loc_across, loc_down, offset, w2, ctr, n, chunk, part2); break;
        case 8: launch_poly_gram<8>(nb, st, loc_across, loc_down, offset, w2, ctr, n, chunk, part2); break;
        case 9: launch_poly_gram<9>(nb, st, loc_across, loc_down, offset, w2, ctr, n, chunk, part2); break;
        default: launch_poly_gram<10>(nb, st, loc_across, loc_down, offset, w2, ctr, n, chunk, part2); break;
    }
    k_poly_solve<<<1, 32, 0, st>>>(part2, nb, ncoef, ctr, coef_out, rank_out);
    const cudaError_t le = cudaGetLastError();
    FIELD_CUDA(cudaFreeAsync(ws, st));
    if (le != cudaSuccess) return field_fail(AMPCOR_ERR_CUDA, "offset polynomial launch: %s", cudaGetErrorString(le));
    return AMPCOR_OK;
}

int ampcor_field_last_error(char* buf, int64_t n) {
    if (!buf || n <= 0) return AMPCOR_ERR_ARG;
    std::snprintf(buf, (size_t)n, "%s", g_field_err.c_str());
    return AMPCOR_OK;
}

}  // extern "C"
