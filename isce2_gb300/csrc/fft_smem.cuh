// In-place mixed-radix FFTs on a 2-D tile held in shared memory.
//
// The forward pass is decimation in frequency (natural order in, digit-
// reversed order out); the matching inverse pass is decimation in time
// (digit-reversed in, natural out).  Point-wise work between the two (the
// conjugate product of a correlation, the spectral zero-padding of an
// oversampler) is done directly in the digit-reversed domain, so no
// permutation pass is ever needed.  Each butterfly reads and writes the same
// R positions, so a pass needs one barrier and no second buffer.
//
// The per-work-item functions are __host__ __device__ so that the index logic
// can be driven by a plain loop on the CPU in tests.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#ifndef AMPCOR_HD
#define AMPCOR_HD __host__ __device__ __forceinline__
#endif

namespace ampcor {

constexpr int kMaxRadixCount = 16;
constexpr int kMaxGenericRadix = 131;  // every prime of an even window side <= 264

// Division by a runtime-invariant divisor with one multiply-high
// (Granlund-Montgomery); valid for every 32-bit dividend.
struct FastDiv {
    uint32_t d, m, s;
    AMPCOR_HD FastDiv() : d(1), m(0), s(0) {}
    AMPCOR_HD explicit FastDiv(uint32_t div) : d(div), m(0), s(0) {
        if (div > 1) {
            uint32_t l = 0;
            while ((1ull << l) < div) ++l;
            m = (uint32_t)((((1ull << 32) * ((1ull << l) - div)) / div) + 1);
            s = l;
        }
    }
    AMPCOR_HD uint32_t div(uint32_t x) const {
        if (d == 1) return x;
#ifdef __CUDA_ARCH__
        const uint32_t t = __umulhi(x, m);
#else
        const uint32_t t = (uint32_t)(((uint64_t)x * m) >> 32);
#endif
        return (t + ((x - t) >> 1)) >> (s - 1);
    }
};

// Factorisation of one transform length.  rad[0] is the first (outermost)
// decimation-in-frequency pass; the dividers split a pass's work items.
struct FftPlan1D {
    int n;
    int npass;
    int rad[kMaxRadixCount];
    int span[kMaxRadixCount];  // block size M at pass p: n / (rad[0]*...*rad[p-1])
    FastDiv dnb[kMaxRadixCount];      // n / rad[p]
    FastDiv dstride[kMaxRadixCount];  // span[p] / rad[p]
};

struct cfloat { float x, y; };

AMPCOR_HD cfloat cmul(cfloat a, cfloat b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
AMPCOR_HD cfloat cadd(cfloat a, cfloat b) { return {a.x + b.x, a.y + b.y}; }
AMPCOR_HD cfloat csub(cfloat a, cfloat b) { return {a.x - b.x, a.y - b.y}; }
AMPCOR_HD cfloat cconj(cfloat a) { return {a.x, -a.y}; }
AMPCOR_HD cfloat cscale(cfloat a, float s) { return {a.x * s, a.y * s}; }

// e^{sign * 2 pi i t / n} for integer t (reduced mod n first), accurate to a
// few ulp because the argument is formed exactly as a fraction of pi.
AMPCOR_HD cfloat unit_root(long long t, int n, int sign) {
    long long r = t % n;
    if (r < 0) r += n;
    float s, c;
#ifdef __CUDA_ARCH__
    sincospif(2.0f * (float)r / (float)n, &s, &c);
#else
    double a = 2.0 * 3.14159265358979323846 * (double)r / (double)n;
    s = (float)sin(a);
    c = (float)cos(a);
#endif
    return {c, sign > 0 ? s : -s};
}

// Host-side: factor n into supported radices (8,4,2 first, then odd primes).
// Returns false when a prime factor exceeds kMaxGenericRadix.
inline bool fft_plan_make(int n, FftPlan1D* p) {
    if (n <= 0) return false;
    p->n = n;
    p->npass = 0;
    int m = n;
    int rads[kMaxRadixCount];
    int k = 0;
    // large composite radices first: fewer passes, each butterfly in registers
    while (m % 16 == 0 && k < kMaxRadixCount) { rads[k++] = 16; m /= 16; }
    if (m % 12 == 0 && k < kMaxRadixCount) { rads[k++] = 12; m /= 12; }
    while (m % 8 == 0 && k < kMaxRadixCount) { rads[k++] = 8; m /= 8; }
    if (m % 4 == 0 && k < kMaxRadixCount) { rads[k++] = 4; m /= 4; }
    if (m % 6 == 0 && k < kMaxRadixCount) { rads[k++] = 6; m /= 6; }
    if (m % 2 == 0 && k < kMaxRadixCount) { rads[k++] = 2; m /= 2; }
    for (int f = 3; m > 1 && k < kMaxRadixCount; f += 2) {
        while (m % f == 0 && k < kMaxRadixCount) {
            if (f > kMaxGenericRadix) return false;
            rads[k++] = f;
            m /= f;
        }
        if (f > kMaxGenericRadix && m > 1) return false;
    }
    if (m != 1) return false;
    int span = n;
    for (int i = 0; i < k; ++i) {
        p->rad[i] = rads[i];
        p->span[i] = span;
        p->dnb[i] = FastDiv((uint32_t)(n / rads[i]));
        p->dstride[i] = FastDiv((uint32_t)(span / rads[i]));
        span /= rads[i];
    }
    p->npass = k;
    return true;
}

// Smallest length >= n whose prime factors are all in {2,3,5,7}.
inline int fft_good_size(int n) {
    for (int m = n > 1 ? n : 1;; ++m) {
        int t = m;
        for (int f : {2, 3, 5, 7})
            while (t % f == 0) t /= f;
        if (t == 1) return m;
    }
}

// natural frequency index of digit-reversed position `pos` (DIF output order)
AMPCOR_HD int fft_pos_to_freq(const FftPlan1D& p, int pos) {
    int f = 0, mul = 1;
    for (int i = 0; i < p.npass; ++i) {
        int blk = p.span[i] / p.rad[i];
        int d = pos / blk;
        pos -= d * blk;
        f += d * mul;
        mul *= p.rad[i];
    }
    return f;
}

// digit-reversed position of natural frequency index f
AMPCOR_HD int fft_freq_to_pos(const FftPlan1D& p, int f) {
    int pos = 0;
    for (int i = 0; i < p.npass; ++i) {
        int d = f % p.rad[i];
        f /= p.rad[i];
        pos += d * (p.span[i] / p.rad[i]);
    }
    return pos;
}

// root w_R^m of a radix-R DFT taken from the length-n table tw[t] = e^{+2 pi i t/n}
AMPCOR_HD cfloat table_root(const cfloat* tw, int n, int R, int m, int sign) {
    const cfloat w = tw[(m % R) * (n / R)];
    return sign > 0 ? w : cconj(w);
}

template <int A, int B>
AMPCOR_HD void dft_composite(cfloat* v, int sign, const cfloat* tw, int n);

// small DFT of R values in registers, y_q = sum_r x_r w^{rq}, w = e^{sign 2pi i/R}
template <int R>
AMPCOR_HD void dft_small(cfloat* v, int sign, const cfloat* tw, int n) {
    if constexpr (R == 16) {
        dft_composite<4, 4>(v, sign, tw, n);
    } else if constexpr (R == 12) {
        dft_composite<4, 3>(v, sign, tw, n);
    } else if constexpr (R == 6) {
        dft_composite<2, 3>(v, sign, tw, n);
    } else if constexpr (R == 2) {
        cfloat a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    } else if constexpr (R == 4) {
        cfloat a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
        cfloat c = cadd(v[1], v[3]), d = csub(v[1], v[3]);
        // d * (sign i)
        cfloat di = sign > 0 ? cfloat{-d.y, d.x} : cfloat{d.y, -d.x};
        v[0] = cadd(a, c);
        v[2] = csub(a, c);
        v[1] = cadd(b, di);
        v[3] = csub(b, di);
    } else if constexpr (R == 8) {
        // two radix-4 on even/odd, then combine with w8 twiddles
        cfloat e[4] = {v[0], v[2], v[4], v[6]};
        cfloat o[4] = {v[1], v[3], v[5], v[7]};
        dft_small<4>(e, sign, tw, n);
        dft_small<4>(o, sign, tw, n);
        const float h = 0.70710678118654752f;
        cfloat t1 = sign > 0 ? cfloat{h * (o[1].x - o[1].y), h * (o[1].x + o[1].y)}
                             : cfloat{h * (o[1].x + o[1].y), h * (o[1].y - o[1].x)};
        cfloat t2 = sign > 0 ? cfloat{-o[2].y, o[2].x} : cfloat{o[2].y, -o[2].x};
        cfloat t3 = sign > 0 ? cfloat{-h * (o[3].x + o[3].y), h * (o[3].x - o[3].y)}
                             : cfloat{h * (o[3].y - o[3].x), -h * (o[3].x + o[3].y)};
        v[0] = cadd(e[0], o[0]);
        v[4] = csub(e[0], o[0]);
        v[1] = cadd(e[1], t1);
        v[5] = csub(e[1], t1);
        v[2] = cadd(e[2], t2);
        v[6] = csub(e[2], t2);
        v[3] = cadd(e[3], t3);
        v[7] = csub(e[3], t3);
    } else {
        // odd R: pair r with R-r, y_q = x0 + sum_r [a_r cos(t) + i s b_r sin(t)],
        // a_r = x_r + x_{R-r}, b_r = x_r - x_{R-r}, t = 2 pi r q / R
        static_assert(R % 2 == 1, "odd radix expected");
        constexpr int H = (R - 1) / 2;
        cfloat a[H + 1], b[H + 1];
        cfloat y0 = v[0];
        for (int r = 1; r <= H; ++r) {
            a[r] = cadd(v[r], v[R - r]);
            b[r] = csub(v[r], v[R - r]);
            y0 = cadd(y0, a[r]);
        }
        const int step = n / R;
        for (int q = 1; q <= H; ++q) {
            cfloat A = v[0], Bs = {0.f, 0.f};
            int m = 0;
            for (int r = 1; r <= H; ++r) {
                m += q;
                if (m >= R) m -= R;
                const cfloat w = tw[m * step];  // (cos t, sin t)
                A.x = fmaf(a[r].x, w.x, A.x);
                A.y = fmaf(a[r].y, w.x, A.y);
                Bs.x = fmaf(b[r].x, w.y, Bs.x);
                Bs.y = fmaf(b[r].y, w.y, Bs.y);
            }
            // i * sign * Bs
            const cfloat iB = sign > 0 ? cfloat{-Bs.y, Bs.x} : cfloat{Bs.y, -Bs.x};
            v[q] = cadd(A, iB);
            v[R - q] = csub(A, iB);
        }
        v[0] = y0;
    }
}

// Composite radix R = A*B in registers (Cooley-Tukey inside the butterfly):
// with r = B*r1 + r0 and q = q0 + A*q1, y_q = sum_r0 w_B^{r0 q1} w_R^{r0 q0}
// sum_r1 x_{B r1 + r0} w_A^{r1 q0}: B transforms of length A, the R-point
// twiddles, A transforms of length B.  Roots come from the line's table
// (tw[t] = e^{+2 pi i t / n}, A and B divide n).
template <int A, int B>
AMPCOR_HD void dft_composite(cfloat* v, int sign, const cfloat* tw, int n) {
    constexpr int R = A * B;
    cfloat u[B][A];
    for (int r0 = 0; r0 < B; ++r0) {
        cfloat t[A];
        for (int r1 = 0; r1 < A; ++r1) t[r1] = v[B * r1 + r0];
        dft_small<A>(t, sign, tw, n);
        for (int q0 = 0; q0 < A; ++q0) u[r0][q0] = t[q0];
    }
    const int step = n / R;
    for (int r0 = 1; r0 < B; ++r0)
        for (int q0 = 1; q0 < A; ++q0) {
            cfloat w = tw[((r0 * q0) % R) * step];
            if (sign < 0) w = cconj(w);
            u[r0][q0] = cmul(u[r0][q0], w);
        }
    for (int q0 = 0; q0 < A; ++q0) {
        cfloat t[B];
        for (int r0 = 0; r0 < B; ++r0) t[r0] = u[r0][q0];
        dft_small<B>(t, sign, tw, n);
        for (int q1 = 0; q1 < B; ++q1) v[q0 + A * q1] = t[q1];
    }
}

template <int R>
AMPCOR_HD void twiddle(cfloat* v, int k, int span, int n, const cfloat* tw, int sign) {
    const int kstep = k * (n / span);  // w_span^{kq} = w_n^{kq*step}, and kq*step < n
    for (int q = 1; q < R; ++q) {
        cfloat w = tw[kstep * q];
        if (sign < 0) w = cconj(w);
        v[q] = cmul(v[q], w);
    }
}

// One butterfly of a DIF pass: positions base + k + r*stride, r < R.
template <int R>
AMPCOR_HD void dif_bfly(cfloat* line, int es, int base, int k, int stride, int span, int n,
                        const cfloat* tw, int sign) {
    cfloat v[R];
    for (int r = 0; r < R; ++r) v[r] = line[(size_t)(base + k + r * stride) * es];
    dft_small<R>(v, sign, tw, n);
    twiddle<R>(v, k, span, n, tw, sign);
    for (int q = 0; q < R; ++q) line[(size_t)(base + k + q * stride) * es] = v[q];
}

// One butterfly of a DIT pass (the exact inverse structure of dif_bfly).
template <int R>
AMPCOR_HD void dit_bfly(cfloat* line, int es, int base, int k, int stride, int span, int n,
                        const cfloat* tw, int sign) {
    cfloat v[R];
    for (int q = 0; q < R; ++q) v[q] = line[(size_t)(base + k + q * stride) * es];
    twiddle<R>(v, k, span, n, tw, sign);
    dft_small<R>(v, sign, tw, n);
    for (int r = 0; r < R; ++r) line[(size_t)(base + k + r * stride) * es] = v[r];
}

// Generic odd prime radix R (23 .. kMaxGenericRadix): the symmetric form of
// dft_small's odd branch.  The R inputs (pre-twiddled for DIT) are folded
// into H = (R-1)/2 sums a_r = x_r + x_{R-r} and differences b_r = x_r - x_{R-r};
// output pair (q, R-q) is A +- i*sign*B with A = x_0 + sum_r a_r cos(2 pi rq/R)
// and B = sum_r b_r sin(2 pi rq/R), the root index advancing by q (mod R)
// without a division.  Every input is read before the first output is
// written, so the pair is stored as soon as it is known.
AMPCOR_HD void generic_bfly(bool dif, cfloat* line, int es, int base, int k, int stride, int R, int span,
                            int n, const cfloat* tw, int sign) {
    constexpr int HM = (kMaxGenericRadix - 1) / 2;
    cfloat a[HM + 1], b[HM + 1];
    const int kstep = k * (n / span);
    const int step = n / R;
    const int H = (R - 1) / 2;
    auto at = [&](int r) -> cfloat& { return line[(size_t)(base + k + r * stride) * es]; };
    auto twk = [&](int q) {  // w_span^{kq} = w_n^{kstep q}, kstep q < n
        cfloat w = tw[kstep * q];
        return sign < 0 ? cconj(w) : w;
    };
    const cfloat x0 = at(0);
    cfloat y0 = x0;
    for (int r = 1; r <= H; ++r) {
        cfloat u = at(r), v = at(R - r);
        if (!dif) {
            u = cmul(u, twk(r));
            v = cmul(v, twk(R - r));
        }
        a[r] = cadd(u, v);
        b[r] = csub(u, v);
        y0 = cadd(y0, a[r]);
    }
    at(0) = y0;
    for (int q = 1; q <= H; ++q) {
        cfloat A = x0, Bs = {0.f, 0.f};
        int m = 0;
        for (int r = 1; r <= H; ++r) {
            m += q;
            if (m >= R) m -= R;
            const cfloat w = tw[m * step];  // (cos, sin) of 2 pi m / R
            A.x = fmaf(a[r].x, w.x, A.x);
            A.y = fmaf(a[r].y, w.x, A.y);
            Bs.x = fmaf(b[r].x, w.y, Bs.x);
            Bs.y = fmaf(b[r].y, w.y, Bs.y);
        }
        const cfloat iB = sign > 0 ? cfloat{-Bs.y, Bs.x} : cfloat{Bs.y, -Bs.x};
        cfloat yq = cadd(A, iB), yr = csub(A, iB);
        if (dif) {
            yq = cmul(yq, twk(q));
            yr = cmul(yr, twk(R - q));
        }
        at(q) = yq;
        at(R - q) = yr;
    }
}

// Split work item `it` of a pass into (line, butterfly j) and j into (block b, k).
struct PassIndex {
    FastDiv dnb, dlines, dstride;
    int nb, nlines, stride;
    bool line_fastest;
    AMPCOR_HD PassIndex(const FftPlan1D& p, int pass, const FastDiv& dl, bool lf)
        : dnb(p.dnb[pass]), dlines(dl), dstride(p.dstride[pass]),
          nb(p.n / p.rad[pass]), nlines((int)dl.d), stride(p.span[pass] / p.rad[pass]), line_fastest(lf) {}
    AMPCOR_HD void split(int it, int& line, int& b, int& k) const {
        int j;
        if (line_fastest) { j = (int)dlines.div(it); line = it - j * nlines; }
        else { line = (int)dnb.div(it); j = it - line * nb; }
        b = (int)dstride.div(j);
        k = j - b * stride;
    }
};

template <int R>
AMPCOR_HD void pass_item_r(bool dif, const FftPlan1D& p, int pass, const PassIndex& ix, cfloat* data, int ls,
                           int es, int it, const cfloat* tw, int sign) {
    int line, b, k;
    ix.split(it, line, b, k);
    cfloat* L = data + (size_t)line * ls;
    const int span = p.span[pass];
    if (dif) dif_bfly<R>(L, es, b * span, k, ix.stride, span, p.n, tw, sign);
    else dit_bfly<R>(L, es, b * span, k, ix.stride, span, p.n, tw, sign);
}

// Work item `item` of pass `pass` over `nlines` lines.  A line starts at
// data + line*ls (elements) and its elements are es apart.  `line_fastest`
// selects the item -> (line, butterfly) order: true for column transforms of
// a row-major tile so that neighbouring threads touch neighbouring addresses.
AMPCOR_HD void fft_pass_item(bool dif, const FftPlan1D& p, int pass, cfloat* data, int nlines, int ls, int es,
                             bool line_fastest, int item, const cfloat* tw, int sign) {
    const PassIndex ix(p, pass, FastDiv((uint32_t)nlines), line_fastest);
    switch (p.rad[pass]) {
        case 2: pass_item_r<2>(dif, p, pass, ix, data, ls, es, item, tw, sign); break;
        case 3: pass_item_r<3>(dif, p, pass, ix, data, ls, es, item, tw, sign); break;
        case 4: pass_item_r<4>(dif, p, pass, ix, data, ls, es, item, tw, sign); break;
        case 5: pass_item_r<5>(dif, p, pass, ix, data, ls, es, item, tw, sign); break;
        case 7: pass_item_r<7>(dif, p, pass, ix, data, ls, es, item, tw, sign); break;
        case 6: pass_item_r<6>(dif, p, pass, ix, data, ls, es, item, tw, sign); break;
        case 8: pass_item_r<8>(dif, p, pass, ix, data, ls, es, item, tw, sign); break;
        case 12: pass_item_r<12>(dif, p, pass, ix, data, ls, es, item, tw, sign); break;
        case 16: pass_item_r<16>(dif, p, pass, ix, data, ls, es, item, tw, sign); break;
        case 11: pass_item_r<11>(dif, p, pass, ix, data, ls, es, item, tw, sign); break;
        case 13: pass_item_r<13>(dif, p, pass, ix, data, ls, es, item, tw, sign); break;
        case 17: pass_item_r<17>(dif, p, pass, ix, data, ls, es, item, tw, sign); break;
        case 19: pass_item_r<19>(dif, p, pass, ix, data, ls, es, item, tw, sign); break;
        default: {
            int line, b, k;
            ix.split(item, line, b, k);
            generic_bfly(dif, data + (size_t)line * ls, es, b * p.span[pass], k, ix.stride, p.rad[pass],
                         p.span[pass], p.n, tw, sign);
        }
    }
}

AMPCOR_HD int fft_pass_items(const FftPlan1D& p, int pass, int nlines) { return nlines * (p.n / p.rad[pass]); }

#ifdef __CUDACC__
// Block-cooperative transforms.  All threads of the block must call these.
template <int R>
__device__ __forceinline__ void block_pass_r(bool dif, const FftPlan1D& p, int pass, cfloat* data,
                                             const FastDiv& dl, int ls, int es, bool lf, const cfloat* tw, int sign) {
    const PassIndex ix(p, pass, dl, lf);
    const int items = ix.nlines * ix.nb;
    for (int it = threadIdx.x; it < items; it += blockDim.x)
        pass_item_r<R>(dif, p, pass, ix, data, ls, es, it, tw, sign);
}

// A generic odd prime radix R pass, parallel inside each butterfly.  The
// work item (butterfly, group g) computes the output pairs (q, R-q) for
// q in [g*kGenericPairs, (g+1)*kGenericPairs) (q = 0: the plain sum) in the
// symmetric form of generic_bfly, reading each input pair once per item.
// Outputs go to registers and are stored after a barrier, so the pass stays
// in place; butterflies are taken in rounds of at most one item per thread.
// A DIT pass applies its input twiddles in place first, a DIF pass its output
// twiddles before storing.  This pays where a pass has fewer butterflies than
// the block has threads and long ones (a 226-point line is 2 butterflies of
// 113); generic_pass_parallel_pays() decides.
constexpr int kGenericPairs = 4;

__device__ inline bool generic_pass_parallel_pays(int R, int nbf) {
    const int H = (R - 1) / 2, T = (int)blockDim.x;
    const int groups = (H + kGenericPairs) / kGenericPairs;  // covers q = 0 .. H
    const int rounds = (nbf * groups + T - 1) / T;
    const int serial = (nbf + T - 1) / T;
    return 5 * rounds * kGenericPairs < 4 * serial * H;
}

__device__ inline void block_generic_pass(bool dif, const FftPlan1D& p, int pass, cfloat* data, int nlines,
                                          int ls, int es, const cfloat* tw, int sign) {
    const int R = p.rad[pass], H = (R - 1) / 2, n = p.n, span = p.span[pass];
    const int stride = span / R, per_line = n / R, step = n / R;
    const int nbf = nlines * per_line;
    const int groups = (H + kGenericPairs) / kGenericPairs;
    const FastDiv dpl((uint32_t)per_line), dst((uint32_t)stride), dg((uint32_t)groups);
    auto locate = [&](int j, int& line, int& base, int& k) {  // butterfly j -> line, block base, k
        line = (int)dpl.div((uint32_t)j);
        const int bf = j - line * per_line;
        const int b = (int)dst.div((uint32_t)bf);
        k = bf - b * stride;
        base = b * span;
    };
    auto twk = [&](int kstep, int q) {
        cfloat w = tw[kstep * q];
        return sign < 0 ? cconj(w) : w;
    };
    if (!dif) {  // input twiddles of the DIT butterflies
        for (int t = threadIdx.x; t < nbf * R; t += blockDim.x) {
            const int j = t / R, r = t - (t / R) * R;
            if (r == 0) continue;
            int line, base, k;
            locate(j, line, base, k);
            cfloat* x = data + (size_t)line * ls + (size_t)(base + k + r * stride) * es;
            *x = cmul(*x, twk(k * (n / span), r));
        }
        __syncthreads();
    }
    const int per_round = max(1, (int)blockDim.x / groups);
    for (int j0 = 0; j0 < nbf; j0 += per_round) {
        const int items = min(per_round, nbf - j0) * groups;
        cfloat ya[kGenericPairs], yb[kGenericPairs];
        int q0 = 0, nq = 0, line = 0, base = 0, k = 0;
        const int it = threadIdx.x;
        if (it < items) {
            const int jb = (int)dg.div((uint32_t)it), g = it - jb * groups;
            locate(j0 + jb, line, base, k);
            q0 = g * kGenericPairs;
            nq = min(kGenericPairs, H + 1 - q0);
            const cfloat* L = data + (size_t)line * ls;
            auto at = [&](int r) { return L[(size_t)(base + k + r * stride) * es]; };
            const cfloat x0 = at(0);
            cfloat A[kGenericPairs], B[kGenericPairs];
            int m[kGenericPairs];
#pragma unroll
            for (int c = 0; c < kGenericPairs; ++c) {
                A[c] = x0;
                B[c] = {0.f, 0.f};
                m[c] = 0;
            }
            for (int r = 1; r <= H; ++r) {
                const cfloat u = at(r), v = at(R - r);
                const cfloat a = cadd(u, v), b = csub(u, v);
#pragma unroll
                for (int c = 0; c < kGenericPairs; ++c) {
                    m[c] += q0 + c;
                    if (m[c] >= R) m[c] -= R;
                    const cfloat w = tw[m[c] * step];  // (cos, sin) of 2 pi m / R
                    A[c].x = fmaf(a.x, w.x, A[c].x);
                    A[c].y = fmaf(a.y, w.x, A[c].y);
                    B[c].x = fmaf(b.x, w.y, B[c].x);
                    B[c].y = fmaf(b.y, w.y, B[c].y);
                }
            }
            const int kstep = k * (n / span);
#pragma unroll
            for (int c = 0; c < kGenericPairs; ++c) {
                const int q = q0 + c;
                const cfloat iB = sign > 0 ? cfloat{-B[c].y, B[c].x} : cfloat{B[c].y, -B[c].x};
                cfloat yq = cadd(A[c], iB), yr = csub(A[c], iB);
                if (dif && q > 0) {
                    yq = cmul(yq, twk(kstep, q));
                    yr = cmul(yr, twk(kstep, R - q));
                }
                ya[c] = yq;
                yb[c] = yr;
            }
        }
        __syncthreads();  // every input of the round's butterflies is read
        if (it < items) {
            cfloat* L = data + (size_t)line * ls;
            for (int c = 0; c < nq; ++c) {
                const int q = q0 + c;
                L[(size_t)(base + k + q * stride) * es] = ya[c];
                if (q > 0) L[(size_t)(base + k + (R - q) * stride) * es] = yb[c];
            }
        }
        __syncthreads();
    }
}

// A pass of a prime radix of 11 or more (generic_bfly, or the in-butterfly
// parallel form).  Kept out of line and small in registers: inlined, or
// with fully unrolled butterflies, it raised the register demand of the
// kernels' common radix 2..16 passes into spills.
static __device__ __noinline__ void block_prime_pass(bool dif, const FftPlan1D& p, int pass, cfloat* data,
                                                     const FastDiv& dl, int ls, int es, bool lf, const cfloat* tw,
                                                     int sign) {
    const int nlines = (int)dl.d;
    if (generic_pass_parallel_pays(p.rad[pass], nlines * (p.n / p.rad[pass]))) {
        block_generic_pass(dif, p, pass, data, nlines, ls, es, tw, sign);
        return;
    }
    const PassIndex ix(p, pass, dl, lf);
    const int items = ix.nlines * ix.nb;
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
        int line, b, k;
        ix.split(it, line, b, k);
        generic_bfly(dif, data + (size_t)line * ls, es, b * p.span[pass], k, ix.stride, p.rad[pass], p.span[pass],
                     p.n, tw, sign);
    }
}

// `dl` divides by the number of lines (built once per kernel: its set-up costs a 64-bit division).
__device__ inline void block_fft_lines(bool dif, const FftPlan1D& p, cfloat* data, const FastDiv& dl, int ls, int es,
                                       bool line_fastest, const cfloat* tw, int sign) {
    const int nlines = (int)dl.d;
    for (int s = 0; s < p.npass; ++s) {
        const int pass = dif ? s : p.npass - 1 - s;
        switch (p.rad[pass]) {
            case 2: block_pass_r<2>(dif, p, pass, data, dl, ls, es, line_fastest, tw, sign); break;
            case 3: block_pass_r<3>(dif, p, pass, data, dl, ls, es, line_fastest, tw, sign); break;
            case 4: block_pass_r<4>(dif, p, pass, data, dl, ls, es, line_fastest, tw, sign); break;
            case 5: block_pass_r<5>(dif, p, pass, data, dl, ls, es, line_fastest, tw, sign); break;
            case 7: block_pass_r<7>(dif, p, pass, data, dl, ls, es, line_fastest, tw, sign); break;
            case 6: block_pass_r<6>(dif, p, pass, data, dl, ls, es, line_fastest, tw, sign); break;
            case 8: block_pass_r<8>(dif, p, pass, data, dl, ls, es, line_fastest, tw, sign); break;
            case 12: block_pass_r<12>(dif, p, pass, data, dl, ls, es, line_fastest, tw, sign); break;
            case 16: block_pass_r<16>(dif, p, pass, data, dl, ls, es, line_fastest, tw, sign); break;
            default:
                block_prime_pass(dif, p, pass, data, dl, ls, es, line_fastest, tw, sign);
                break;
        }
        __syncthreads();
    }
}

// table[t] = e^{+2 pi i t / n}
__device__ inline void block_fill_roots(cfloat* table, int n) {
    for (int t = threadIdx.x; t < n; t += blockDim.x) table[t] = unit_root(t, n, +1);
}
#endif

}  // namespace ampcor
