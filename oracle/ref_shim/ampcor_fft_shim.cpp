/*
 * Radix-2 body of the FFTW-free AmpcorFFT stand-in (see AmpcorFFT.h in this
 * directory): in-place, unnormalised, decimation in time after a
 * bit-reversal permutation, twiddles computed once per length in double and
 * stored as float.  Test infrastructure for the reference CPU build only.
 */
#include <cmath>
#include <cstdio>

#include "AmpcorFFT.h"

static int log2_exact(int n)
{
    int k = 0;
    while ((1 << k) < n) ++k;
    return ((1 << k) == n) ? k : -1;
}

void AmpcorFFT::fft1d(int n, std::complex<float>* a, int dir)
{
    const int k = log2_exact(n);
    if (k < 2 || k > 16) {
        std::printf("ERROR: FFT length of %d unsupported. Will not execute.\n", n);
        return;
    }
    Plan& p = plans[k];
    if (p.n != n) {  // build the tables (the reference's dir == 0 does this)
        p.n = n;
        p.rev.assign(n, 0);
        for (int i = 0; i < n; ++i) {
            int r = 0;
            for (int b = 0; b < k; ++b) r |= ((i >> b) & 1) << (k - 1 - b);
            p.rev[i] = r;
        }
        p.tw.resize(n / 2);
        for (int i = 0; i < n / 2; ++i) {
            const double ang = -2.0 * M_PI * (double)i / (double)n;
            p.tw[i] = std::complex<float>((float)std::cos(ang), (float)std::sin(ang));
        }
    }
    if (dir == 0 || dir == 2) return;
    if (dir != -1 && dir != 1) {
        std::printf("ERROR: Unspecified 'dir' flag (received '%d'), FFT will not execute.\n", dir);
        return;
    }
    for (int i = 0; i < n; ++i) {
        const int r = p.rev[i];
        if (r > i) std::swap(a[i], a[r]);
    }
    const bool inverse = (dir == 1);
    for (int len = 2; len <= n; len <<= 1) {
        const int half = len >> 1;
        const int step = n / len;
        for (int s = 0; s < n; s += len) {
            for (int j = 0; j < half; ++j) {
                std::complex<float> w = p.tw[j * step];
                if (inverse) w = std::conj(w);
                const std::complex<float> u = a[s + j];
                const std::complex<float> v = a[s + j + half] * w;
                a[s + j] = u + v;
                a[s + j + half] = u - v;
            }
        }
    }
}
