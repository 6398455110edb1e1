/*
 * AmpcorFFT.h - FFTW-free stand-in for the reference CPU port's FFT wrapper,
 * used only to build the reference's C++ CPU ampcor as a timed baseline
 * (test infrastructure, never shipped).
 *
 * The reference wraps FFTW (components/zerodop/GPUampcor/include/
 * AmpcorFFT.h:15-23, src/AmpcorFFT.cpp:20-67): fft1d(n, data, dir) on a
 * power-of-two length 4..65536, in place and unnormalised; dir 0 prepares a
 * plan, -1 runs the forward (e^{-i}) transform, +1 the backward (e^{+i})
 * one, 2 releases the plan.  FFTW is not installed on either machine; this
 * class keeps that call and runs an iterative radix-2 transform with
 * precomputed bit-reversal and twiddle tables per length
 * (ampcor_fft_shim.cpp).  Any exact DFT gives the same numbers up to float
 * rounding; a slower FFT only makes the timed baseline slower, so the
 * baseline's FFT is named wherever its time is reported.
 */
#ifndef AMPCOR_REF_SHIM_AMPCORFFT_H
#define AMPCOR_REF_SHIM_AMPCORFFT_H

#include <complex>
#include <vector>

#include "Constants.h"

struct AmpcorFFT {
    struct Plan {
        int n = 0;
        std::vector<int> rev;                   // bit-reversal permutation
        std::vector<std::complex<float> > tw;   // e^{-2 pi i k / n}, k < n/2
    };
    std::vector<Plan> plans = std::vector<Plan>(17);

    void fft1d(int nPoints, std::complex<float>* imgArr, int fftDir);
};

#endif
