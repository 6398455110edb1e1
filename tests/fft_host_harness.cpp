// Test-only host driver of the shared-memory FFT pass functions: runs every
// work item of every pass sequentially (the loop boundary stands in for the
// block barrier) so the index logic can be checked against numpy on a CPU.
#include <vector>
#include "fft_smem.cuh"

using namespace ampcor;

static void run_lines(bool dif, const FftPlan1D& p, cfloat* d, int nlines, int ls, int es, bool lf, int sign) {
    std::vector<cfloat> tw(p.n);
    for (int t = 0; t < p.n; ++t) tw[t] = unit_root(t, p.n, +1);
    for (int s = 0; s < p.npass; ++s) {
        int pass = dif ? s : p.npass - 1 - s;
        int items = fft_pass_items(p, pass, nlines);
        for (int it = 0; it < items; ++it) fft_pass_item(dif, p, pass, d, nlines, ls, es, lf, it, tw.data(), sign);
    }
}

extern "C" {
// 2-D: rows (length n2) then columns (length n1) for DIF; reverse for DIT.
int h_fft2(int dif, float* data, int n1, int n2, int sign) {
    FftPlan1D p1, p2;
    if (!fft_plan_make(n1, &p1) || !fft_plan_make(n2, &p2)) return 1;
    cfloat* d = reinterpret_cast<cfloat*>(data);
    if (dif) {
        run_lines(true, p2, d, n1, n2, 1, false, sign);
        run_lines(true, p1, d, n2, 1, n2, true, sign);
    } else {
        run_lines(false, p1, d, n2, 1, n2, true, sign);
        run_lines(false, p2, d, n1, n2, 1, false, sign);
    }
    return 0;
}
int h_pos_to_freq(int n, int pos) { FftPlan1D p; fft_plan_make(n, &p); return fft_pos_to_freq(p, pos); }
int h_freq_to_pos(int n, int f) { FftPlan1D p; fft_plan_make(n, &p); return fft_freq_to_pos(p, f); }
int h_good_size(int n) { return fft_good_size(n); }
}
