// Kernel declarations and shared-memory sizing for the dense ampcor stages.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>
#include "ampcor_plan.h"

namespace ampcor {

// One job of a persistent batched launch (device copy).
struct BatchJob {
    WindowPlan P;
    const cfloat* ref;
    const cfloat* sec;
    long long ldr, lds;
    const WindowCoords* coords;
    float2* offset;
    float* snr;
    float* cov;
    int merge;
    int pad;
};

// Byte offsets inside one CTA's scratch slot of the persistent kernel.
struct SlotLayout {
    size_t vbox, rawl2, osl2, osRef, osSch, surf, res, bytes;
};

// Threads per CTA of the plain-path kernels whose shared-memory layout
// depends on the thread count.
constexpr int kCosThreads = 256;
constexpr int kZoomThreads = 256;
constexpr int kMaxDirectZp = 128;  // largest kept oversampled surface side (direct-sum correlation)
constexpr int kCosTcMaxZp = 16;    // largest kept surface side of the tensor-core oversampled correlation
// sinc surface oversampler: kernel length int(6 / 0.75 + 0.5) and phases per
// input sample (cuSincOverSampler.h:30-45, cuSincOverSampler.cu:24-25)
constexpr int kSincLen = 8;
constexpr int kSincPhases = 4096;

// Largest dynamic shared memory of any stage body run by a CTA of nt threads.
size_t batch_smem_bytes(const WindowPlan& P, int nt);
SlotLayout batch_slot_layout(const WindowPlan* plans, int n);
bool fit_plan_smem(WindowPlan& P, int nt, size_t limit);
void plan_enable_bulk_corr(WindowPlan& P, int nt, size_t limit);
cudaError_t launch_persist(int nt, int per_sm, int grid, size_t smem, cudaStream_t st, const BatchJob* jobs,
                           const int2* items, int nitems, int* next, unsigned char* scratch, const SlotLayout& L);
int persist_blocks_per_sm(int nt, int per_sm, size_t smem);
// one per compiled launch shape of the persistent kernel
cudaError_t launch_persist_512x1(int grid, size_t smem, cudaStream_t st, const BatchJob* jobs, const int2* items,
                                 int nitems, int* next, unsigned char* scratch, const SlotLayout& L);
cudaError_t launch_persist_256x1(int grid, size_t smem, cudaStream_t st, const BatchJob* jobs, const int2* items,
                                 int nitems, int* next, unsigned char* scratch, const SlotLayout& L);
cudaError_t launch_persist_256x2(int grid, size_t smem, cudaStream_t st, const BatchJob* jobs, const int2* items,
                                 int nitems, int* next, unsigned char* scratch, const SlotLayout& L);
int persist_occupancy_512x1(size_t smem);
int persist_occupancy_256x1(size_t smem);
int persist_occupancy_256x2(size_t smem);

// Batched chain (four persistent stage kernels over a wave of mixed items).
constexpr int kWaveRawThreads = 512;
constexpr int kWaveOsThreads = 256;
constexpr int kWaveCosThreads = 512;
constexpr int kWaveZoomThreads = 256;
struct WaveLayout {
    RawResult* res;                        // per item
    float* osRef;                          // per item, osRefStride floats apart
    float* osSch;
    float* surf;
    size_t osRefStride, osSchStride, surfStride;
    unsigned char* slots;                  // per CTA of the raw / oversampling kernels
    size_t slotBytes;
    SlotLayout L;                          // vbox, rawl2 and osl2 offsets inside a slot
};
size_t wave_stage_smem(const WindowPlan& P, int stage);
bool corr_os_bulk_applies(const WindowPlan& P);
size_t corr_os_bulk_smem_bytes(const WindowPlan& P, int cols, int nt);
int wave_blocks_per_sm(int stage, const WindowPlan& P, size_t smem);
int wave_path_key(const WindowPlan& P);
bool launch_wave_cos_tma(const WindowPlan& P, int n, cudaStream_t st, const WaveLayout& W, int* err);


// Plans of the jobs in one wave, passed in the launch parameters.
constexpr int kWavePlans = 9;  // 9 plans of 3 252 bytes fit the 32 764-byte parameter space
struct WavePlans {
    int count;
    int job[kWavePlans];
    WindowPlan P[kWavePlans];
};
cudaError_t launch_wave_stage(int stage, int grid, size_t smem, cudaStream_t st, const WavePlans& WP,
                              const BatchJob* jobs, const int2* items, int i0, int n, const WaveLayout& W,
                              int* err);

// One wave of the chain and the plan of a whole chain run.
struct ChainWave {
    int i0, n;
    size_t smem[4];
    int grid[4];
    bool single_geometry;  // every job of the wave has the same chip sizes
    WavePlans plans;
};
struct ChainPlan {
    std::vector<ChainWave> waves;
    size_t osr = 0, oss = 0, sf = 0;  // per-item strides (floats) of the wave workspace
    SlotLayout L{};
    size_t slotBytes = 0;
    int maxGrid01 = 1, nmax = 0;
    size_t bytes() const;              // wave workspace bytes
};
// by_geometry: cut waves where the chip sizes change, so that every wave can
// use the TMA-staged correlation and each window's code path depends on its
// own plan only.
bool plan_chain(const std::vector<WindowPlan>& plans, const std::vector<int2>& items, int sms, size_t budget,
                ChainPlan* out, std::string* err, bool by_geometry = false);
void chain_layout(const ChainPlan& C, unsigned char* base, WaveLayout* W);
// Optional stage timing of a chain run (event pairs around every launch).
struct ChainTimer {
    virtual cudaError_t begin(int stage, cudaStream_t st) const = 0;
    virtual cudaError_t end(int stage, cudaStream_t st) const = 0;
    virtual ~ChainTimer() {}
};
cudaError_t launch_chain(const ChainPlan& C, const WaveLayout& W, const BatchJob* jobs, const int2* items,
                         cudaStream_t st, int* err, const ChainTimer* timer = nullptr);

size_t raw_smem_bytes(const WindowPlan& P);
size_t raw_l2_smem_bytes(const WindowPlan& P);
size_t raw_l2_slot_bytes(const WindowPlan& P);
size_t os_smem_bytes(const WindowPlan& P);
size_t corr_os_smem_bytes(const WindowPlan& P, int nt = kCosThreads);
size_t zoom_smem_bytes(const WindowPlan& P, int nt = kZoomThreads);
size_t os2_smem_bytes(const WindowPlan& P);
// raw = 2 with even chip sides: the separable oversampler applies
__host__ __device__ inline bool os2_applies(const WindowPlan& P) {
    return P.raw == 2 && P.Wh % 2 == 0 && P.Ww % 2 == 0 && P.Hz % 2 == 0 && P.Wz % 2 == 0;
}

// tensor-core oversampler (split-BF16 or BF16 contractions)
constexpr int kOsTcThreads = 256;
constexpr int kOsTcMaxSide = 80;
__host__ __device__ inline int pad16(int n) { return (n + 15) & ~15; }
__host__ __device__ inline bool os_tc_applies(const WindowPlan& P) {
    return os2_applies(P) && pad16(P.Wh) <= kOsTcMaxSide && pad16(P.Ww) <= kOsTcMaxSide &&
           pad16(P.Hz) <= kOsTcMaxSide && pad16(P.Wz) <= kOsTcMaxSide;
}
inline size_t os_tc_smem_bytes(const WindowPlan& P) {
    const int np = (pad16(P.Wh) > pad16(P.Ww) ? pad16(P.Wh) : pad16(P.Ww)) > (pad16(P.Hz) > pad16(P.Wz) ? pad16(P.Hz) : pad16(P.Wz))
                       ? (pad16(P.Wh) > pad16(P.Ww) ? pad16(P.Wh) : pad16(P.Ww))
                       : (pad16(P.Hz) > pad16(P.Wz) ? pad16(P.Hz) : pad16(P.Wz));
    const size_t K = 2 * (size_t)np;
    return 128 + 128 * K * 4 + K * K * 4 + 40 * sizeof(double) + 64;  // + alignment of the base to 128
}
__global__ void k_oversample_tc(const __grid_constant__ WindowPlan P, const cfloat* __restrict__ ref, long long ldr,
                                const cfloat* __restrict__ sec, long long lds,
                                const WindowCoords* __restrict__ coords, int w0, int wend,
                                RawResult* __restrict__ res, float* __restrict__ osRef, float* __restrict__ osSch,
                                const uint4* __restrict__ tabRow0, const uint4* __restrict__ tabCol0,
                                const uint4* __restrict__ tabRow1, const uint4* __restrict__ tabCol1,
                                int* __restrict__ err);
size_t os2_l2_smem_bytes(const WindowPlan& P);
size_t os2_l2_slot_bytes(const WindowPlan& P);
constexpr int kOs2L2Threads = 256;
__global__ void k_oversample2_l2(const __grid_constant__ WindowPlan P, const cfloat* __restrict__ ref, long long ldr,
                                 const cfloat* __restrict__ sec, long long lds,
                                 const WindowCoords* __restrict__ coords, int w0, int wend,
                                 RawResult* __restrict__ res, float* __restrict__ osRef, float* __restrict__ osSch,
                                 unsigned char* __restrict__ slots, size_t slot_bytes);

__global__ void k_raw(const __grid_constant__ WindowPlan P, const cfloat* __restrict__ ref, long long ldr,
                      const cfloat* __restrict__ sec, long long lds, const WindowCoords* __restrict__ coords,
                      int w0, int wend, RawResult* __restrict__ res, float2* __restrict__ vbox);
int raw_l2_threads(const WindowPlan& P);
int raw_l2_blocks_per_sm(const WindowPlan& P);
cudaError_t launch_raw_l2(const WindowPlan& P, int grid, cudaStream_t st, const cfloat* ref, long long ldr,
                          const cfloat* sec, long long lds, const WindowCoords* coords, int w0, int wend,
                          RawResult* res, unsigned char* slots, size_t slot_bytes);
__global__ void k_oversample(const __grid_constant__ WindowPlan P, const cfloat* __restrict__ ref, long long ldr,
                             const cfloat* __restrict__ sec, long long lds,
                             const WindowCoords* __restrict__ coords, int w0, int wend,
                             RawResult* __restrict__ res, float* __restrict__ osRef, float* __restrict__ osSch);
__global__ void k_oversample2(const __grid_constant__ WindowPlan P, const cfloat* __restrict__ ref, long long ldr,
                              const cfloat* __restrict__ sec, long long lds,
                              const WindowCoords* __restrict__ coords, int w0, int wend,
                              RawResult* __restrict__ res, float* __restrict__ osRef, float* __restrict__ osSch);
void launch_oversample(const WindowPlan& P, int nb, cudaStream_t st, const cfloat* ref, long long ldr,
                       const cfloat* sec, long long lds, const WindowCoords* coords, int w0, int wend,
                       RawResult* res, float* osRef, float* osSch);
void launch_corr_os(const WindowPlan& P, int nb, cudaStream_t st, int w0, int wend, const RawResult* res,
                    const float* osRef, const float* osSch, float* surf);
bool corr_os_supported(int zp);
void launch_corr_os_best(const WindowPlan& P, int nb, cudaStream_t st, int w0, int wend, const RawResult* res,
                         const float* osRef, const float* osSch, float* surf, int* err);
int cos_tc_band_groups(const WindowPlan& P);
bool launch_corr_os_tc(const WindowPlan& P, int nb, cudaStream_t st, int w0, int wend, const RawResult* res,
                       const float* osRef, const float* osSch, float* surf, int* err, long long tStride,
                       long long sStride, long long fStride);
bool launch_corr_os_tma(const WindowPlan& P, int nb, cudaStream_t st, int w0, int wend, const RawResult* res,
                        const float* osRef, const float* osSch, float* surf, int* err);
__global__ void k_zoom(const __grid_constant__ WindowPlan P, int w0, int wend, const RawResult* __restrict__ res,
                       const WindowCoords* __restrict__ coords, const float* __restrict__ surf, int merge_gross,
                       float2* __restrict__ offset, float* __restrict__ snr, float* __restrict__ cov,
                       int* __restrict__ diag);

}  // namespace ampcor
