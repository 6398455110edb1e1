// Internal state of a handle, shared by the C ABI translation units
// (ampcor_capi.cu: set-up and runs; ampcor_server.cu: the request server).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "ampcor_gb.h"
#include "ampcor_plan.h"

namespace ampcor {
constexpr size_t kSmemLimit = 232448;  // opt-in shared memory per block on sm_100/sm_103
constexpr size_t kWorkspaceBudget = size_t(1) << 30;
constexpr int kNumStages = 4;  // raw, oversample, oversampled correlation, zoom
}  // namespace ampcor

struct ampcor_handle {
    ampcor_params p{};
    bool is_setup = false;
    bool has_starts = false;
    ampcor::WindowPlan plan{};
    ampcor_geometry geo{};
    std::vector<int32_t> refD, refA, grossD, grossA;
    std::vector<ampcor::WindowCoords> coords;
    bool coords_dirty = true;
    int dev = -1;
    ampcor::WindowCoords* d_coords = nullptr;
    size_t coords_cap = 0;
    ampcor::RawResult* d_res = nullptr;
    size_t res_cap = 0;
    float* d_ws = nullptr;
    size_t ws_cap = 0;  // floats
    void* d_ref = nullptr;
    size_t ref_cap = 0;
    void* d_sec = nullptr;
    size_t sec_cap = 0;
    float* d_out = nullptr;
    size_t out_cap = 0;
    int32_t* d_diag = nullptr;
    size_t diag_cap = 0;
    // device error word of ampcor_run_device: set by a kernel whose bounded
    // wait gave up, kept until ampcor_run_status reads and clears it
    int* d_errw = nullptr;
    int last_run = 0;  // 0 none, 1 ampcor_run_device, 2 ampcor_run_device_noalloc
    bool attrs_set = false;
    int raw_mode = 0;    // 0 automatic, 1 shared-memory tile, 2 L2-staged tile
    int precision = 0;   // oversampler: 0 FP32 FFT, 1 split-BF16 tensor cores, 2 BF16 tensor cores
    int corr_precision = 0;  // oversampled correlation: 0 FP32, 1 split-BF16 tensor cores, 2 BF16 tensor cores
    unsigned char* d_tc = nullptr;  // shift tables of the tensor-core oversampler
    size_t tc_off[4] = {0, 0, 0, 0};  // tables for Ww, Wh, Wz, Hz
    int nsm = 0;         // SM count of the device
    int raw_l2_grid = 0; // resident CTAs of k_raw_l2 on the device
    int os_l2_grid = 0;  // resident CTAs of k_oversample2_l2 on the device
    // stage timing: one event pair around every launch while enabled
    bool timing = false;
    std::vector<cudaEvent_t> ev_start, ev_end;
    std::vector<int> ev_stage;
    size_t ev_used = 0;
    long long launches[ampcor::kNumStages] = {0, 0, 0, 0};
    std::string err;
};

