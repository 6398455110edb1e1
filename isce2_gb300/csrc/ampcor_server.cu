// Request server: continuous batching of offset-tracking requests on one GPU.
//
// No counterpart in the reference, whose controller runs one image pair per
// call (cuAmpcorController.cpp:37-178).  A request is a set-up handle (its
// plan and start pixels are copied at submission) plus two images.  The
// server
//   * admits queued requests in arrival order while their device memory
//     (images, start pixels, output fields) fits the HBM budget, copying the
//     images into server-owned memory from a stream-ordered pool on an
//     ingest stream;
//   * builds steps of at most `step_windows` windows taken from the admitted
//     requests, oldest first, and runs each step as the batched chain on the
//     compute stream, keeping two steps in flight so
//     that requests arriving meanwhile join the next step (iteration-level
//     batching: a request's windows may span several steps and a step mixes
//     windows of many requests);
//   * retires steps as their completion events fire, marks requests whose
//     windows are all done as complete, and hands their fields out on a
//     separate output stream, after which their memory returns to the budget.
// Each step runs as the batched chain (four stage kernels per wave of
// windows of one chip geometry; the waves of a step spread over several
// streams so that small ones overlap), and a window's arithmetic depends only on
// its own job plan, so a request's results are bit-identical whether it runs
// alone or in any mix, and equal to the plain chain's.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <string>
#include <unordered_map>
#include <vector>

#include "ampcor_gb.h"
#include "ampcor_internal.h"
#include "ampcor_kernels.h"

using namespace ampcor;

namespace {

constexpr size_t kStepWorkspace = size_t(2) << 30;  // wave workspace of one wave stream
constexpr int kStepRing = 3;      // step slots (staging buffers); at most two in flight
constexpr int kMaxInFlight = 2;
// A step's waves (one chip geometry each, so usually one request each) run on
// this many streams at once, each stream with its own workspace region:
// the small waves of small requests then share the GPU instead of taking
// turns on it.
constexpr int kWaveStreams = 4;

enum ReqState { kQueued = 0, kActive = 1, kComplete = 2 };

struct Request {
    int64_t id = 0;
    WindowPlan P{};
    int merge = 0;
    int nwin = 0;
    std::vector<WindowCoords> coords;
    const void* src_ref = nullptr;
    const void* src_sec = nullptr;
    int64_t src_ref_ld = 0, src_sec_ld = 0;
    int on_device = 0;
    int ref_rows = 0, ref_cols = 0, sec_rows = 0, sec_cols = 0;
    size_t bytes = 0;
    unsigned char* mem = nullptr;
    cfloat* ref = nullptr;
    cfloat* sec = nullptr;
    WindowCoords* d_coords = nullptr;
    float* d_off = nullptr;
    float* d_snr = nullptr;
    float* d_cov = nullptr;
    cudaEvent_t ready = nullptr;   // images and start pixels copied
    bool waited = false;           // compute stream already waits on `ready`
    int next = 0;                  // next window to schedule
    int done = 0;                  // windows finished
    int state = kQueued;
    double t_submit = 0, t_admit = 0, t_done = 0;
};

struct Step {
    cudaEvent_t ev = nullptr;
    cudaEvent_t ev_start = nullptr;               // staging copies done, waves may start
    cudaEvent_t ev_wave[kWaveStreams] = {};       // each wave stream's share done
    bool in_flight = false;
    std::vector<std::pair<int64_t, int>> parts;  // (request, windows in this step)
    BatchJob* h_jobs = nullptr;                  // pinned staging
    int2* h_items = nullptr;
    BatchJob* d_jobs = nullptr;
    int2* d_items = nullptr;
    size_t jobs_cap = 0, items_cap = 0;
};

size_t a256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

struct ampcor_server {
    int dev = 0;
    size_t budget = 0, used = 0, peak_used = 0;
    int step_windows = 8192;
    cudaMemPool_t pool = nullptr;
    cudaStream_t in_stream = nullptr, out_stream = nullptr;
    cudaStream_t wave_stream[kWaveStreams] = {};
    std::deque<int64_t> queued;
    std::vector<int64_t> active;  // admitted and not complete, in arrival order
    std::unordered_map<int64_t, Request> reqs;
    std::vector<int64_t> completed;  // complete, not yet reported by poll
    Step steps[kStepRing];
    std::deque<int> inflight;  // step slots in launch order
    unsigned char* scratch = nullptr;  // wave workspace of the steps (stream-ordered reuse)
    size_t scratch_cap = 0;
    int* d_next = nullptr;  // work counter, device error word
    int* h_err = nullptr;   // error word after each step (pinned, one per step slot)
    int sms = 0;
    int64_t next_id = 1;
    long long steps_launched = 0, windows_done = 0, max_active = 0;
    std::chrono::steady_clock::time_point t0;
    std::string err;
};

static int sfail(ampcor_server* s, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (s) s->err = buf;
    return code;
}

#define SCUDA_TRY(s, call)                                                                        \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return sfail(s, AMPCOR_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));     \
    } while (0)

static double now_s(const ampcor_server* s) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - s->t0).count();
}

extern "C" int ampcor_server_create(ampcor_server** out, int32_t deviceID, int64_t hbm_budget_bytes,
                                    int32_t step_windows) {
    if (!out || hbm_budget_bytes <= 0 || step_windows <= 0) return AMPCOR_ERR_ARG;
    *out = nullptr;
    ampcor_server* s = new (std::nothrow) ampcor_server();
    if (!s) return AMPCOR_ERR_ALLOC;
    s->dev = deviceID;
    s->budget = (size_t)hbm_budget_bytes;
    s->step_windows = step_windows;
    s->t0 = std::chrono::steady_clock::now();
    auto bad = [&](cudaError_t e, const char* what) {
        std::fprintf(stderr, "ampcor_server_create: %s: %s\n", what, cudaGetErrorString(e));
        delete s;
        return AMPCOR_ERR_CUDA;
    };
    cudaError_t e = cudaSetDevice(deviceID);
    if (e != cudaSuccess) return bad(e, "cudaSetDevice");
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = deviceID;
    if ((e = cudaMemPoolCreate(&s->pool, &props)) != cudaSuccess) return bad(e, "cudaMemPoolCreate");
    uint64_t keep = (uint64_t)hbm_budget_bytes;  // keep freed blocks for reuse up to the budget
    cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    if ((e = cudaStreamCreateWithFlags(&s->in_stream, cudaStreamNonBlocking)) != cudaSuccess)
        return bad(e, "cudaStreamCreate");
    if ((e = cudaStreamCreateWithFlags(&s->out_stream, cudaStreamNonBlocking)) != cudaSuccess)
        return bad(e, "cudaStreamCreate");
    for (cudaStream_t& ws : s->wave_stream)
        if ((e = cudaStreamCreateWithFlags(&ws, cudaStreamNonBlocking)) != cudaSuccess)
            return bad(e, "cudaStreamCreate");
    for (Step& st : s->steps) {
        if ((e = cudaEventCreateWithFlags(&st.ev, cudaEventDisableTiming)) != cudaSuccess)
            return bad(e, "cudaEventCreate");
        if ((e = cudaEventCreateWithFlags(&st.ev_start, cudaEventDisableTiming)) != cudaSuccess)
            return bad(e, "cudaEventCreate");
        for (cudaEvent_t& we : st.ev_wave)
            if ((e = cudaEventCreateWithFlags(&we, cudaEventDisableTiming)) != cudaSuccess)
                return bad(e, "cudaEventCreate");
    }
    if ((e = cudaMalloc(&s->d_next, 2 * sizeof(int))) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = cudaMemset(s->d_next, 0, 2 * sizeof(int))) != cudaSuccess) return bad(e, "cudaMemset");
    if ((e = cudaMallocHost(&s->h_err, kStepRing * sizeof(int))) != cudaSuccess) return bad(e, "cudaMallocHost");
    if ((e = cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, deviceID)) != cudaSuccess)
        return bad(e, "cudaDeviceGetAttribute");
    *out = s;
    return AMPCOR_OK;
}

static void release_request(ampcor_server* s, Request& r, cudaStream_t st) {
    if (r.mem) {
        cudaFreeAsync(r.mem, st);
        s->used -= r.bytes;
        r.mem = nullptr;
    }
    if (r.ready) {
        cudaEventDestroy(r.ready);
        r.ready = nullptr;
    }
}

extern "C" int ampcor_server_destroy(ampcor_server* s) {
    if (!s) return AMPCOR_ERR_ARG;
    cudaSetDevice(s->dev);
    cudaDeviceSynchronize();
    for (auto& kv : s->reqs) release_request(s, kv.second, s->out_stream);
    cudaStreamSynchronize(s->out_stream);
    for (Step& st : s->steps) {
        if (st.ev) cudaEventDestroy(st.ev);
        if (st.ev_start) cudaEventDestroy(st.ev_start);
        for (cudaEvent_t we : st.ev_wave)
            if (we) cudaEventDestroy(we);
        cudaFreeHost(st.h_jobs);
        cudaFreeHost(st.h_items);
        cudaFree(st.d_jobs);
        cudaFree(st.d_items);
    }
    if (s->scratch) cudaFree(s->scratch);
    cudaFree(s->d_next);
    cudaFreeHost(s->h_err);
    if (s->in_stream) cudaStreamDestroy(s->in_stream);
    if (s->out_stream) cudaStreamDestroy(s->out_stream);
    for (cudaStream_t ws : s->wave_stream)
        if (ws) cudaStreamDestroy(ws);
    if (s->pool) cudaMemPoolDestroy(s->pool);
    delete s;
    return AMPCOR_OK;
}

extern "C" int ampcor_server_submit(ampcor_server* s, ampcor_handle* h, const void* ref, int64_t ref_ld,
                                    const void* sec, int64_t sec_ld, int32_t images_on_device,
                                    int64_t* request_id) {
    if (!s || !h || !ref || !sec) return AMPCOR_ERR_ARG;
    s->err.clear();
    if (!h->is_setup || !h->has_starts)
        return sfail(s, AMPCOR_ERR_STATE, "setupParams and a gross-offset setter must be called before submission");
    int rc = ampcor_check_range(h);
    if (rc) return sfail(s, rc, "%s", h->err.c_str());
    if (ref_ld < h->p.referenceImageWidth || sec_ld < h->p.secondaryImageWidth)
        return sfail(s, AMPCOR_ERR_ARG, "leading dimension smaller than the image width");
    if (!corr_os_supported(h->plan.zp))
        return sfail(s, AMPCOR_ERR_UNSUPPORTED,
                     "kept oversampled surface side %d runs only through ampcor_run_device", h->plan.zp);
    if (h->p.deviceID != s->dev) return sfail(s, AMPCOR_ERR_ARG, "request for device %d, server on %d",
                                              h->p.deviceID, s->dev);
    // every stage body fits by set-up; the oversampled correlation of chips
    // without a TMA path is double-buffered by bulk copies when that fits
    // (all a function of the request's own plan)
    WindowPlan P = h->plan;
    P.cosCols = 0;
    if (corr_os_bulk_applies(P))
        for (int c : {32, 16})
            if (corr_os_bulk_smem_bytes(P, c, kWaveCosThreads) <= kSmemLimit) {
                P.cosCols = c;
                break;
            }
    Request r;
    r.id = s->next_id++;
    r.P = P;
    r.merge = h->p.mergeGrossOffset;
    r.nwin = h->geo.numberWindows;
    r.coords = h->coords;
    r.src_ref = ref;
    r.src_sec = sec;
    r.src_ref_ld = ref_ld;
    r.src_sec_ld = sec_ld;
    r.on_device = images_on_device != 0;
    r.ref_rows = h->p.referenceImageHeight;
    r.ref_cols = h->p.referenceImageWidth;
    r.sec_rows = h->p.secondaryImageHeight;
    r.sec_cols = h->p.secondaryImageWidth;
    r.bytes = a256((size_t)r.ref_rows * r.ref_cols * sizeof(cfloat)) +
              a256((size_t)r.sec_rows * r.sec_cols * sizeof(cfloat)) +
              a256((size_t)r.nwin * sizeof(WindowCoords)) + a256((size_t)r.nwin * 6 * sizeof(float));
    if (r.bytes > s->budget)
        return sfail(s, AMPCOR_ERR_ALLOC, "request needs %zu bytes of device memory, the budget is %zu", r.bytes,
                     s->budget);
    r.t_submit = now_s(s);
    const int64_t id = r.id;
    s->reqs.emplace(id, std::move(r));
    s->queued.push_back(id);
    if (request_id) *request_id = id;
    return AMPCOR_OK;
}

// Admit queued requests in arrival order while they fit the budget.
static int admit(ampcor_server* s) {
    while (!s->queued.empty()) {
        Request& r = s->reqs.at(s->queued.front());
        if (s->used + r.bytes > s->budget) break;
        void* mem = nullptr;
        SCUDA_TRY(s, cudaMallocFromPoolAsync(&mem, r.bytes, s->pool, s->in_stream));
        r.mem = static_cast<unsigned char*>(mem);
        s->used += r.bytes;
        s->peak_used = std::max(s->peak_used, s->used);
        size_t off = 0;
        r.ref = reinterpret_cast<cfloat*>(r.mem + off);
        off += a256((size_t)r.ref_rows * r.ref_cols * sizeof(cfloat));
        r.sec = reinterpret_cast<cfloat*>(r.mem + off);
        off += a256((size_t)r.sec_rows * r.sec_cols * sizeof(cfloat));
        r.d_coords = reinterpret_cast<WindowCoords*>(r.mem + off);
        off += a256((size_t)r.nwin * sizeof(WindowCoords));
        r.d_off = reinterpret_cast<float*>(r.mem + off);
        r.d_snr = r.d_off + 2 * (size_t)r.nwin;
        r.d_cov = r.d_snr + (size_t)r.nwin;
        const cudaMemcpyKind k = r.on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
        SCUDA_TRY(s, cudaMemcpy2DAsync(r.ref, (size_t)r.ref_cols * sizeof(cfloat), r.src_ref,
                                       (size_t)r.src_ref_ld * sizeof(cfloat), (size_t)r.ref_cols * sizeof(cfloat),
                                       (size_t)r.ref_rows, k, s->in_stream));
        SCUDA_TRY(s, cudaMemcpy2DAsync(r.sec, (size_t)r.sec_cols * sizeof(cfloat), r.src_sec,
                                       (size_t)r.src_sec_ld * sizeof(cfloat), (size_t)r.sec_cols * sizeof(cfloat),
                                       (size_t)r.sec_rows, k, s->in_stream));
        SCUDA_TRY(s, cudaMemcpyAsync(r.d_coords, r.coords.data(), (size_t)r.nwin * sizeof(WindowCoords),
                                     cudaMemcpyHostToDevice, s->in_stream));
        SCUDA_TRY(s, cudaEventCreateWithFlags(&r.ready, cudaEventDisableTiming));
        SCUDA_TRY(s, cudaEventRecord(r.ready, s->in_stream));
        r.state = kActive;
        r.t_admit = now_s(s);
        s->active.push_back(r.id);
        s->queued.pop_front();
    }
    s->max_active = std::max<long long>(s->max_active, (long long)s->active.size());
    return AMPCOR_OK;
}

// Retire completed steps (non-blocking).
static int retire(ampcor_server* s) {
    while (!s->inflight.empty()) {
        Step& st = s->steps[s->inflight.front()];
        const cudaError_t e = cudaEventQuery(st.ev);
        if (e == cudaErrorNotReady) break;
        if (e != cudaSuccess) return sfail(s, AMPCOR_ERR_CUDA, "server step failed: %s", cudaGetErrorString(e));
        if (s->h_err[s->inflight.front()])
            return sfail(s, AMPCOR_ERR_CUDA, "a device-side wait gave up in a server step (its results are invalid)");
        const double t = now_s(s);
        for (const auto& part : st.parts) {
            Request& r = s->reqs.at(part.first);
            r.done += part.second;
            s->windows_done += part.second;
            if (r.done == r.nwin) {
                r.state = kComplete;
                r.t_done = t;
                s->completed.push_back(r.id);
                s->active.erase(std::find(s->active.begin(), s->active.end(), r.id));
            }
        }
        st.parts.clear();
        st.in_flight = false;
        s->inflight.pop_front();
    }
    return AMPCOR_OK;
}

template <typename T>
static int grow_pair(ampcor_server* s, T** h, T** d, size_t* cap, size_t n) {
    if (*cap >= n) return AMPCOR_OK;
    cudaFreeHost(*h);
    cudaFree(*d);
    *h = nullptr;
    *d = nullptr;
    *cap = 0;
    const size_t m = std::max<size_t>(n, 1024);
    SCUDA_TRY(s, cudaMallocHost((void**)h, m * sizeof(T)));
    SCUDA_TRY(s, cudaMalloc((void**)d, m * sizeof(T)));
    *cap = m;
    return AMPCOR_OK;
}

// Build and launch one step from the admitted requests, oldest first.
static int launch_step(ampcor_server* s, cudaStream_t stream, bool* launched) {
    *launched = false;
    int slot = -1;
    for (int i = 0; i < kStepRing; ++i)
        if (!s->steps[i].in_flight) { slot = i; break; }
    if (slot < 0) return AMPCOR_OK;
    Step& st = s->steps[slot];
    std::vector<int64_t> ids;
    std::vector<int> counts;
    int room = s->step_windows;
    for (int64_t id : s->active) {
        if (room == 0) break;
        Request& r = s->reqs.at(id);
        const int n = std::min(room, r.nwin - r.next);
        if (n <= 0) continue;
        ids.push_back(id);
        counts.push_back(n);
        room -= n;
    }
    if (ids.empty()) return AMPCOR_OK;
    int rc;
    // staging buffers: a step slot is reused only after its step retired
    if ((rc = grow_pair(s, &st.h_jobs, &st.d_jobs, &st.jobs_cap, ids.size()))) return rc;
    if ((rc = grow_pair(s, &st.h_items, &st.d_items, &st.items_cap, (size_t)(s->step_windows - room)))) return rc;
    std::vector<WindowPlan> plans;
    std::vector<int2> items;
    int nitems = 0;
    for (size_t j = 0; j < ids.size(); ++j) {
        Request& r = s->reqs.at(ids[j]);
        BatchJob J{};
        J.P = r.P;
        J.ref = r.ref;
        J.sec = r.sec;
        J.ldr = r.ref_cols;
        J.lds = r.sec_cols;
        J.coords = r.d_coords;
        J.offset = reinterpret_cast<float2*>(r.d_off);
        J.snr = r.d_snr;
        J.cov = r.d_cov;
        J.merge = r.merge;
        st.h_jobs[j] = J;
        plans.push_back(r.P);
        for (int w = r.next; w < r.next + counts[j]; ++w) {
            st.h_items[nitems++] = make_int2((int)j, w);
            items.push_back(make_int2((int)j, w));
        }
        r.next += counts[j];
        st.parts.emplace_back(ids[j], counts[j]);
        if (!r.waited) {
            SCUDA_TRY(s, cudaStreamWaitEvent(stream, r.ready, 0));
            r.waited = true;
        }
    }
    // the step runs as the batched chain: four stage kernels per wave, waves
    // of one chip geometry (so every window's code path is its plan's)
    ChainPlan C;
    std::string msg;
    if (!plan_chain(plans, items, s->sms, kStepWorkspace, &C, &msg, true))
        return sfail(s, AMPCOR_ERR_UNSUPPORTED, "%s", msg.c_str());
    // the waves are independent (disjoint items and outputs): spread them over
    // the wave streams, the costliest first onto the least loaded stream, each
    // stream keeping launch order and its own workspace region
    const int G = std::min<int>(kWaveStreams, (int)C.waves.size());
    std::vector<ChainPlan> parts(G);
    {
        std::vector<int> order(C.waves.size());
        std::vector<double> cost(C.waves.size()), load(G, 0.0);
        for (size_t i = 0; i < C.waves.size(); ++i) {
            const WindowPlan& P = C.waves[i].plans.P[0];
            order[i] = (int)i;
            cost[i] = (double)C.waves[i].n * ((double)P.P * P.Q + 2.0 * P.osHz * P.osWz + (double)P.osWh * P.osWw);
        }
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
        std::vector<std::vector<int>> pick(G);
        for (int i : order) {
            const int g = (int)(std::min_element(load.begin(), load.end()) - load.begin());
            pick[g].push_back(i);
            load[g] += cost[i];
        }
        for (int g = 0; g < G; ++g) {
            std::sort(pick[g].begin(), pick[g].end());
            ChainPlan& Cg = parts[g];
            Cg = C;
            Cg.waves.clear();
            Cg.maxGrid01 = 1;
            Cg.nmax = 0;
            for (int i : pick[g]) {
                const ChainWave& w = C.waves[i];
                Cg.waves.push_back(w);
                Cg.nmax = std::max(Cg.nmax, w.n);
                Cg.maxGrid01 = std::max(Cg.maxGrid01, std::max(w.grid[0], w.plans.P[0].osL2 ? w.grid[1] : 0));
            }
        }
    }
    std::vector<size_t> part_off(G + 1, 0);
    for (int g = 0; g < G; ++g) part_off[g + 1] = part_off[g] + a256(parts[g].bytes());
    const size_t need = part_off[G];
    if (s->scratch_cap < need) {
        // stream-ordered: the old workspace is freed after the steps queued before
        if (s->scratch) SCUDA_TRY(s, cudaFreeAsync(s->scratch, stream));
        s->scratch = nullptr;
        s->scratch_cap = 0;
        void* p = nullptr;
        SCUDA_TRY(s, cudaMallocFromPoolAsync(&p, need, s->pool, stream));
        s->scratch = static_cast<unsigned char*>(p);
        s->scratch_cap = need;
    }
    SCUDA_TRY(s, cudaMemcpyAsync(st.d_jobs, st.h_jobs, ids.size() * sizeof(BatchJob), cudaMemcpyHostToDevice,
                                 stream));
    SCUDA_TRY(s, cudaMemcpyAsync(st.d_items, st.h_items, (size_t)nitems * sizeof(int2), cudaMemcpyHostToDevice,
                                 stream));
    SCUDA_TRY(s, cudaEventRecord(st.ev_start, stream));
    for (int g = 0; g < G; ++g) {
        WaveLayout W{};
        chain_layout(parts[g], s->scratch + part_off[g], &W);
        SCUDA_TRY(s, cudaStreamWaitEvent(s->wave_stream[g], st.ev_start, 0));
        SCUDA_TRY(s, launch_chain(parts[g], W, st.d_jobs, st.d_items, s->wave_stream[g], s->d_next + 1));
        SCUDA_TRY(s, cudaEventRecord(st.ev_wave[g], s->wave_stream[g]));
        SCUDA_TRY(s, cudaStreamWaitEvent(stream, st.ev_wave[g], 0));
    }
    SCUDA_TRY(s, cudaMemcpyAsync(s->h_err + slot, s->d_next + 1, sizeof(int), cudaMemcpyDeviceToHost, stream));
    SCUDA_TRY(s, cudaEventRecord(st.ev, stream));
    st.in_flight = true;
    s->inflight.push_back(slot);
    s->steps_launched += 1;
    *launched = true;
    return AMPCOR_OK;
}

extern "C" int ampcor_server_progress(ampcor_server* s, void* stream, int32_t* busy) {
    if (!s) return AMPCOR_ERR_ARG;
    s->err.clear();
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (!st) return sfail(s, AMPCOR_ERR_ARG, "the server needs a non-default compute stream");
    SCUDA_TRY(s, cudaSetDevice(s->dev));
    int rc;
    if ((rc = retire(s))) return rc;
    if ((rc = admit(s))) return rc;
    while ((int)s->inflight.size() < kMaxInFlight) {
        bool launched = false;
        if ((rc = launch_step(s, st, &launched))) return rc;
        if (!launched) break;
    }
    if (busy) *busy = (!s->inflight.empty() || !s->queued.empty() || !s->active.empty()) ? 1 : 0;
    return AMPCOR_OK;
}

extern "C" int ampcor_server_poll(ampcor_server* s, int64_t* ids, int32_t max_ids, int32_t* n) {
    if (!s || !n || (max_ids > 0 && !ids)) return AMPCOR_ERR_ARG;
    const int k = std::min<int>(max_ids, (int)s->completed.size());
    for (int i = 0; i < k; ++i) ids[i] = s->completed[i];
    s->completed.erase(s->completed.begin(), s->completed.begin() + k);
    *n = k;
    return AMPCOR_OK;
}

extern "C" int ampcor_server_take(ampcor_server* s, int64_t id, float* offset, float* snr, float* cov,
                                  int32_t dst_on_device) {
    if (!s) return AMPCOR_ERR_ARG;
    s->err.clear();
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return sfail(s, AMPCOR_ERR_ARG, "unknown request %lld", (long long)id);
    Request& r = it->second;
    if (r.state != kComplete) return sfail(s, AMPCOR_ERR_STATE, "request %lld is not complete", (long long)id);
    SCUDA_TRY(s, cudaSetDevice(s->dev));
    const cudaMemcpyKind k = dst_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    const size_t n = (size_t)r.nwin;
    if (offset) SCUDA_TRY(s, cudaMemcpyAsync(offset, r.d_off, 2 * n * sizeof(float), k, s->out_stream));
    if (snr) SCUDA_TRY(s, cudaMemcpyAsync(snr, r.d_snr, n * sizeof(float), k, s->out_stream));
    if (cov) SCUDA_TRY(s, cudaMemcpyAsync(cov, r.d_cov, 3 * n * sizeof(float), k, s->out_stream));
    release_request(s, r, s->out_stream);
    SCUDA_TRY(s, cudaStreamSynchronize(s->out_stream));
    s->reqs.erase(it);
    return AMPCOR_OK;
}

extern "C" int ampcor_server_request_info(const ampcor_server* s, int64_t id, int32_t* state, int32_t* windows,
                                          double* times) {
    if (!s) return AMPCOR_ERR_ARG;
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return AMPCOR_ERR_ARG;
    const Request& r = it->second;
    if (state) *state = r.state;
    if (windows) *windows = r.nwin;
    if (times) {
        times[0] = r.t_submit;
        times[1] = r.t_admit;
        times[2] = r.t_done;
    }
    return AMPCOR_OK;
}

extern "C" int ampcor_server_stats(const ampcor_server* s, int64_t* out, int32_t n) {
    if (!s || !out || n < AMPCOR_SERVER_STATS) return AMPCOR_ERR_ARG;
    out[0] = (int64_t)s->queued.size();
    out[1] = (int64_t)s->active.size();
    out[2] = (int64_t)s->inflight.size();
    out[3] = (int64_t)s->used;
    out[4] = (int64_t)s->peak_used;
    out[5] = (int64_t)s->steps_launched;
    out[6] = (int64_t)s->windows_done;
    out[7] = (int64_t)s->max_active;
    return AMPCOR_OK;
}

extern "C" int ampcor_server_last_error(const ampcor_server* s, char* buf, int64_t n) {
    if (!s || !buf || n <= 0) return AMPCOR_ERR_ARG;
    std::snprintf(buf, (size_t)n, "%s", s->err.c_str());
    return AMPCOR_OK;
}
