/*
 * ampcor_gb.h - C ABI of the GB300 dense amplitude cross-correlation engine.
 *
 * Drop-in boundary for ISCE2's PyCuAmpcor.  The reference exposes a pybind11
 * class (contrib/PyCuAmpcor/src/PyCuAmpcor.cpp:14-101) over
 * cuAmpcorController/cuAmpcorParameter; this header exports the same
 * parameter surface and the same five methods as plain C functions with
 * integer status codes (the reference calls exit() on errors,
 * cudaError.cpp:18-43, cuAmpcorParameter.cpp:100-103,283-327).
 *
 * Conventions (cuAmpcorParameter.h:16-21): "down" = azimuth = row = x,
 * "across" = range = column = y.  Images are complex64 (interleaved float
 * pairs), row-major, leading dimension given in elements.  Outputs are laid
 * out window-row-major: offset[2*w] = down, offset[2*w+1] = across;
 * cov[3*w] = xx, [3*w+1] = yy, [3*w+2] = xy (cuAmpcorController.cpp:129-158).
 *
 * Threading: a handle is used by one host thread at a time.  Calls on
 * different handles may run concurrently.
 */
#ifndef AMPCOR_GB_H
#define AMPCOR_GB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define AMPCOR_OK 0
#define AMPCOR_ERR_ARG 1          /* null pointer, bad size or value */
#define AMPCOR_ERR_RANGE 2        /* window outside the image (checkPixelInImageRange) */
#define AMPCOR_ERR_UNSUPPORTED 3  /* geometry the kernels do not handle */
#define AMPCOR_ERR_CUDA 4         /* a CUDA runtime call failed */
#define AMPCOR_ERR_STATE 5        /* call order (setup before start pixels, ...) */
#define AMPCOR_ERR_ALLOC 6        /* device or host allocation failed */

/* The PyCuAmpcor property set (PyCuAmpcor.cpp:31-76); names follow the
 * Python property names.  Defaults come from ampcor_params_default()
 * (cuAmpcorParameter.cpp:18-64). */
typedef struct ampcor_params {
    int32_t algorithm;                      /* 0 frequency domain, 1 time domain: same result */
    int32_t deviceID;
    int32_t nStreams;
    int32_t derampMethod;                   /* 0 amplitude, 1 complex with linear-ramp removal */
    int32_t referenceImageHeight;
    int32_t referenceImageWidth;
    int32_t secondaryImageHeight;
    int32_t secondaryImageWidth;
    int32_t numberWindowDown;
    int32_t numberWindowAcross;
    int32_t windowSizeHeight;               /* windowSizeHeightRaw */
    int32_t windowSizeWidth;                /* windowSizeWidthRaw */
    int32_t halfSearchRangeDown;
    int32_t halfSearchRangeAcross;
    int32_t skipSampleDown;
    int32_t skipSampleAcross;
    int32_t referenceStartPixelDownStatic;
    int32_t referenceStartPixelAcrossStatic;
    int32_t rawDataOversamplingFactor;
    int32_t corrStatWindowSize;
    int32_t corrSurfaceOverSamplingMethod;  /* 0 FFT, 1 sinc */
    int32_t corrSurfaceOverSamplingFactor;
    int32_t corrSurfaceZoomInWindow;
    int32_t numberWindowDownInChunk;
    int32_t numberWindowAcrossInChunk;
    int32_t mergeGrossOffset;
    int32_t useMmap;
    int32_t mmapSize;
} ampcor_params;

/* Derived geometry after ampcor_setup (cuAmpcorParameter::setupParameters,
 * cuAmpcorParameter.cpp:70-109). */
typedef struct ampcor_geometry {
    int32_t numberWindows;
    int32_t searchWindowSizeHeightRaw;
    int32_t searchWindowSizeWidthRaw;
    int32_t zoomWindowSize;                 /* after the min(zoom, 2*raw*min(hs)) clamp */
    int32_t halfZoomWindowSizeRaw;
    int32_t corrRawZoomInHeight;
    int32_t corrRawZoomInWidth;
    int32_t fftHeight;                      /* padded tile of the raw correlation */
    int32_t fftWidth;
} ampcor_geometry;

typedef struct ampcor_handle ampcor_handle;

/* Fill the reference defaults (cuAmpcorParameter.cpp:18-64). */
void ampcor_params_default(ampcor_params* p);

/* Replaces `PyCuAmpcor()` (PyCuAmpcor.cpp:15). */
int ampcor_create(ampcor_handle** out);
/* Frees the handle and its device workspace. */
int ampcor_destroy(ampcor_handle* h);

/* Replaces the property setters (PyCuAmpcor.cpp:31-76). */
int ampcor_set_params(ampcor_handle* h, const ampcor_params* p);
int ampcor_get_params(const ampcor_handle* h, ampcor_params* p);

/* Replaces setupParams() (PyCuAmpcor.cpp:84-86 -> cuAmpcorParameter.cpp:70-109). */
int ampcor_setup(ampcor_handle* h);
int ampcor_get_geometry(const ampcor_handle* h, ampcor_geometry* g);

/* Replaces setConstantGrossOffset(goDown, goAcross) (PyCuAmpcor.cpp:88-94
 * -> cuAmpcorParameter.cpp:189-205). */
int ampcor_set_constant_gross_offset(ampcor_handle* h, int32_t goDown, int32_t goAcross);

/* Replaces setVaryingGrossOffset(vD, vA) (PyCuAmpcor.cpp:95-101 ->
 * cuAmpcorParameter.cpp:170-186); n must equal numberWindows. */
int ampcor_set_varying_gross_offset(ampcor_handle* h, const int32_t* vD, const int32_t* vA, int64_t n);

/* The general form all three reference overloads reduce to
 * (cuAmpcorParameter.cpp:155-167): explicit reference starts + gross offsets. */
int ampcor_set_start_pixels(ampcor_handle* h, const int32_t* refD, const int32_t* refA,
                            const int32_t* grossD, const int32_t* grossA, int64_t n);

/* Copies back the per-window start pixels and gross offsets (int32, n each). */
int ampcor_get_start_pixels(const ampcor_handle* h, int32_t* refD, int32_t* refA, int32_t* grossD,
                            int32_t* grossA, int64_t n);

/* Replaces checkPixelInImageRange() (PyCuAmpcor.cpp:80-82 ->
 * cuAmpcorParameter.cpp:275-331): AMPCOR_ERR_RANGE instead of exit(). */
int ampcor_check_range(ampcor_handle* h);

/* Replaces runAmpcor() (cuAmpcorController.cpp:37-178) for images already
 * in device memory.  offset: 2*n float, snr: n float, cov: 3*n float, all
 * device pointers.  diag (optional, device, 8*n int32): raw arg-max (down,
 * across), clamped zoom start (down, across), zoom arg-max (down, across),
 * bit patterns of the raw peak value and the zoomed peak value.  `stream`
 * is a cudaStream_t (NULL = legacy default stream).  The call is
 * asynchronous with respect to the host: check the run with
 * ampcor_run_status once its work is done. */
int ampcor_run_device(ampcor_handle* h, const void* ref, int64_t ref_ld, const void* sec, int64_t sec_ld,
                      float* offset, float* snr, float* cov, int32_t* diag, void* stream);

/* Status of the handle's asynchronous runs (no counterpart in the reference,
 * whose runs are synchronous and exit() on errors).  Every kernel wait on a
 * copy is bounded; a wait that gives up sets a device error word and its run's
 * results are invalid.  This call waits for `stream`, reads that word (for
 * ampcor_run_device the handle's own word, set by any run since the last
 * status call; for ampcor_run_device_noalloc the word at the head of the
 * device's static scratch, shared by every handle on the device), clears it,
 * stores it in *device_error (may be NULL) and returns AMPCOR_ERR_CUDA if it
 * was set.  It allocates nothing. */
int ampcor_run_status(ampcor_handle* h, void* stream, int32_t* device_error);

/* Self-test of the bounded waits (no counterpart in the reference): launches
 * one block that waits on an mbarrier nothing ever completes, with a limit of
 * `polls` polls (1 .. 2^20); the wait gives up, the block sets the handle's
 * error word and returns, and the next ampcor_run_status reports
 * AMPCOR_ERR_CUDA.  The context stays usable. */
int ampcor_selftest_wait_timeout(ampcor_handle* h, uint32_t polls, void* stream);

/* As ampcor_run_device for host images and host outputs: copies the images
 * to the device, runs, copies the fields back and synchronises. */
int ampcor_run_host(ampcor_handle* h, const void* ref, int64_t ref_ld, const void* sec, int64_t sec_ld,
                    float* offset, float* snr, float* cov, int32_t* diag);

/* Allocation-free run (no counterpart in the reference).  For callers that
 * cannot call cudaMalloc — hosts whose own pool owns the device memory, or
 * hot paths where a driver allocation may synchronise the device or fail
 * under memory pressure.  Same arguments and results as ampcor_run_device
 * without `diag`, but all working memory (per-window coordinates and results
 * plus the stage workspace of the windows in flight) comes from one static
 * device array of AMPCOR_NOALLOC_SCRATCH_BYTES that the library module holds
 * on every GPU where it is loaded, until process exit.  Its device address is
 * looked up with cudaGetSymbolAddress on the first call on each device, so
 * make that first call before any stream capture.  Windows are processed in
 * batches that fit the array; a geometry whose coordinates and results for
 * all windows, plus one window's workspace, exceed it is rejected with
 * AMPCOR_ERR_UNSUPPORTED.  Every call shares the array: calls that overlap on
 * the GPU (other streams, other handles) race, so serialise them.  No call
 * reads what an earlier call left in the array, except the device error word
 * in its first bytes, which a run whose bounded wait gave up sets and which
 * stays set until ampcor_run_status reads and clears it.  The per-window
 * coordinates go up with a host-to-device copy from the handle's (pageable)
 * memory on `stream`. */
#define AMPCOR_NOALLOC_SCRATCH_BYTES (32u << 20)
int ampcor_run_device_noalloc(ampcor_handle* h, const void* ref, int64_t ref_ld, const void* sec, int64_t sec_ld,
                              float* offset, float* snr, float* cov, void* stream);

/* Stage timing (no counterpart in the reference, whose only timers are
 * prints in ampcor.F:1405,1412).  While enabled, every kernel launch of a run
 * is bracketed by CUDA events on the run's stream.  ampcor_read_timing waits
 * for the recorded events and returns, per stage (raw correlation,
 * oversampling, oversampled correlation, surface zoom; nstage >= 4), the summed
 * milliseconds and the number of launches since the last read, then resets. */
int ampcor_set_timing(ampcor_handle* h, int enable);
int ampcor_read_timing(ampcor_handle* h, float* ms, int64_t* launches, int32_t nstage);

/* Raw-correlation tile placement (no counterpart in the reference, which
 * always runs cuFFT on global buffers).  0 (default): the padded tile of the
 * raw correlation lives in shared memory when it fits, else in an
 * L2-resident global slot per resident CTA, staged through shared memory in
 * groups of lines; 1: shared memory only (ampcor_setup fails with
 * AMPCOR_ERR_UNSUPPORTED when the tile does not fit); 2: L2-staged always;
 * 3: L2-staged with 256-thread CTAs, two per SM (block sums in another
 * order: equal to the others within float32 rounding, not bit for bit).
 * Modes 0-2 give bit-identical results.  Takes effect at the next
 * ampcor_setup (the call clears the set-up state). */
int ampcor_set_raw_mode(ampcor_handle* h, int32_t mode);

/* Oversampler arithmetic (no counterpart in the reference, whose oversampler
 * is an FP32 cuFFT pair, cuOverSampler.cpp:72-78).  0 (default): FP32 FFTs;
 * 1: the three half-sample-shift planes as dense contractions on the tensor
 * cores (tcgen05) with split-BF16 operands (hi*hi + hi*lo + lo*hi, FP32
 * accumulation); 2: the same with single BF16 operands.  Modes 1 and 2 need
 * raw = 2, even chip sides and sides of at most 80 after rounding up to 16
 * (ampcor_setup fails with AMPCOR_ERR_UNSUPPORTED otherwise).  The plain run
 * entry points use it; takes effect at the next ampcor_setup. */
int ampcor_set_precision(ampcor_handle* h, int32_t mode);

/* Oversampled-correlation arithmetic (no counterpart in the reference, which
 * correlates the oversampled chips with FP32 cuFFT transforms,
 * cuAmpcorChunk.cpp:148-157).  0 (default): FP32 direct sums on the FMA
 * pipes; 1: the lag sums as tcgen05 tensor-core contractions with split-BF16
 * operands (hi*hi + hi*lo + lo*hi, FP32 accumulation in tensor memory); 2:
 * the same with single BF16 operands.  Box sums and the normalisation stay
 * exact float sums with the variance subtraction in FP64.  Modes 1 and 2 need
 * a kept surface of at most 16 x 16 lags (2*hz*raw <= 16), oversampled chip
 * rows of whole 16-byte units, and bands of 8 template rows that fit shared
 * memory (oversampled search chips up to about 330 columns, windows up to
 * about 150 wide at raw = 2); ampcor_setup fails with AMPCOR_ERR_UNSUPPORTED
 * otherwise.  Used by the plain runs, the batched chain and the request
 * server; the fused persistent batch shapes do not run it (a batch holding
 * such a job takes the chain shape unless a shape was set, and refuses a
 * fused one with AMPCOR_ERR_UNSUPPORTED; ampcor_batch_tune skips them).
 * Takes effect at the next ampcor_setup. */
int ampcor_set_corr_precision(ampcor_handle* h, int32_t mode);

/* Batched runs (no counterpart in the reference, whose controller runs one
 * image pair per call, cuAmpcorController.cpp:37-178).  A batch holds jobs of
 * any geometry: each job is a handle after ampcor_setup and a start-pixel
 * setter, its device images and its device outputs (same layout as
 * ampcor_run_device).  ampcor_batch_run processes every window of every job
 * in one persistent kernel: CTAs take windows, most expensive first, from a
 * global work queue and run all stages of a window with the intermediates in
 * a per-CTA scratch slot.  flags bit 0 captures the launch in a CUDA graph on
 * the first run and replays it while the job set is unchanged (non-default
 * stream only).  ampcor_batch_tune times the feasible launch shapes (threads
 * per CTA x CTAs per SM x raw-tile placement: ms_out gets
 * AMPCOR_BATCH_TUNE_CANDIDATES times, negative where a shape does not fit) on
 * the current jobs and keeps the fastest; ampcor_batch_config reads the shape
 * back (raw_l2 bit 0: all raw tiles L2-staged; bit 2: chain mode, i.e. four
 * persistent stage kernels per wave of (job, window) items, each at its own
 * launch shape, instead of the fused kernel).  All return status codes; messages via
 * ampcor_batch_last_error. */
#define AMPCOR_BATCH_TUNE_CANDIDATES 6
typedef struct ampcor_batch ampcor_batch;
int ampcor_batch_create(ampcor_batch** out, int32_t deviceID);
int ampcor_batch_destroy(ampcor_batch* b);
int ampcor_batch_clear(ampcor_batch* b);
int ampcor_batch_add(ampcor_batch* b, ampcor_handle* h, const void* ref, int64_t ref_ld, const void* sec,
                     int64_t sec_ld, float* offset, float* snr, float* cov, int32_t* job_index);
int ampcor_batch_run(ampcor_batch* b, void* stream, int32_t flags);
int ampcor_batch_tune(ampcor_batch* b, void* stream, float* ms_out);
/* Waits for the batch's work on `stream`; AMPCOR_ERR_CUDA if a bounded
 * device-side wait of the last run gave up (its results are invalid). */
int ampcor_batch_sync(ampcor_batch* b, void* stream);
/* Selects a launch shape by its index in ampcor_batch_tune's candidate order
 * (a shape that does not fit falls back at the next run). */
int ampcor_batch_set_shape(ampcor_batch* b, int32_t candidate);
/* Stage timing of chain-mode runs (graph replay is off while enabled): per
 * stage (raw correlation, oversampling, oversampled correlation, zoom; nstage
 * >= 4) the summed milliseconds and launches since the last read. */
int ampcor_batch_set_timing(ampcor_batch* b, int32_t enable);
int ampcor_batch_read_timing(ampcor_batch* b, float* ms, int64_t* launches, int32_t nstage);
int ampcor_batch_config(const ampcor_batch* b, int32_t* nt, int32_t* per_sm, int32_t* grid, int64_t* nitems,
                        int32_t* raw_l2);
int ampcor_batch_last_error(const ampcor_batch* b, char* buf, int64_t n);

/* Request server (no counterpart in the reference, whose controller runs one
 * image pair per call, cuAmpcorController.cpp:37-178): continuous batching
 * of offset-tracking requests on one GPU.  ampcor_server_submit queues a
 * request (a handle after ampcor_setup and a start-pixel setter, whose plan
 * and start pixels are copied, plus its two images, host or device pointers
 * that must stay valid until the request has completed, state 2: admission,
 * state 1, only enqueues the copy of the images on the ingest stream, which
 * may still be reading them).  Host images are best in pinned memory: the
 * admission copy is then asynchronous.
 * ampcor_server_progress, called repeatedly from the host loop, never
 * blocks: it retires finished steps, admits queued requests in arrival order
 * while their device memory (images, start pixels, fields) fits the HBM
 * budget (the images are copied into server-owned memory on an ingest
 * stream), and keeps two steps of at most step_windows windows in flight on
 * `stream` (non-default), each mixing windows of every admitted request,
 * oldest first, and run as the batched chain (four stage kernels per wave of
 * windows of one chip geometry).  ampcor_server_poll returns the ids of
 * requests completed since the last poll; ampcor_server_take copies a
 * completed request's fields (ampcor_run_device layout) to host or device
 * memory and frees its device memory.  Times (ampcor_server_request_info:
 * submitted, admitted, completed) are seconds since server creation.
 * A request's results are bit-identical alone and in any mix. */
typedef struct ampcor_server ampcor_server;
#define AMPCOR_SERVER_STATS 8  /* queued, active, steps in flight, bytes used, peak bytes,
                                  steps launched, windows done, peak active requests */
int ampcor_server_create(ampcor_server** out, int32_t deviceID, int64_t hbm_budget_bytes, int32_t step_windows);
int ampcor_server_destroy(ampcor_server* s);
int ampcor_server_submit(ampcor_server* s, ampcor_handle* h, const void* ref, int64_t ref_ld, const void* sec,
                         int64_t sec_ld, int32_t images_on_device, int64_t* request_id);
int ampcor_server_progress(ampcor_server* s, void* stream, int32_t* busy);
int ampcor_server_poll(ampcor_server* s, int64_t* ids, int32_t max_ids, int32_t* n);
int ampcor_server_take(ampcor_server* s, int64_t id, float* offset, float* snr, float* cov, int32_t dst_on_device);
int ampcor_server_request_info(const ampcor_server* s, int64_t id, int32_t* state, int32_t* windows, double* times);
int ampcor_server_stats(const ampcor_server* s, int64_t* out, int32_t n);
int ampcor_server_last_error(const ampcor_server* s, char* buf, int64_t n);

/* ---- Offset-field post-processing (no handle) ----------------------------
 *
 * Outlier culling of an offset field; replaces ISCE2's Offoutliers
 * (components/isceobj/Util/offoutliers: Offoutliers.py:80-92 offoutliers(),
 * the Fortran offoutliers.F:53-127 it calls, and the SNR pre-cull of
 * Offoutliers.py:268-276).  Every array is DEVICE memory of n entries,
 * FP64 like the reference's lists: across / down locations and shifts,
 * `sig` the per-point sigmas (NULL: all 1, as addOffsets sets them), `snr`
 * FP32 SNRs (NULL: no SNR pre-cull).  With `snr`, points whose SNR is below
 * `snr_threshold` are dropped before the fit (OffsetField.cull keeps
 * snr >= threshold).  `distance` is the REAL*4 cull distance.  Outputs
 * (device): index_out (n entries) the 0-based indices of the kept points in
 * input order, count_out their number, average_across / average_down the
 * REAL*4 intercepts of the two fits (getAverageOffsetAcross / Down; may be
 * NULL), fit_out (4 doubles, may be NULL; an addition) the FP64 across
 * intercept, across slope, down intercept, down slope.  Asynchronous on
 * `stream`; AMPCOR_ERR_ARG for n <= 0 (the reference raises on zero-size
 * arrays). */
int ampcor_offoutliers(const double* loc_across, const double* off_across, const double* loc_down,
                       const double* off_down, const double* sig, const float* snr, double snr_threshold,
                       float distance, int64_t n, int32_t* index_out, int32_t* count_out, float* average_across,
                       float* average_down, double* fit_out, void* stream);

/* Offset polynomial; replaces ISCE2's Offsetpoly (stdproc/stdproc/offsetpoly:
 * Offsetpoly.py offsetpoly(), offsetpoly.f90:53-84 with svdfit,
 * resampLib/src/svd.f:1-40, and poly_funcs.f90).  Weighted least-squares fit
 * of `offset` (device, n FP64) as the first `ncoef` (1 .. 10) of 1, x, y,
 * x y, x^2, y^2, x y^2, x^2 y, x^3, y^3 with x = loc_across, y = loc_down
 * (device, FP64), weights 1 / (1 + 1/snr) (snr device FP64), singular values
 * of the design matrix below 1e-12 of the largest dropped (minimum-norm
 * solution).  coef_out (device, ncoef doubles): getOffsetPoly's
 * coefficients; rank_out (device int, may be NULL; an addition): the
 * singular values kept.  Asynchronous on `stream`. */
int ampcor_offsetpoly(const double* loc_across, const double* loc_down, const double* offset, const double* snr,
                      int64_t n, int32_t ncoef, double* coef_out, int32_t* rank_out, void* stream);

/* Nearest-neighbour decimation of a full-resolution raster onto the offset
 * grid; replaces prepareGeometry's gdal.Translate (contrib/PyCuAmpcor/
 * examples/cuDenseOffsets.py:400-460: source window x_start, y_start,
 * cols*xstep x rows*ystep onto cols x rows, nearest sampling, noData 0).
 * dst[i][j] = src[y0 + i*ystep + ystep/2][x0 + j*xstep + xstep/2] (the
 * source pixel under the output pixel's centre), 0 outside the source.  src
 * and dst are device memory, src row-major with leading dimension src_ld
 * elements, dst dense rows x cols; elem_bytes 1, 2, 4 or 8 (any type of that
 * size: the values are copied). */
int ampcor_decimate(const void* src, int64_t src_rows, int64_t src_cols, int64_t src_ld, int32_t elem_bytes,
                    int64_t y0, int64_t x0, int64_t ystep, int64_t xstep, void* dst, int64_t rows, int64_t cols,
                    void* stream);

/* Message of the last failing offset-field call of this host thread. */
int ampcor_field_last_error(char* buf, int64_t n);

/* Message of the last failing call on this handle (empty if none). */
int ampcor_last_error(const ampcor_handle* h, char* buf, int64_t n);

/* Library version string. */
const char* ampcor_version(void);

#ifdef __cplusplus
}
#endif
#endif /* AMPCOR_GB_H */
