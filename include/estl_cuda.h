/* estl_cuda.h — C ABI of the GB300 FFT engine (libestl_cuda.so).
 *
 * This is the boundary the ESTL plugin layer binds: plain C types, device
 * and host pointers, no exceptions, every call returns an estl_status and
 * estl_last_error() gives the message of the last failure on the calling
 * thread.  The C++ plugin FFT_CUDA<D> (FFT_CUDA.h) is written on top of it.
 *
 * Data layout: interleaved complex64 (re, im as float pairs), transform b of
 * a batch at element offset b*n — the layout FFT_FFTW3 plans on
 * (FFT_FFTW3.h:24-28, SplitInterleavedDataInterface(n*batch, false),
 * DataInterface.h:37-45).  Transforms are unnormalised in both directions
 * (FFTW_FORWARD = exp(-2 pi i jk/n), FFTW_BACKWARD = exp(+2 pi i jk/n)).
 */
#ifndef ESTL_CUDA_H
#define ESTL_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  Replaces the reference's exception paths: CLException via
 * xCLErr (uOpenCL.h:21-55) and the printed-only capacity failure
 * (FFT_OpenCL_Contiguous.h:49). */
typedef enum estl_status {
  ESTL_OK = 0,
  ESTL_INVALID_ARG = 1,
  ESTL_UNSUPPORTED_SIZE = 2,
  ESTL_OUT_OF_MEMORY = 3,
  ESTL_ADMISSION_REJECTED = 4,
  ESTL_DEVICE_ERROR = 5,
  ESTL_TIMEOUT = 6,
  ESTL_NOT_INITIALIZED = 7
} estl_status;

/* Direction, FFTW sign convention (FFT_FFTW3.h:28: forward ? FFTW_FORWARD : FFTW_BACKWARD). */
#define ESTL_FORWARD (-1)
#define ESTL_BACKWARD (+1)

/* Arithmetic of a plan.  FP32 is the plain path. */
#define ESTL_PREC_FP32 0
/* Split precision: every radix-16 DFT stage runs as a
 * tensor-core GEMM (mma.sync m16n8k16, FP32 accumulate) on operands split
 * into 16-bit terms; twiddles and the other passes stay FP32.
 *   FP16:     fp16 hi + lo, each butterfly scaled by a power of two first
 *   BF16:     bf16 hi + lo (about 16 significant bits)
 *   BF16X3:   bf16 hi + mid + lo (FP32-level, six products per stage)
 * n <= 2^13 runs one tile kernel, larger n four-step (n <= 2^24). */
#define ESTL_PREC_SPLIT_FP16 1
#define ESTL_PREC_SPLIT_BF16 2
#define ESTL_PREC_SPLIT_BF16X3 3

typedef struct estl_plan_s* estl_plan;

/* Select the CUDA device, allocate the twiddle bank and set the HBM budget
 * (bytes; 0 = 90% of the memory free at init).  Replaces OpenCLAlgorithm's
 * constructor (uOpenCL.h:284-321: platform/device/context/queue set-up).
 * Idempotent for the same device. */
estl_status estl_init(int device, size_t hbm_budget_bytes);

/* Release every plan and the twiddle bank. */
estl_status estl_shutdown(void);

/* Message of the last failed call on this thread ("" if none). */
const char* estl_last_error(void);

/* Name of a status code. */
const char* estl_status_string(estl_status status);

/* Largest batch of n-point transforms the HBM budget admits for a plan with
 * its own input, output and scratch buffers; clamped to INT32_MAX.
 * Replaces FFT_OpenCL_Contiguous::getMaxBatchSize (FFT_OpenCL_Contiguous.h:43-44),
 * computed in 64 bits instead of the int that overflows above 2 GiB
 * (uOpenCL.h:323-332).  Lengths that are not powers of two (Bluestein plans)
 * first set aside the plan's fixed buffers (chirp, kernel spectrum, work and
 * scratch: at most 8 (n + M) + 1.5 GiB).  Returns 0 before estl_init or for
 * unsupported n. */
int64_t estl_max_batch(int64_t n);

/* Plan `batch` transforms of length n (power of two, 1 <= n <= 2^24).
 * direction: ESTL_FORWARD / ESTL_BACKWARD; precision: ESTL_PREC_FP32 or one of
 * the ESTL_PREC_SPLIT_* tensor-core forms.
 * Replaces the FFT_OpenCL_Contiguous constructor (FFT_OpenCL_Contiguous.h:46-71):
 * radix plan, kernels (precompiled, no runtime compile) and device scratch.
 * Uses an autotuned configuration when the tuning cache holds one for
 * (n, batch). */
estl_status estl_plan_create(int64_t n, int64_t batch, int direction, int precision, estl_plan* plan);

/* Explicit plan shape (what estl_autotune searches).  mode: 0 automatic
 * (tuning cache, else defaults), 1 single kernel (n <= 2^14 in one CTA per
 * transform, or one transform per thread-block cluster up to 2^17, see
 * single_cluster_log2), 2 four-step as a column launch and a row launch per
 * chunk of transforms (two HBM round trips), 4 three-pass (N = R * Q * P,
 * 2^21 <= N <= 2^24, each of R, Q, P in 2^7..2^9): two column launches and a
 * row launch per chunk, three HBM round trips of wide runs instead of two of
 * narrow ones.  Mode 3 is not used.  lag must be 0.
 * chunk (mode 2): transforms per launch pair (0 = default).
 * explicit_tiles != 0 (modes 1 and 2) also fixes the tile kernels, each field
 * -1 for the planner's choice: split_log2 = log2 N2 of N = N1 * N2 (the column
 * DFT length), *_loge = log2 elements per thread, *_logc = log2 transforms
 * (single) or columns / rows (four-step) per CTA, pipelined = 2 for the
 * persistent bulk-load variants (row tiles by bulk copies, column tiles by 2D
 * tensor copies), 3 / 4 for the resident single tiles (whole / half exchange
 * buffer; 2^12..2^14).  Mode 4 reads split_log2 as log2 R and split2_log2 as log2 Q
 * (0 or -1 = default).  *_logr: log2 of the largest radix of the tile
 * (-1 or 4: radix 16; 5: radix-32 passes with 32 elements per thread).  A zero-initialised struct with mode = 0 is the
 * automatic plan. */
typedef struct estl_plan_options {
  int mode;
  int lag;
  int64_t chunk;
  int explicit_tiles;
  int split_log2;
  int single_loge, single_logc;
  int col_loge, col_logc;
  int row_loge, row_logc;
  int pipelined;
  int split2_log2;
  int single_logr, col_logr, row_logr;
  /* single-kernel plans (mode 1): > 0 runs one transform per thread-block
   * cluster of 2^single_cluster_log2 CTAs whose four-step transpose goes
   * through distributed shared memory, with column DFTs of 2^split_log2
   * points (one HBM pass up to 2^17 points); 0 = one CTA per transform,
   * -1 = planner's choice */
  int single_cluster_log2;
} estl_plan_options;

estl_status estl_plan_create_ex(int64_t n, int64_t batch, int direction, int precision,
                                const estl_plan_options* options, estl_plan* plan);

/* 2D transforms: `batch` arrays of ydim rows by xdim columns, row-major (x
 * fastest), the layout of ESTL's FFT2D<D> (FFT.h:54-84), which runs xdim-point
 * FFTs over the rows and then ydim-point FFTs over the columns, in place.
 * Here: one row pass (any 1D plan of xdim, batched over ydim * batch rows)
 * and one column pass in place on the output.  Powers of two, ydim <= 2^12,
 * xdim * ydim <= 2^26, FP32.  Executed with estl_execute / estl_execute_host
 * like a 1D plan of n = xdim * ydim. */
estl_status estl_plan2d_create(int64_t xdim, int64_t ydim, int64_t batch, int direction, int precision,
                               estl_plan* plan);

/* Free the plan and its device buffers (FFT_OpenCL_Contiguous.h:186-191). */
estl_status estl_plan_destroy(estl_plan plan);

/* One-line JSON description of the plan: launches, HBM passes, tile kernels,
 * scratch bytes.  Writes at most len bytes including the terminator. */
estl_status estl_plan_describe(estl_plan plan, char* buf, size_t len);

/* Waits for the device; returns ESTL_TIMEOUT if a bounded device wait of a
 * persistent kernel (a bulk-load or resident tile's copy wait) gave up since
 * the last check (the outputs of that execute are
 * then incomplete), else ESTL_OK.  If a bulk-load kernel also could not drain
 * the copies it had in flight, the plan is marked unusable: this returns
 * ESTL_DEVICE_ERROR and later executes of the plan are refused. */
estl_status estl_plan_check(estl_plan plan);

/* Number of kernel launches (and device copies) one execute issues. */
int64_t estl_plan_launches(estl_plan plan);

/* Device-resident execute, stream ordered (stream: a cudaStream_t, NULL =
 * legacy default stream).  d_in / d_out: n*batch complex64 elements each,
 * 8-byte aligned, out-of-place (d_in is not modified; d_in == d_out is
 * rejected).  Replaces the kernel loop of FFT_OpenCL_Contiguous::execute
 * (FFT_OpenCL_Contiguous.h:107-124) without its host copies; backward
 * transforms are computed for every transform of the batch (the reference
 * conjugates only batch 0, FFT_OpenCL_Contiguous.h:100-102,134-136).
 * Successive executes of a plan that holds device scratch (four-step and
 * three-pass plans, Bluestein, layout staging) are serialised on the device;
 * a one-launch plan (n <= 2^14) has no state and its executes on different
 * streams may overlap.  Use separate plans for concurrent multi-pass work. */
estl_status estl_execute(estl_plan plan, const void* d_in, void* d_out, void* stream);

/* Host-to-host execute with the semantics of FFT<D>::execute (FFT.h:35,
 * FFT_OpenCL_Contiguous.h:97-142): copies h_in to the device, transforms,
 * copies the result to h_out and returns when h_out is complete.  The copy
 * in, the transform and the copy out run pipelined over chunks of the batch
 * on three streams.  h_in/h_out should be pinned (estl_host_register) for
 * full bandwidth; pageable memory works but is slower. */
estl_status estl_execute_host(estl_plan plan, const float* h_in, float* h_out);

/* Other host layouts of the complex data (the reference's DataInterface
 * classes, DataInterface.h:26-45):
 *   ESTL_LAYOUT_INTERLEAVED   re, im pairs (SplitInterleavedDataInterface(n, false));
 *   ESTL_LAYOUT_BLOCK_PLANAR  blocks of 32 real parts then 32 imaginary parts
 *                             (PlannarizedDataInterface, the layout of
 *                             FFT_OpenCL_Contiguous, FFT_OpenCL_Contiguous.h:28);
 *   ESTL_LAYOUT_SPLIT         all real parts, then all imaginary parts
 *                             (SplitInterleavedDataInterface(n, true)).
 * The whole batch (n * batch elements) is one array in the layout; arrays
 * hold estl_layout_floats(layout, n * batch) floats.  The data is converted
 * on the device around the plan's kernels.  estl_execute_layout allocates two
 * interleaved staging buffers of n * batch complex on its first call;
 * estl_execute_host_layout converts per chunk of its host pipeline. */
#define ESTL_LAYOUT_INTERLEAVED 0
#define ESTL_LAYOUT_BLOCK_PLANAR 1
#define ESTL_LAYOUT_SPLIT 2
int64_t estl_layout_floats(int layout, int64_t total);
estl_status estl_execute_layout(estl_plan plan, int layout, const float* d_in, float* d_out, void* stream);
estl_status estl_execute_host_layout(estl_plan plan, int layout, const float* h_in, float* h_out);

/* Per-launch device timing, the counterpart of OpenCLAlgorithm's
 * kernelTimers / timerComputation (uOpenCL.h:281-282) that
 * FFT_OpenCL_Contiguous::execute fills from event profiling
 * (FFT_OpenCL_Contiguous.h:129-131).  While enabled, every launch of an
 * execute is bracketed by CUDA events on the execute's stream; enabling or
 * disabling resets the statistics. */
estl_status estl_plan_set_profiling(estl_plan plan, int enable);

/* Per kernel kind (index 0 single-tile, 1 column pass, 2 row pass, 3 device
 * copy, 4 unused, 5 2D column pass): launches, summed device milliseconds and
 * summed algorithmic bytes (16 bytes per complex element read and written).
 * Waits for the profiled launches to finish.  Arrays have ESTL_KERNEL_KINDS
 * entries; any may be NULL. */
#define ESTL_KERNEL_KINDS 6
estl_status estl_plan_kernel_stats(estl_plan plan, int64_t* launches, double* total_ms, double* bytes);

/* Page-lock / unlock host memory for estl_execute_host. */
estl_status estl_host_register(void* ptr, size_t bytes);
estl_status estl_host_unregister(void* ptr);

/* Time every candidate plan for (n, batch) on the device (iters executes
 * each, after two warm-up executes), store the fastest in the tuning cache
 * ($ESTL_TUNE_CACHE, else ~/.cache/estl_gb300/tune.jsonl) and use it for
 * later estl_plan_create calls with the same n and log2(batch).  Writes a
 * JSON summary to result_json (may be NULL).  The reference has no tuner: its
 * radix is fixed at 16 (FFT_OpenCL_Contiguous.h:55). */
estl_status estl_autotune(int64_t n, int64_t batch, int iters, char* result_json, size_t len);

/* Allocation-free FFT for callers that cannot allocate device memory: plugins
 * whose host owns all device memory through its own allocator or pool,
 * latency-critical loops where cudaMalloc/cudaFree would synchronise the
 * device, and hosts that forbid device allocation in plugin calls.  This
 * entry point has no counterpart in the reference.
 *
 * Runs `batch` transforms of length n with four-step column and row kernels
 * (the plain tiles of estl_execute's tile shapes, which have no device-side
 * waits; estl_execute runs bulk-load variants of them at 2^16..2^22 and is
 * faster there), but keeps their scratch in one fixed device array
 * of 2^22 complex64 (32 MiB) and uses its own 4.4 MB twiddle table; every GPU
 * that loads this library holds both until the process exits.  Needs neither
 * estl_init nor a plan and allocates nothing (no cudaMalloc, cudaFree or
 * allocating library call); the caller passes the input and output buffers
 * (n*batch complex64 each, distinct, 8-byte aligned) and a stream.
 *  - n must be a power of two in [2^14, 2^22]; other sizes are rejected with
 *    ESTL_UNSUPPORTED_SIZE (estl_execute handles them).
 *  - The first call on a device resolves the arrays' device addresses and
 *    fills the twiddle table, synchronising `stream`; make that first call
 *    before any stream capture.  The same set-up runs again on the first call
 *    after the device's context changed (cudaDeviceReset).
 *  - All calls share the array and leave their last contents in it; nothing
 *    in it needs to start at zero.  Calls whose work overlaps on the GPU
 *    (unordered streams, or several threads) race on it: order them. */
estl_status estl_execute_noalloc(int64_t n, int64_t batch, int direction, const void* d_in, void* d_out,
                                 void* stream);

/* ---- FFT convolution (Convolution2D_FFT, Convolution.h:95-154, in 1D) ----
 * Real signal x (length L) with real filter h (length K): both zero-padded to
 * n = nextPow2(L + K - 1) (Convolution.h:89-97), forward FFTs, pointwise
 * product (conj(H) for correlation, :125-137), inverse FFT, scaled by 1/n.
 * Default output: the full linear convolution, L + K - 1 samples.
 * ESTL_CONV_REFERENCE_COMPAT reproduces Convolution.h's normalisation and crop
 * instead: kernel centred by (K + 1)/2 (:113-120), result divided by n * H[0]
 * (:141-143), L samples kept (:146-148).  n may be at most 2^22. */
#define ESTL_CONV_CORRELATE 1
#define ESTL_CONV_REFERENCE_COMPAT 2
/* Real-input specialisation (the default for padded lengths n <= 2^14): two
 * requests of the same n share one complex transform (signals as real and
 * imaginary parts; the two spectra separated with X_{n-k}), so a pair costs
 * one forward and one inverse FFT.  This flag runs every request as its own
 * complex transform instead. */
#define ESTL_CONV_NO_PAIRING 4
/* Real-input specialisation for padded lengths n > 2^14 (the default in
 * FP32): each real request runs as an n/2-point complex transform whose
 * spectrum is split and recombined in the middle kernel, half the bytes of a
 * complex transform.  This flag (which implies ESTL_CONV_NO_PAIRING) runs
 * every request of every length as a full complex transform. */
#define ESTL_CONV_COMPLEX 8
/* Split precision of the convolution's FFT stages (ESTL_PREC_SPLIT_*), or'd
 * into the flags; 0 = FP32. */
#define ESTL_CONV_PRECISION(p) ((p) << 8)

/* One request of a batched convolution.  Offsets are in floats into the
 * caller's packed signal / filter / output arrays. */
typedef struct estl_conv_request {
  int64_t signal_len, filter_len;
  int64_t signal_offset, filter_offset, output_offset;
} estl_conv_request;

/* Output samples of one request: L + K - 1, or L with REFERENCE_COMPAT. */
int64_t estl_conv_output_length(int64_t signal_len, int64_t filter_len, int flags);

/* Device workspace (bytes) estl_conv_execute needs for these requests. */
estl_status estl_conv_workspace_size(const estl_conv_request* reqs, int64_t count, int flags, size_t* bytes);

/* Batched convolution of requests with their own filters and lengths.
 * Requests are grouped by padded length; each group runs a spectrum launch
 * and a fused convolution launch (n <= 2^14), or five four-step launches.
 * Blocking: returns when the outputs are written. */
estl_status estl_conv_execute(const estl_conv_request* reqs, int64_t count, int flags, const float* d_signals,
                              const float* d_filters, float* d_out, void* d_workspace, size_t workspace_bytes,
                              void* stream);

/* A convolution plan: `count` signals of signal_len samples, packed
 * back-to-back, all with one filter whose spectrum is computed once
 * (estl_conv_plan_set_filter) and cached on the device; outputs are packed
 * back-to-back with estl_conv_output_length samples each.  Stream ordered.
 * The executes of one plan share its device scratch: executes on unordered
 * streams race on it, so order them or make one plan per stream. */
typedef struct estl_conv_plan_s* estl_conv_plan;
estl_status estl_conv_plan_create(int64_t signal_len, int64_t filter_len, int64_t count, int flags,
                                  estl_conv_plan* plan);
estl_status estl_conv_plan_set_filter(estl_conv_plan plan, const float* d_filter, void* stream);
estl_status estl_conv_plan_execute(estl_conv_plan plan, const float* d_signals, float* d_out, void* stream);
int64_t estl_conv_plan_launches(estl_conv_plan plan);
estl_status estl_conv_plan_destroy(estl_conv_plan plan);

/* ---- 2D FFT convolution (Convolution2D_FFT::convolve, Convolution.h:95-148) ----
 * `count` real images of height x width floats (row-major, x fastest, packed
 * back-to-back) convolved with one real filter of kheight x kwidth floats:
 * both zero-padded to Pw x Ph = nextPow2(width + kwidth - 1) x
 * nextPow2(height + kheight - 1) (:96-97), 2D FFTs, pointwise product
 * (conj of the filter spectrum with ESTL_CONV_CORRELATE, :125-137), inverse
 * 2D FFT scaled by 1 / (Pw Ph).  Default output: the full linear convolution,
 * (height + kheight - 1) x (width + kwidth - 1) per image.  With
 * ESTL_CONV_REFERENCE_COMPAT the reference's own result: the filter centred
 * by ((kwidth + 1) / 2, (kheight + 1) / 2) cyclically (:113-120), divided by
 * Pw Ph K^[0] (:141-143), height x width kept (:146-148).  FP32; Pw <= 2^14,
 * Ph <= 2^12, Pw Ph <= 2^26.  Three launches per execute (row FFTs of the
 * padded rows, column FFT x spectrum x inverse column FFT, inverse row FFTs
 * with the real crop); the filter spectrum is computed once per
 * estl_conv2d_plan_set_filter.  Stream ordered; the executes of one plan
 * share its device scratch, so executes on unordered streams race on it:
 * order them or make one plan per stream. */
estl_status estl_conv2d_output_size(int64_t width, int64_t height, int64_t kwidth, int64_t kheight, int flags,
                                    int64_t* out_width, int64_t* out_height);
typedef struct estl_conv2d_plan_s* estl_conv2d_plan;
estl_status estl_conv2d_plan_create(int64_t width, int64_t height, int64_t kwidth, int64_t kheight, int64_t count,
                                    int flags, estl_conv2d_plan* plan);
estl_status estl_conv2d_plan_set_filter(estl_conv2d_plan plan, const float* d_filter, void* stream);
estl_status estl_conv2d_plan_execute(estl_conv2d_plan plan, const float* d_images, float* d_out, void* stream);
int64_t estl_conv2d_plan_launches(estl_conv2d_plan plan);
/* One image, host buffers, blocking (the call Convolution2D_FFT::convolve
 * makes): h_image height x width floats, h_kernel kheight x kwidth floats,
 * h_out estl_conv2d_output_size floats.  Device buffers are allocated and
 * freed inside the call. */
estl_status estl_conv2d_host(int64_t width, int64_t height, int64_t kwidth, int64_t kheight, int flags,
                             const float* h_image, const float* h_kernel, float* h_out);
estl_status estl_conv2d_plan_destroy(estl_conv2d_plan plan);

/* ---- Uneven batches: packed transforms of mixed lengths ----
 * count transforms, transform i of length sizes[i] (a power of two in
 * [2, 2^18]) at complex-element offset offsets[i] of both the input and the
 * output buffer (transforms must not overlap).  The reference has one FFT
 * object per size (tests/Test.cpp:45-60) and no uneven batch.
 * ESTL_PACKED_PERSISTENT: one persistent launch; CTAs take work items (whole
 *   small transforms, four-step column and row tiles of large ones) from a
 *   device queue, largest first; a row tile waits (bounded) for its column
 *   tiles.  ESTL_PACKED_PER_SIZE: one launch per size class (two for
 *   four-step classes).  Either way the launch sequence is captured once per
 *   (d_in, d_out) pair in a CUDA graph and replayed. */
#define ESTL_PACKED_PERSISTENT 0
#define ESTL_PACKED_PER_SIZE 1
/* ESTL_PACKED_BUCKETED: one bucket per length, each run by the engine's own
 * plan for (length, count) -- the autotuner's cached choice if there is one,
 * else the planner default: single-CTA, resident or thread-block-cluster tiles
 * in one pass, four-step through a dense per-bucket scratch above -- reading
 * and writing the transforms through their offsets.  The buckets are parallel
 * branches of the captured CUDA graph. */
#define ESTL_PACKED_BUCKETED 2
typedef struct estl_packed_plan_s* estl_packed_plan;
estl_status estl_packed_plan_create(const int64_t* offsets, const int64_t* sizes, int64_t count, int direction,
                                    int mode, estl_packed_plan* plan);
estl_status estl_packed_execute(estl_packed_plan plan, const void* d_in, void* d_out, void* stream);
/* Waits for the device and returns ESTL_TIMEOUT if a dependency wait of the
 * persistent kernel gave up since the last check (its outputs are then
 * incomplete), else ESTL_OK. */
estl_status estl_packed_check(estl_packed_plan plan);
estl_status estl_packed_plan_describe(estl_packed_plan plan, char* buf, size_t len);
/* Test hook for the bounded dependency wait (the reference's error path is
 * xCLErr / CLException, uOpenCL.h:21-55).  skip_column_items != 0 leaves the
 * four-step column items out of later executes, so their row items' waits can
 * never be satisfied; spin_limit (0 = the default of 2^24 polls of 128 ns)
 * bounds those waits.  The wait then runs out on the device without a fault,
 * the row items are skipped, and estl_packed_check returns ESTL_TIMEOUT.
 * skip_column_items = 0, spin_limit = 0 restores normal executes. */
estl_status estl_packed_plan_set_test_hook(estl_packed_plan plan, int skip_column_items, uint64_t spin_limit);
estl_status estl_packed_plan_destroy(estl_packed_plan plan);

/* Mixed uneven batches: the count transforms above (count may be 0) and
 * nconv FFT convolutions (estl_conv_request, offsets in floats into the
 * caller's signal / filter / output arrays; conv_flags: ESTL_CONV_CORRELATE,
 * ESTL_CONV_REFERENCE_COMPAT, ESTL_CONV_NO_PAIRING, ESTL_CONV_COMPLEX; FP32)
 * in one plan, one graph.  The semantics per request are estl_conv_execute's
 * (Convolution.h:95-154 in 1D).
 * ESTL_PACKED_PERSISTENT / PER_SIZE: a convolution of padded length <= 2^12
 *   is a work item of the packed kernel (with the transforms in the one
 *   persistent launch, or one launch per padded length): one CTA computes
 *   the request whole -- signal and filter as the real and imaginary parts of
 *   one complex transform, their spectra separated with X_{n-k}, product,
 *   inverse transform -- reading the signal and the filter once and writing
 *   the output once.  Longer convolutions run the convolution engine's
 *   launches on a branch of the same graph.
 * ESTL_PACKED_BUCKETED: every convolution runs the convolution engine's own
 *   launches (grouped by padded length, two requests per transform, the
 *   real-input four-step above 2^14) on a branch beside the buckets.
 * The plan's graph is captured again when a buffer changes. */
estl_status estl_packed_mixed_plan_create(const int64_t* offsets, const int64_t* sizes, int64_t count, int direction,
                                          const estl_conv_request* reqs, int64_t nconv, int conv_flags, int mode,
                                          estl_packed_plan* plan);
/* d_in / d_out: the transforms' buffers (may be NULL when count is 0);
 * d_signals, d_filters, d_conv_out: the convolutions' float arrays (4-byte
 * aligned), at least the conv_signal_floats / conv_filter_floats /
 * conv_out_floats that estl_packed_plan_describe reports (the largest offset
 * + length over the requests): the call cannot check the size behind a raw
 * pointer.  A plan with convolutions runs only through this call. */
estl_status estl_packed_mixed_execute(estl_packed_plan plan, const void* d_in, void* d_out, const float* d_signals,
                                      const float* d_filters, float* d_conv_out, void* stream);
/* One blocking call for a batch used once: plan (persistent mode), execute on
 * `stream`, wait, check, release. */
estl_status estl_execute_packed(const int64_t* offsets, const int64_t* sizes, int64_t count, int direction,
                                const void* d_in, void* d_out, void* stream);

/* ---- Serving: a request loop with continuous batching ----
 * Requests (1D FFTs and FFT convolutions of mixed lengths, host buffers) are
 * queued by estl_serve_submit and completed by a device-owner thread: when a
 * stream slot is free it admits queued requests in arrival order while their
 * device memory fits the HBM budget, runs them as one batch (inputs in,
 * kernels grouped by size, outputs out, all stream ordered) and keeps up to
 * max_inflight_batches batches overlapping on the device.  A request's host
 * buffers must stay valid until its estl_serve_poll returns.  Each request's
 * result is bit-identical alone and in any batch.
 * max_batch_requests = 1 and max_inflight_batches = 1 give the plain
 * per-request behaviour of the reference (FFT<D>::execute, FFT.h:35, and
 * Convolution2D_FFT::convolve, Convolution.h:95, are blocking calls). */
#define ESTL_REQ_FFT 0
#define ESTL_REQ_CONV 1

typedef struct estl_serve_config {
  size_t hbm_budget_bytes;   /* device bytes in flight (0 = what the engine budget leaves) */
  int max_inflight_batches;  /* stream slots; batches that overlap on the device (0 = 4) */
  int max_batch_requests;    /* requests per batch (0 = 256) */
  int64_t max_queue;         /* queued requests before submit rejects (0 = 2^20) */
} estl_serve_config;

typedef struct estl_serve_request {
  int kind;                  /* ESTL_REQ_FFT or ESTL_REQ_CONV */
  int direction;             /* FFT: ESTL_FORWARD / ESTL_BACKWARD */
  int flags;                 /* CONV: ESTL_CONV_*; both kinds: ESTL_CONV_PRECISION(ESTL_PREC_*) */
  int reserved;
  int64_t n;                 /* FFT: length (power of two <= 2^24) */
  int64_t signal_len;        /* CONV */
  int64_t filter_len;        /* CONV */
  const float* in;           /* FFT: n complex64; CONV: signal_len floats */
  const float* filter;       /* CONV: filter_len floats */
  float* out;                /* FFT: n complex64; CONV: estl_conv_output_length floats */
} estl_serve_request;

typedef struct estl_serve_result {
  estl_status status;
  int batch_requests;        /* size of the batch the request ran in */
  double latency_us;         /* submit -> outputs in the host buffer */
  double queue_us;           /* submit -> admitted */
  double device_us;          /* batch launch -> outputs in the host buffer */
} estl_serve_result;

typedef struct estl_serve_stats {
  int64_t submitted, completed, rejected, batches, max_batch_requests, queued;
  uint64_t inflight_bytes, max_inflight_bytes;
} estl_serve_stats;

typedef struct estl_server_s* estl_server;
estl_status estl_serve_start(const estl_serve_config* cfg, estl_server* server);
/* Queues a request; ESTL_ADMISSION_REJECTED if it can never fit the budget or
 * the queue is full. */
estl_status estl_serve_submit(estl_server server, const estl_serve_request* req, uint64_t* ticket);
/* Waits up to timeout_ms for the request (ESTL_TIMEOUT if not done; the
 * ticket stays valid); on completion fills res and releases the ticket. */
estl_status estl_serve_poll(estl_server server, uint64_t ticket, int timeout_ms, estl_serve_result* res);
estl_status estl_serve_stats_get(estl_server server, estl_serve_stats* stats);
/* Completes every queued and in-flight request, then stops the loop. */
estl_status estl_serve_stop(estl_server server);

/* Bytes currently held by the engine on the device (plans, scratch, staging,
 * twiddle bank) and the budget set at init. */
estl_status estl_memory_usage(size_t* used_bytes, size_t* budget_bytes);

#ifdef __cplusplus
}
#endif

#endif /* ESTL_CUDA_H */
