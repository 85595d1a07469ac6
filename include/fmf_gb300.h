/*
 * fmf_gb300.h -- C ABI of the GB300 matched-filter library (libfmf_gb300.so).
 *
 * Array conventions are those of the reference library
 * (fast_matched_filter/src/matched_filter_GPU.h:1-4, matched_filter.cu:171-176,
 * argument packing at fast_matched_filter/fast_matched_filter.py:253-316):
 *
 *   templates            (T, S, C, L)  float32, C-contiguous
 *   sum_square_templates (T, S, C)     float32, sum of templates**2 over L.  An
 *                                      extension: fmf_matched_filter[_ex], matched_filter,
 *                                      fmf_batch_add and fmf_matched_filter_detect accept
 *                                      NULL and then compute it on the device,
 *                                      bit-identical to the reference wrapper's
 *                                      numpy.sum(templates**2, axis=-1) on float32 templates
 *   moveouts             (T, S, C)     int32, samples (may be negative)
 *   data                 (S, C, N)     float32
 *   weights              (T, S, C)     float32; weight 0 skips the channel
 *   cc_out               (T, n_corr)          when sum_cc_mode != 0
 *                        (T, n_corr, S, C)    when sum_cc_mode == 0
 *   normalize            0 = "short", 1 = "full" (window mean removed)
 *
 * with n_corr = (N - L) / step + 1.  Output index k of template t is valid
 * when start <= k*step <= N - L - max(0, max moveout of t), start =
 * ceil(-min(0, min moveout of t) / step) * step; every other output element
 * is written as 0.  Every entry point returns an FMF_* status and never
 * terminates the process.  All entry points run on the calling thread's
 * current CUDA device.
 */
#ifndef FMF_GB300_H
#define FMF_GB300_H

#include <stddef.h>

#if defined(__GNUC__)
#define FMF_API __attribute__((visibility("default")))
#else
#define FMF_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define FMF_OK 0
#define FMF_ERR_ARG 1         /* invalid sizes, null pointers, bad option */
#define FMF_ERR_OOM 2         /* device memory allocation failed */
#define FMF_ERR_SMEM 3        /* problem does not fit the kernel's shared memory */
#define FMF_ERR_CUDA 4        /* CUDA runtime / launch error */
#define FMF_ERR_TIMEOUT 5     /* a bounded device-side wait gave up */
#define FMF_ERR_UNSUPPORTED 6 /* option not available in this build/device */

/* numerator precision */
#define FMF_PREC_FP32 0       /* plain FP32 CUDA-core form */
#define FMF_PREC_SPLIT_BF16 1 /* tensor cores, bf16 hi+lo, 3 products, FP32 accumulate */
#define FMF_PREC_BF16 2       /* tensor cores, single bf16 product (loss demonstration) */
/* FMF_PREC_SPLIT_BF16 where an error model of that form puts the search's
 * largest error at or below 1e-5 (of max(1, sum |w|) for network sums), else
 * FMF_PREC_FP32: the model is 4.4e-6 / sqrt(effective taps) per coefficient
 * (x sqrt(1 + L m^2 / V) for 'full', m and V the window mean and centred
 * energy), a 2.8e-6 bias, and the Gaussian maximum over the outputs plus a
 * margin.  The estimate reads the templates, weights and window statistics
 * on the device and waits for its one-word result (the call synchronizes
 * `stream` once).  fmf_last_precision() reports the choice.  Not for
 * batches. */
#define FMF_PREC_AUTO 3

/* flags of fmf_matched_filter_ex */
#define FMF_FLAG_DEVICE_POINTERS 1 /* all array arguments are device pointers */
/* tensor-core tile: lag blocks of 128 outputs per tile (32, 64 or 128; default: largest that fits) */
#define FMF_FLAG_TILE(lag_blocks) ((((lag_blocks) / 16) & 0xff) << 8)
/* tensor-core tile queue: templates interleaved per group of items (1..255; default 16) */
#define FMF_FLAG_TEMPLATE_GROUP(n) (((n) & 0xff) << 16)
/* numerator precision (FMF_PREC_*) of the entry points without a precision
 * argument (fmf_matched_filter_variable_ex); default FMF_PREC_FP32 */
#define FMF_FLAG_PRECISION(p) (((p) & 3) << 24)
#define FMF_FLAG_PRECISION_OF(flags) (((flags) >> 24) & 3)

/*
 * Drop-in for the reference GPU entry point
 *   void matched_filter(float*, float*, int*, float*, float*, size_t step,
 *                       size_t n_samples_template, size_t n_samples_data,
 *                       size_t n_templates, size_t n_stations,
 *                       size_t n_components, size_t n_corr, float* cc_out,
 *                       int normalize, int sum_cc_mode)
 * (fast_matched_filter/src/matched_filter_GPU.h:1-4, matched_filter.cu:171-176).
 * Host pointers; plain FP32 form; synchronous.
 */
FMF_API int fmf_matched_filter(const float *templates, const float *sum_square_templates,
                       const int *moveouts, const float *data, const float *weights,
                       size_t step, size_t n_samples_template, size_t n_samples_data,
                       size_t n_templates, size_t n_stations, size_t n_components,
                       size_t n_corr, float *cc_out, int normalize, int sum_cc_mode);

/*
 * Same symbol name and argument list as the reference GPU library
 * (matched_filter.cu:171-176), so that the reference's ctypes wrapper
 * (fast_matched_filter.py:52-55, 314-316) can load this library in place of
 * matched_filter_GPU.so.  Identical to fmf_matched_filter.
 */
FMF_API int matched_filter(const float *templates, const float *sum_square_templates,
                   const int *moveouts, const float *data, const float *weights,
                   size_t step, size_t n_samples_template, size_t n_samples_data,
                   size_t n_templates, size_t n_stations, size_t n_components,
                   size_t n_corr, float *cc_out, int normalize, int sum_cc_mode);

/*
 * Extended form of fmf_matched_filter (no reference counterpart beyond the
 * arguments above): selects the numerator precision (FMF_PREC_*), accepts
 * device pointers (FMF_FLAG_DEVICE_POINTERS) and runs on `stream`
 * (a cudaStream_t, NULL = legacy default stream).  With device pointers the
 * call is asynchronous with respect to the host; with host pointers it
 * returns after the result has been copied back.
 */
FMF_API int fmf_matched_filter_ex(const float *templates, const float *sum_square_templates,
                          const int *moveouts, const float *data, const float *weights,
                          size_t step, size_t n_samples_template, size_t n_samples_data,
                          size_t n_templates, size_t n_stations, size_t n_components,
                          size_t n_corr, float *cc_out, int normalize, int sum_cc_mode,
                          int precision, int flags, void *stream);

/*
 * fmf_matched_filter_ex plus the reference wrapper's check_zeros count
 * (fast_matched_filter.py:322-361), done on the device before the result is
 * copied out: zero_counts[t] (T values, host or device pointer like the other
 * arrays) = number of outputs of template t equal to 0 whose last-axis index
 * is below zero_stop -- the lag for the network sum, the component for the
 * per-channel layout (the reference slices the last axis in both cases).
 * zero_stop is clamped to [0, last-axis length].  No reference counterpart as
 * an entry point.
 */
FMF_API int fmf_matched_filter_check_zeros(const float *templates, const float *sum_square_templates,
                                           const int *moveouts, const float *data, const float *weights,
                                           size_t step, size_t n_samples_template, size_t n_samples_data,
                                           size_t n_templates, size_t n_stations, size_t n_components,
                                           size_t n_corr, float *cc_out, int normalize, int sum_cc_mode,
                                           int precision, int flags, void *stream, long long zero_stop,
                                           unsigned long long *zero_counts);

/*
 * Allocation-free entry point.  No counterpart in the reference.
 *
 * For callers that cannot allocate device memory while they run -- a
 * real-time detection loop that reserves its memory at start-up and must not
 * call cudaMalloc/cudaFree (which can synchronise the device and take
 * unbounded time) in its processing path, or a host application that owns
 * the GPU's memory budget (a pre-reserved pool, a per-process cap) in which
 * allocations by this library would fail or fragment.
 *
 * Same arguments as fmf_matched_filter plus a stream; every array argument is
 * a 4-byte-aligned device pointer (a misaligned one is rejected with
 * FMF_ERR_ARG); plain FP32 form; asynchronous on `stream`.  As in
 * fmf_matched_filter, sum_square_templates may be NULL and is then computed on
 * the device.  It allocates nothing: its working arrays live in one
 * file-scope device array of FMF_NOALLOC_SCRATCH_BYTES that every GPU loading
 * this library holds until the process exits.  The scratch needed is
 * 4*S*C*N + 8*T bytes for normalize=0 and 12*S*C*N + 4*T*S*C*(L+1) + 4*S*C +
 * 8*T bytes for normalize=1, plus 4*T*S*C when sum_square_templates is NULL
 * (each part rounded up to 256 bytes); larger searches are rejected with
 * FMF_ERR_ARG.  The first call on a device looks up the array's
 * device address with that device current: make it before any stream
 * capture.  All calls share the array, so calls that overlap on the GPU race
 * and must be serialised by the caller.
 */
#define FMF_NOALLOC_SCRATCH_BYTES 33554432u /* 32 MiB */
FMF_API int fmf_matched_filter_noalloc(const float *templates, const float *sum_square_templates,
                                       const int *moveouts, const float *data, const float *weights,
                                       size_t step, size_t n_samples_template, size_t n_samples_data,
                                       size_t n_templates, size_t n_stations, size_t n_components,
                                       size_t n_corr, float *cc_out, int normalize, int sum_cc_mode,
                                       void *stream);

/*
 * Batches of independent searches (no reference counterpart; the reference
 * runs one search per call, matched_filter.cu:171-399).  A batch records
 * searches of any sizes -- device pointers, the same 15 arguments as
 * fmf_matched_filter -- and runs them all as one CUDA graph: the searches'
 * preprocessing, then one persistent tensor-core launch per 64 searches over
 * a shared tile queue (FMF_PREC_SPLIT_BF16 / FMF_PREC_BF16) or the plain kernel
 * per search (FMF_PREC_FP32).  The graph is captured by the first
 * fmf_batch_run after the last fmf_batch_add and replayed by later runs,
 * which read the input buffers anew.  fmf_batch_run is asynchronous on
 * `stream` (NULL = legacy default stream).  A batch belongs to the device
 * that was current at fmf_batch_create.
 */
typedef struct fmf_batch fmf_batch;
FMF_API int fmf_batch_create(fmf_batch **batch, int precision);
FMF_API int fmf_batch_add(fmf_batch *batch, const float *templates, const float *sum_square_templates,
                          const int *moveouts, const float *data, const float *weights, size_t step,
                          size_t n_samples_template, size_t n_samples_data, size_t n_templates,
                          size_t n_stations, size_t n_components, size_t n_corr, float *cc_out,
                          int normalize, int sum_cc_mode);
/* Tensor-core tile shape of the batch: lag blocks per tile (0 = largest that
 * fits every search, else 32/64/128) and templates interleaved per group of
 * tile-queue items (0 = 16). */
FMF_API int fmf_batch_set_tiles(fmf_batch *batch, int lag_blocks, int template_group);
FMF_API int fmf_batch_run(fmf_batch *batch, void *stream);
/* Kernel launches in one run of the batch graph (known after the first run). */
FMF_API int fmf_batch_launch_count(const fmf_batch *batch);
FMF_API int fmf_batch_destroy(fmf_batch *batch);

/*
 * Per-channel template lengths with a Fisher-z network sum: the arguments of
 * the reference's CPU-only matched_filter_variable_precise
 * (fast_matched_filter/src/matched_filter_CPU.h, matched_filter.c:321-325,
 * called from fast_matched_filter.py:307-309), run on the GPU (plain FP32
 * form; the tensor-core form through the flags of the _ex entry point).
 * n_samples_template (T, S, C) gives each channel's length; templates
 * are (T, S, C, max length), zero-padded; cc_sum is (T, n_corr) with
 * n_corr = (N - max length) / step + 1.  Host pointers, synchronous.
 * Semantics, including the reference's template-cumulative scale, are those
 * of matched_filter.c:321-412 (see fmf_variable.cu).
 */
FMF_API int fmf_matched_filter_variable(const float *templates, const float *sum_square_templates,
                                        const int *moveouts, const float *data, const float *weights,
                                        size_t step, const int *n_samples_template,
                                        size_t n_samples_data, size_t n_templates, size_t n_stations,
                                        size_t n_components, size_t n_corr, float *cc_sum,
                                        int normalize);
/* Same, with flags and a stream: FMF_FLAG_DEVICE_POINTERS;
 * FMF_FLAG_PRECISION(FMF_PREC_SPLIT_BF16 or FMF_PREC_BF16) runs the numerators
 * on the tensor cores (each channel's K range cut at its own length),
 * FMF_FLAG_TILE / FMF_FLAG_TEMPLATE_GROUP as for fmf_matched_filter_ex. */
FMF_API int fmf_matched_filter_variable_ex(const float *templates, const float *sum_square_templates,
                                           const int *moveouts, const float *data, const float *weights,
                                           size_t step, const int *n_samples_template,
                                           size_t n_samples_data, size_t n_templates, size_t n_stations,
                                           size_t n_components, size_t n_corr, float *cc_sum,
                                           int normalize, int flags, void *stream);

/*
 * Detection on network-summed cc rows (no reference counterpart: what the
 * reference's callers do next with cc_sum, done on the GPU so the rows need
 * not be copied out).  For each template t, over lags [lag_begin[t],
 * lag_end[t]) of row t of cc (T, n_corr) -- the whole row when both arrays
 * are NULL:
 *   median_out[t]    = numpy.median of the window (float32 arithmetic)
 *   mad_out[t]       = numpy.median of |x - median|
 *   threshold_out[t] = median + n_mad * mad (float32, no fused multiply-add)
 *   peaks            = scipy.signal.find_peaks(window, height=threshold,
 *                      distance=min_separation); equal heights keep the later lag
 *   count_out[t]     = number of peaks, or -1 if more than FMF_DETECT_CAPACITY
 *                      local maxima reach the threshold (no peaks reported)
 *   lag_out / value_out (T, max_detections): the first min(count,
 *                      max_detections) peaks in lag order (absolute lag index).
 * median_out, mad_out, threshold_out may be NULL; lag_out and value_out may be
 * NULL when max_detections is 0.  min_separation >= 1.  Rows must be free of
 * NaN.  Host pointers: synchronous, FMF_ERR_UNSUPPORTED when a row exceeded
 * the capacity.  FMF_FLAG_DEVICE_POINTERS: every array on the device,
 * asynchronous on `stream`; check count_out for -1.  Working memory, from the
 * stream-ordered pool: about 1.5 bytes per lag of the rows detected at once
 * (up to 1,024 rows; lists of median candidates and of values whose MAD class
 * waits for the median), plus about 25 MB.
 */
#define FMF_DETECT_CAPACITY 16384
FMF_API int fmf_detect(const float *cc, size_t n_templates, size_t n_corr, const int *lag_begin,
                       const int *lag_end, float n_mad, size_t min_separation, size_t max_detections,
                       float *median_out, float *mad_out, float *threshold_out, int *count_out,
                       int *lag_out, float *value_out, int flags, void *stream);

/*
 * Search and detection in one call (no reference counterpart): the network-sum
 * search of fmf_matched_filter_ex (arguments as there, sum_cc_mode = 1) into
 * device memory, then fmf_detect over each template's valid lag range (the
 * lags the search can produce: the reference's per-template start/stop,
 * matched_filter.c:53-76).  Only the detections are returned; the (T, n_corr)
 * cc rows never leave the device.  Templates are processed in chunks whose cc
 * rows take at most 16 GiB of device memory (environment variable
 * FMF_SEARCH_DETECT_CHUNK_BYTES overrides the limit).
 */
FMF_API int fmf_matched_filter_detect(const float *templates, const float *sum_square_templates,
                                      const int *moveouts, const float *data, const float *weights,
                                      size_t step, size_t n_samples_template, size_t n_samples_data,
                                      size_t n_templates, size_t n_stations, size_t n_components,
                                      size_t n_corr, int normalize, int precision, float n_mad,
                                      size_t min_separation, size_t max_detections,
                                      float *median_out, float *mad_out, float *threshold_out,
                                      int *count_out, int *lag_out, float *value_out, int flags,
                                      void *stream);

/*
 * Template energies (no reference counterpart; the reference wrapper computes
 * them with numpy, fast_matched_filter.py:256-261): out[r] = sum over L of
 * templates[r][:]**2 for rows r < n_rows, float32 squares summed in numpy's
 * pairwise order, so out is bit-identical to numpy.sum(templates**2, axis=-1)
 * for float32 templates.  Host pointers (synchronous) or, with
 * FMF_FLAG_DEVICE_POINTERS, device pointers (asynchronous on `stream`).
 */
FMF_API int fmf_template_energies(const float *templates, size_t n_rows, size_t n_samples_template,
                                  float *out, int flags, void *stream);

/* Copies the calling thread's last error message (NUL-terminated, truncated
 * to len) and returns its status.  The reference printed and exited instead
 * (matched_filter.cu:30-39, 236-242, 286-299). */
FMF_API int fmf_last_error(char *buf, size_t len);

/* Library version string, e.g. "fmf_gb300 0.1.0 sm_103a". */
FMF_API const char *fmf_version(void);

/* Number of kernel launches issued by this thread's last entry-point call
 * (all kernels of the library; copies and memsets are not counted). */
FMF_API int fmf_last_launch_count(void);

/* Waits for the current device and reports FMF_ERR_TIMEOUT if a kernel of
 * this library gave up a bounded device-side wait since the last check (the
 * host-pointer entry points check this themselves).  No reference
 * counterpart. */
FMF_API int fmf_device_errors(void);

/* Self-test of the bounded device waits (no reference counterpart): runs
 * one CTA that waits on a barrier nothing ever arrives on, with a limit of
 * `ms` milliseconds (1..5000).  Returns FMF_ERR_TIMEOUT when the wait gave up
 * and reported it as the library's kernels do; the device stays usable. */
FMF_API int fmf_selftest_wait_timeout(unsigned ms);

/* Measurement helper (no reference counterpart): the FP32 multiply-add rate
 * of the current device in TFLOP/s (2 flops per FMA), from a kernel of
 * independent FMA chains on every SM, best of three timed runs (about 10 ms
 * in all; synchronizes the device).  The denominator of the plain FP32
 * kernel's roofline. */
FMF_API int fmf_measure_fp32_fma(double *tflops);

/* Accuracy check of the atanh used by the tensor-core form of the per-channel
 * length search (no reference counterpart): out[i] = atanh(y[i]) as that
 * epilogue computes it, for n device floats, asynchronous on `stream`. */
FMF_API int fmf_eval_atanh(const float *y, float *out, size_t n, void *stream);

/* Event timing (no reference counterpart; used by the benchmark).
 * fmf_timing_begin() makes every later call on this thread record CUDA
 * events on its stream around its preprocessing kernels and around its
 * correlation kernel; fmf_timing_end() waits for those events, returns the
 * summed milliseconds of each class and the number of calls, and stops the
 * recording. */
FMF_API int fmf_timing_begin(void);
FMF_API int fmf_timing_end(double *prep_ms, double *kernel_ms, int *n_calls);
/* The same with every class: ms[0] preprocessing, ms[1] correlation kernels,
 * and for host-pointer calls ms[2] the input copies, ms[3] the result's
 * copies from the first start to the last end (they overlap later kernels),
 * ms[4] the part of those copies after the last correlation kernel; the
 * first n_kinds (at most 5) are written. */
FMF_API int fmf_timing_end_ex(double *ms, int n_kinds, int *n_calls);

/* The numerator precision (FMF_PREC_FP32, _SPLIT_BF16 or _BF16) the last
 * search entry point called on this thread used; with FMF_PREC_AUTO, the one
 * it chose.  -1 before the first search. */
FMF_API int fmf_last_precision(void);

/* Releases device memory cached by the library on the current device. */
FMF_API int fmf_release_cache(void);

#ifdef __cplusplus
}
#endif

#endif /* FMF_GB300_H */
