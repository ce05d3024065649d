/*
 * imagew_gb300.h -- additive C ABI of libimagew_gb300.
 *
 * These entry points have no counterpart in the reference's public header
 * (ImageWorsener 1.3.5 src/imagew.h); they extend the libimagew API without
 * changing any existing declaration.  An application written against
 * imagew.h alone never needs them.
 *
 * Precision forms.  iw_process_image() chooses between
 *   - "fp32" (default): FP32 resampling with a per-sample error bound; every
 *     sample whose bound touches a quantisation decision is recomputed in FP64.
 *     Integer output is identical to the reference's.
 *   - "fp64": the reference's double-precision arithmetic throughout.
 * Select one per context with iw_set_option(ctx, "gpu:precision", "fp64").
 *
 * Vertical pass of the fp32 form.  For 8-bit inputs decoded through a table
 * (no alpha) the vertical pass can run on the tensor cores as exact integer
 * products of 8-bit digits of the fixed-point sample and weight; its error
 * bound is far tighter than an FP32 sum's, so fewer samples are re-evaluated.
 * iw_set_option(ctx, "gpu:vertical", v) with v = "auto" (default: tensor
 * cores for windows of 48 rows or more), "tensor" (whenever eligible) or
 * "cuda" (never).  The output is the same in every case.
 */
#ifndef IMAGEW_GB300_H
#define IMAGEW_GB300_H

#include "imagew.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Statistics of the last iw_process_image() call on a context. */
struct iwg_stats {
	double ms_total;       /* host wall time of iw_process_image */
	double ms_device;      /* GPU time of the pixel passes (input already on the device) */
	double ms_part[4];     /* the same, per launch group: [0] vertical pass,
	                          [1] horizontal pass + quantisation, [2] exact
	                          re-evaluation (fp32 form) or serial dither scan */
	long long flagged;     /* pixels the fp32 form re-evaluated (double-float, then FP64) */
	int form;              /* 0 = fp64, 1 = fp32 + guard band */
	int kernels;           /* kernel launches per pass */
	int zero_copy;         /* 1: kernels read the input and wrote the output in
	                          host memory directly (no staging copies) */
	long long flagged_exact; /* of the flagged pixels, those the double-float
	                          tier could not decide and FP64 recomputed */
	int vertical_tensor;   /* 1: the vertical pass ran on the tensor cores
	                          (exact integer digit products; see the
	                          "gpu:vertical" option) */
	int graph;             /* 1: iwg_process_image_timed replayed the passes
	                          as a CUDA graph (ms_device is then the mean time
	                          of one replay) */
	int fused;             /* 1: the fp32 form ran its vertical and
	                          horizontal passes as one fused launch (no
	                          intermediate image in device memory; see the
	                          "gpu:fuse" option) */
	double ms_phase[6];    /* iw_process_image() by phase, ms: [0] planning
	                          (host), [1] input upload, [2] device passes,
	                          [3] output download (these three by CUDA events
	                          on the library's stream), [4] output post-pass
	                          (host), [5] the device part's host wall time
	                          (tables, launches, waits; contains 1-3) */
};

/* Copies the statistics of the context's last run into *out.  Returns 1. */
IW_EXPORT(int) iwg_get_stats(struct iw_context *ctx, struct iwg_stats *out);

/* Like iw_process_image(), but runs the device passes warmup + iters times
 * back to back with the input resident in device memory, and reports in
 * iwg_stats the mean GPU time of the last 'iters' runs (CUDA events on the
 * library's stream).  The output image is that of the final run, identical to
 * what iw_process_image() returns.  Meant for benchmarking the pixel passes
 * apart from host<->device transfers.  Returns 1 on success. */
IW_EXPORT(int) iwg_process_image_timed(struct iw_context *ctx, int warmup, int iters);

/* Debug readback for measuring the FP32 form's error against the FP64 form.
 * No counterpart in the reference.  After iw_process_image() on a context
 * with the option "gpu:debug_values" set to "1" (integer output), copies one
 * array of the run into out (at most max_count doubles) and its three
 * dimensions into dims (if not NULL):
 *   which 0: the intermediate image after the vertical pass, one plane per
 *            intermediate channel (alpha in its own plane), [n][rows][cols];
 *   which 1: per output sample, the linear-light value the quantisation
 *            starts from (after unassociating alpha), [channel][row][col];
 *   which 2: the FP32 form's rigorous bound on that value's distance from
 *            the FP64 form's (0 in the FP64 form).
 * NaN marks a sample the tail decided without a value (a blackened colour
 * sample, an undecidable alpha).  Returns the array's length (also with
 * out == NULL), or -1 for an unknown 'which'. */
IW_EXPORT(long long) iwg_debug_values(struct iw_context *ctx, int which, double *out, long long max_count, int *dims);

/* Writes a one-line description of the CUDA device the library uses into
 * buf (NUL-terminated, at most buflen bytes).  Returns 0 if no device. */
IW_EXPORT(int) iwg_device_info(char *buf, int buflen);

/* Host time of iwg_process_batch() calls, process-wide sums in ms: [0]
 * planning (on all host threads, wall time), [1] the fast-form batches, [2]
 * the plain-form batches, [3] the output post-pass (all host threads, wall),
 * [4..13] the batched calls' phases as in iwg_server_info.batch_phase_ms.
 * Writes at most n values; returns how many. */
IW_EXPORT(int) iwg_batch_phase_ms(double *out, int n);

/* Processes n contexts as one batch.  Each context must be set up as for
 * iw_process_image() and not yet processed; afterwards each holds exactly the
 * output iw_process_image() would have given it alone (and counts as
 * processed).  The images the FP32 form takes run together, one kernel launch
 * per kernel variant and pass for the whole batch, in chunks of at most 8 GiB
 * of device memory; the others run one after another.  Planning and the
 * output post-pass run on several host threads, so warning callbacks may be
 * called from them.  Returns the number of contexts processed successfully; a
 * context that failed has its error set as with iw_process_image().
 * iwg_get_stats() of a context processed with the others reports the whole
 * call's wall time (ms_total) and the device time of all its batched passes
 * (ms_device). */
IW_EXPORT(int) iwg_process_batch(struct iw_context **ctxs, int n);

/* ---- request server: continuous batching under a device-memory budget ----
 * A server owns host threads that plan submitted contexts as they arrive, a
 * dispatcher that runs every planned request fitting the budget as one batch
 * (as iwg_process_batch) while the next requests are being planned, scan
 * workers that run requests ending in a serial dither scan (error diffusion,
 * random dither) on device lanes of their own -- a large one alone, small ones
 * together -- and threads that run the output post-pass.  Each request's output is exactly
 * what iw_process_image() gives it alone.  The caller keeps ownership of the
 * contexts: a context may be read or destroyed once its completion was polled. */
struct iwg_server;
struct iwg_completion {
	unsigned long long tag;  /* as given to iwg_server_submit */
	int ok;                  /* 1: processed; 0: failed (error set on the context) */
	double latency_ms;       /* submit -> completion */
	double planned_ms;       /* submit -> planning done */
	double started_ms;       /* submit -> its device work began (0 if it never ran) */
	double ran_ms;           /* submit -> its device work ended (the rest is the post-pass) */
};
struct iwg_server_stats {
	int in_flight;               /* submitted, completion not yet polled */
	int queued;                  /* waiting for planning or for the GPU */
	long long batches;           /* device batches run */
	long long batched_requests;  /* requests in them */
	double device_ms;            /* device time of the batched passes */
	long long slow_batches;      /* of them on the scan workers' lanes (serial dither scans) */
	long long slow_requests;
	double slow_device_ms;
	double batch_wall_ms;        /* host wall time of the dispatcher's batched calls */
	double rest_wall_ms;         /* ... and of the requests they left to the plain form */
	double plan_ms;              /* planning time, summed over requests */
	double batch_phase_ms[10];   /* batched calls' host time (process-wide sums): preparation,
	                                uploads, the passes' launches, the fix-up's launch, device
	                                wait with downloads, the rest; within the passes' launches,
	                                the table upload and the kernel attribute calls; within the
	                                staged downloads, the device wait and the host copies */
};
/* device_budget: bytes of device memory one batch may hold (0: 8 GiB);
 * max_batch: requests per batch (0: 4096); host_threads (0: all cores). */
IW_EXPORT(struct iwg_server *) iwg_server_create(size_t device_budget, int max_batch, int host_threads);
/* Queues a configured, unprocessed context.  Returns 1, or 0 if refused. */
IW_EXPORT(int) iwg_server_submit(struct iwg_server *s, struct iw_context *ctx, unsigned long long tag);
/* Moves up to max completions into out; waits up to wait_ms for the first
 * (0: no wait, negative: until one completes).  Returns the number moved. */
IW_EXPORT(int) iwg_server_poll(struct iwg_server *s, struct iwg_completion *out, int max, int wait_ms);
IW_EXPORT(int) iwg_server_info(struct iwg_server *s, struct iwg_server_stats *out);
/* Finishes every submitted request, then stops the server's threads. */
IW_EXPORT(void) iwg_server_destroy(struct iwg_server *s);

/* Resamples one 8-bit image without allocating any memory, host or device.
 * No counterpart in the reference: it is the iw_process_image() pixel path
 * (reference arithmetic, FP64 form, bit-identical output) narrowed to what a
 * caller that cannot allocate needs:
 *   - imgtype IW_IMGTYPE_GRAY, _GRAYA, _RGB or _RGBA, 8 bits per sample, the
 *     same type in and out; alpha is premultiplied for resampling and colour
 *     samples of fully transparent output pixels are set to 0, as
 *     iw_process_image() does for an output profile that keeps transparency
 *     (a gray image comes out as iw_process_image() returns it once its
 *     output post-pass has packed the three equal channels back to gray);
 *   - one resize algorithm for both dimensions (IW_RESIZETYPE_*, with
 *     param1/param2 as in iw_set_resize_alg(), blur 1, standard edges);
 *   - one colour space (IW_CSTYPE_*, gamma for IW_CSTYPE_GAMMA) for input and
 *     output; no dithering, background, crop, offsets or posterisation.
 * src and dst must be readable / writable by kernels on the current device:
 * device or managed memory, mapped pinned memory, or ordinary host memory on a
 * device with pageable memory access.  The work is queued on 'stream' (a
 * cudaStream_t; NULL for the default stream) and the call returns without
 * waiting; dst is complete when the stream is.
 * Limits: dimensions 1..16384; weight lists of both dimensions within a 4 MiB
 * staging area; tables + weight lists + the float intermediate image
 * (4 * channels * dst_h * src_w bytes) within a 32 MiB device scratch array.
 * A job beyond a limit is rejected with a message and nothing is launched.
 * All calls share that scratch array and staging area: calls must be ordered
 * (one stream, or synchronised between streams); overlapping calls on
 * unsynchronised streams race.  The first call on each device resolves the
 * scratch array's address (which may load the library's module on that
 * device).  That address is kept for the life of the process: after
 * cudaDeviceReset() on a device, this entry point must not be called on that
 * device again in the same process.
 * Returns 1 on success; 0 on error, with a message in errmsg (at most
 * errmsg_len bytes, NUL-terminated) when errmsg is not NULL. */
IW_EXPORT(int) iwg_resize_u8_noalloc(const unsigned char *src, int src_w, int src_h, long long src_bpr,
	unsigned char *dst, int dst_w, int dst_h, long long dst_bpr, int imgtype, int resize_type,
	double param1, double param2, int cstype, double gamma, void *stream, char *errmsg, int errmsg_len);

#ifdef __cplusplus
}
#endif

#endif /* IMAGEW_GB300_H */
