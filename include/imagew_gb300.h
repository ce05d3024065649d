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
	long long flagged;     /* pixels recomputed in FP64 by the fp32 form */
	int form;              /* 0 = fp64, 1 = fp32 + guard band */
	int kernels;           /* kernel launches per pass */
	int zero_copy;         /* 1: kernels read the input and wrote the output in
	                          host memory directly (no staging copies) */
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

/* Writes a one-line description of the CUDA device the library uses into
 * buf (NUL-terminated, at most buflen bytes).  Returns 0 if no device. */
IW_EXPORT(int) iwg_device_info(char *buf, int buflen);

#ifdef __cplusplus
}
#endif

#endif /* IMAGEW_GB300_H */
