// api.cpp -- the libimagew context and settings API of libimagew_gb300.
//
// Semantics follow src/imagew-api.c and src/imagew-util.c of ImageWorsener
// 1.3.5 (cited per function); iw_process_image() hands the pixel work to the
// GPU pipeline (pipeline.cu) after host planning (plan.cpp).
#include "iwg_internal.h"

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <strings.h>
#include <algorithm>
#include <atomic>
#include <chrono>
#include <mutex>
#include <ctime>
#include <thread>
#include <vector>

using iwg::kMsgMax;

// ===== allocation (src/imagew-util.c:24-137) ===============================

static void *default_malloc(void *, unsigned int flags, size_t n)
{
	return (flags & IW_MALLOCFLAG_ZEROMEM) ? calloc(n, 1) : malloc(n);
}
static void default_free(void *, void *m) { free(m); }

extern "C" {

void *iw_malloc_ex(struct iw_context *ctx, unsigned int flags, size_t n)
{
	void *m = nullptr;
	if(n <= ctx->max_malloc) m = ctx->mallocfn(ctx->userdata, flags, n);
	if(!m && !(flags & IW_MALLOCFLAG_NOERRORS)) iw_set_error(ctx, "Out of memory");
	return m;
}
void *iw_malloc(struct iw_context *ctx, size_t n) { return iw_malloc_ex(ctx, 0, n); }
void *iw_mallocz(struct iw_context *ctx, size_t n) { return iw_malloc_ex(ctx, IW_MALLOCFLAG_ZEROMEM, n); }

void *iw_malloc_large(struct iw_context *ctx, size_t n1, size_t n2)
{
	if(n2 && n1 > ctx->max_malloc / n2) {
		iw_set_error(ctx, "Image too large to process");
		return nullptr;
	}
	return iw_malloc_ex(ctx, 0, n1 * n2);
}

void *iw_realloc_ex(struct iw_context *ctx, unsigned int flags, void *old, size_t oldn, size_t n)
{
	if(!old) return iw_malloc_ex(ctx, flags, n);
	if(n > ctx->max_malloc) {
		if(!(flags & IW_MALLOCFLAG_NOERRORS)) iw_set_error(ctx, "Out of memory");
		return nullptr;
	}
	void *m = ctx->mallocfn(ctx->userdata, flags, n);   // always a new block
	if(m) memcpy(m, old, oldn < n ? oldn : n);
	ctx->freefn(ctx->userdata, old);                      // old block freed even on failure
	if(!m && !(flags & IW_MALLOCFLAG_NOERRORS)) iw_set_error(ctx, "Out of memory");
	return m;
}
void *iw_realloc(struct iw_context *ctx, void *m, size_t oldn, size_t n) { return iw_realloc_ex(ctx, 0, m, oldn, n); }

void iw_free(struct iw_context *ctx, void *m)
{
	if(m) ctx->freefn(ctx->userdata, m);
}

char *iw_strdup(struct iw_context *ctx, const char *s)
{
	if(!s) return nullptr;
	size_t n = strlen(s) + 1;
	char *d = (char *)iw_malloc(ctx, n);
	if(d) memcpy(d, s, n);
	return d;
}

// ===== strings, messages, errors (src/imagew-api.c:15-162) ================

void iw_strlcpy(char *dst, const char *src, size_t dstlen)
{
	size_t n = strlen(src);
	if(n > dstlen - 1) n = dstlen - 1;
	memcpy(dst, src, n);
	dst[n] = '\0';
}

void iw_vsnprintf(char *buf, size_t buflen, const char *fmt, va_list ap)
{
	vsnprintf(buf, buflen, fmt, ap);
	buf[buflen - 1] = '\0';
}

void iw_snprintf(char *buf, size_t buflen, const char *fmt, ...)
{
	va_list ap;
	va_start(ap, fmt);
	iw_vsnprintf(buf, buflen, fmt, ap);
	va_end(ap);
}

int iw_stricmp(const char *a, const char *b) { return strcasecmp(a, b); }
void iw_zeromem(void *m, size_t n) { memset(m, 0, n); }

void iw_translate(struct iw_context *ctx, unsigned int flags, char *dst, size_t dstlen, const char *src)
{
	dst[0] = '\0';
	if(ctx && ctx->xlate && ctx->xlate(ctx, flags, dst, dstlen, src)) return;
	iw_strlcpy(dst, src, dstlen);
}

void iw_translatev(struct iw_context *ctx, unsigned int flags, char *dst, size_t dstlen, const char *fmt, va_list ap)
{
	if(!ctx || !ctx->xlate) {
		iw_vsnprintf(dst, dstlen, fmt, ap);
		return;
	}
	char a[kMsgMax], b[kMsgMax];
	iw_translate(ctx, IW_TRANSLATEFLAG_FORMAT | flags, a, sizeof(a), fmt);
	iw_vsnprintf(b, sizeof(b), a, ap);
	iw_translate(ctx, IW_TRANSLATEFLAG_POSTFORMAT | flags, dst, dstlen, b);
}

void iw_translatef(struct iw_context *ctx, unsigned int flags, char *dst, size_t dstlen, const char *fmt, ...)
{
	va_list ap;
	va_start(ap, fmt);
	iw_translatev(ctx, flags, dst, dstlen, fmt, ap);
	va_end(ap);
}

static void record_error(struct iw_context *ctx, const char *msg)
{
	if(ctx->error_flag) return;   // only the first error is kept
	ctx->error_flag = 1;
	if(!ctx->error_msg) {
		ctx->error_msg = (char *)iw_malloc_ex(ctx, IW_MALLOCFLAG_NOERRORS, kMsgMax);
		if(!ctx->error_msg) return;
	}
	iw_strlcpy(ctx->error_msg, msg, kMsgMax);
}

void iw_set_error(struct iw_context *ctx, const char *s)
{
	if(ctx->error_flag) return;
	char buf[kMsgMax];
	iw_translate(ctx, IW_TRANSLATEFLAG_ERRORMSG, buf, sizeof(buf), s);
	record_error(ctx, buf);
}

void iw_set_errorv(struct iw_context *ctx, const char *fmt, va_list ap)
{
	if(ctx->error_flag) return;
	char buf[kMsgMax];
	iw_translatev(ctx, IW_TRANSLATEFLAG_ERRORMSG, buf, sizeof(buf), fmt, ap);
	record_error(ctx, buf);
}

void iw_set_errorf(struct iw_context *ctx, const char *fmt, ...)
{
	va_list ap;
	va_start(ap, fmt);
	iw_set_errorv(ctx, fmt, ap);
	va_end(ap);
}

void iw_warning(struct iw_context *ctx, const char *s)
{
	if(!ctx->warn) return;
	char buf[kMsgMax];
	iw_translate(ctx, IW_TRANSLATEFLAG_WARNINGMSG, buf, sizeof(buf), s);
	ctx->warn(ctx, buf);
}

void iw_warningv(struct iw_context *ctx, const char *fmt, va_list ap)
{
	if(!ctx->warn) return;
	char buf[kMsgMax];
	iw_translatev(ctx, IW_TRANSLATEFLAG_WARNINGMSG, buf, sizeof(buf), fmt, ap);
	ctx->warn(ctx, buf);
}

void iw_warningf(struct iw_context *ctx, const char *fmt, ...)
{
	if(!ctx->warn) return;
	va_list ap;
	va_start(ap, fmt);
	iw_warningv(ctx, fmt, ap);
	va_end(ap);
}

const char *iw_get_errormsg(struct iw_context *ctx, char *buf, int buflen)
{
	if(ctx->error_msg) iw_strlcpy(buf, ctx->error_msg, buflen);
	else iw_translate(ctx, IW_TRANSLATEFLAG_ERRORMSG, buf, buflen, "Error message not available");
	return buf;
}

int iw_get_errorflag(struct iw_context *ctx) { return ctx->error_flag; }

// ===== small helpers (src/imagew-api.c:164-196) ============================

int iw_imgtype_num_channels(int t)
{
	switch(t) {
	case IW_IMGTYPE_RGBA: return 4;
	case IW_IMGTYPE_RGB: return 3;
	case IW_IMGTYPE_GRAYA: return 2;
	}
	return 1;
}

size_t iw_calc_bytesperrow(int num_pixels, int bits_per_pixel)
{
	return (size_t)(((num_pixels * bits_per_pixel) + 7) / 8);
}

int iw_check_image_dimensions(struct iw_context *ctx, int w, int h)
{
	if(w > ctx->max_w || h > ctx->max_h) {
		iw_set_errorf(ctx, "Image dimensions too large (%d\xc3\x97%d)", w, h);
		return 0;
	}
	if(w < 1 || h < 1) {
		iw_set_errorf(ctx, "Invalid image dimensions (%d\xc3\x97%d)", w, h);
		return 0;
	}
	return 1;
}

int iw_is_valid_density(double dx, double dy, int code)
{
	if(dx < 0.0001 || dy < 0.0001) return 0;
	if(dx > 10000000.0 || dy > 10000000.0) return 0;
	if(dx / 10.0 > dy || dy / 10.0 > dx) return 0;
	return code == IW_DENSITY_UNITS_UNKNOWN || code == IW_DENSITY_UNITS_PER_METER;
}

// ===== context (src/imagew-api.c:198-289) ==================================

struct iw_context *iw_create_context(struct iw_init_params *params)
{
	bool custom = params && params->mallocfn;
	void *mem = custom ? params->mallocfn(params->userdata, IW_MALLOCFLAG_ZEROMEM, sizeof(iw_context))
	                   : default_malloc(nullptr, IW_MALLOCFLAG_ZEROMEM, sizeof(iw_context));
	if(!mem) return nullptr;
	iw_context *ctx = new(mem) iw_context();
	if(params) {
		ctx->userdata = params->userdata;
		ctx->api_version = params->api_version;
	}
	ctx->mallocfn = custom ? params->mallocfn : default_malloc;
	ctx->freefn = custom ? params->freefn : default_free;
	iw_make_srgb_csdescr_2(&ctx->cs_in);
	iw_make_srgb_csdescr_2(&ctx->cs_out);
	return ctx;
}

void iw_destroy_context(struct iw_context *ctx)
{
	if(!ctx) return;
	if(ctx->opts) {
		for(int i = 0; i <= ctx->nopts && i < 32; i++) {
			iw_free(ctx, ctx->opts[i].name);
			iw_free(ctx, ctx->opts[i].val);
		}
		iw_free(ctx, ctx->opts);
	}
	iw_free(ctx, ctx->img1.pixels);
	iw_free(ctx, ctx->img2.pixels);
	iw_free(ctx, ctx->error_msg);
	iw_free(ctx, ctx->opt.tmp);
	iw_free(ctx, ctx->opt.pal);
	iw_freefn_type freefn = ctx->freefn;
	void *ud = ctx->userdata;
	ctx->~iw_context();
	freefn(ud, ctx);
}

void iw_set_userdata(struct iw_context *ctx, void *u) { ctx->userdata = u; }
void *iw_get_userdata(struct iw_context *ctx) { return ctx->userdata; }
void iw_set_translate_fn(struct iw_context *ctx, iw_translatefn_type f) { ctx->xlate = f; }
void iw_set_warning_fn(struct iw_context *ctx, iw_warningfn_type f) { ctx->warn = f; }
void iw_set_max_malloc(struct iw_context *ctx, size_t n) { ctx->max_malloc = n; }

// Takes ownership of img->pixels (freed with the context's free function).
void iw_set_input_image(struct iw_context *ctx, const struct iw_image *img) { ctx->img1 = *img; }

void iw_set_output_canvas_size(struct iw_context *ctx, int w, int h)
{
	ctx->canvas_w = w;
	ctx->canvas_h = h;
}

void iw_set_output_image_size(struct iw_context *ctx, double w, double h)
{
	ctx->true_w = w < 0.01 ? 0.01 : w;
	ctx->true_h = h < 0.01 ? 0.01 : h;
	ctx->true_valid = 1;
}

void iw_set_input_crop(struct iw_context *ctx, int x, int y, int w, int h)
{
	ctx->crop_x = x; ctx->crop_y = y; ctx->crop_w = w; ctx->crop_h = h;
}

void iw_set_output_profile(struct iw_context *ctx, unsigned int n) { ctx->profile = n; }
void iw_set_output_depth(struct iw_context *ctx, int bps) { ctx->req_depth = bps; }

void iw_set_output_max_color_code(struct iw_context *ctx, int ct, int n)
{
	if(ct >= 0 && ct < iwg::kNCTypes) ctx->req_maxcc[ct] = n;
}

// Per-channel-type setting with the ALL / NONALPHA group codes
// (src/imagew-api.c:391-433).
static void set_by_ctype(int *arr, int ct, int v)
{
	if(ct >= 0 && ct < iwg::kNCTypes) arr[ct] = v;
	if(ct == IW_CHANNELTYPE_ALL) arr[IW_CHANNELTYPE_ALPHA] = v;
	if(ct == IW_CHANNELTYPE_ALL || ct == IW_CHANNELTYPE_NONALPHA) {
		arr[IW_CHANNELTYPE_RED] = arr[IW_CHANNELTYPE_GREEN] = v;
		arr[IW_CHANNELTYPE_BLUE] = arr[IW_CHANNELTYPE_GRAY] = v;
	}
}

void iw_set_dither_type(struct iw_context *ctx, int ct, int f, int s)
{
	set_by_ctype(ctx->dfam, ct, f);
	set_by_ctype(ctx->dsub, ct, s);
}

void iw_set_color_count(struct iw_context *ctx, int ct, int c) { set_by_ctype(ctx->req_cc, ct, c); }

void iw_set_channel_offset(struct iw_context *ctx, int ct, int dimension, double offs)
{
	if(ct < 0 || ct > 2) return;
	if(dimension < 0 || dimension > 1) dimension = 0;
	ctx->dim[dimension].chan_offset[ct] = offs;
}

void iw_set_input_max_color_code(struct iw_context *ctx, int ch, int c)
{
	if(ch >= 0 && ch < iwg::kMaxCh) ctx->in_maxcc[ch] = c;
}

void iw_set_input_bkgd_label_2(struct iw_context *ctx, const struct iw_color *clr)
{
	ctx->inlabel_set = 1;
	ctx->inlabel = *clr;
}

void iw_set_input_bkgd_label(struct iw_context *ctx, double r, double g, double b)
{
	struct iw_color c = {{r, g, b, 1.0}};
	iw_set_input_bkgd_label_2(ctx, &c);
}

void iw_set_output_bkgd_label_2(struct iw_context *ctx, const struct iw_color *clr)
{
	ctx->outlabel_valid = 1;
	ctx->outlabel = *clr;
}

void iw_set_output_bkgd_label(struct iw_context *ctx, double r, double g, double b)
{
	struct iw_color c = {{r, g, b, 1.0}};
	iw_set_output_bkgd_label_2(ctx, &c);
}

void iw_set_apply_bkgd_2(struct iw_context *ctx, const struct iw_color *clr)
{
	ctx->bkgd_valid = 1;
	ctx->bkgd = *clr;
}

void iw_set_apply_bkgd(struct iw_context *ctx, double r, double g, double b)
{
	struct iw_color c = {{r, g, b, 1.0}};
	iw_set_apply_bkgd_2(ctx, &c);
}

void iw_set_bkgd_checkerboard_2(struct iw_context *ctx, int sz, const struct iw_color *clr)
{
	ctx->bkgd_checker = 1;
	ctx->check_size = sz;
	ctx->bkgd2 = *clr;
}

void iw_set_bkgd_checkerboard(struct iw_context *ctx, int sz, double r, double g, double b)
{
	struct iw_color c = {{r, g, b, 1.0}};
	iw_set_bkgd_checkerboard_2(ctx, sz, &c);
}

void iw_set_bkgd_checkerboard_origin(struct iw_context *ctx, int x, int y)
{
	ctx->check_origin[0] = x;
	ctx->check_origin[1] = y;
}

int iw_get_input_density(struct iw_context *ctx, double *px, double *py, int *pcode)
{
	*px = 1.0; *py = 1.0; *pcode = IW_DENSITY_UNKNOWN;
	if(ctx->img1.density_code == IW_DENSITY_UNKNOWN) return 0;
	if(!iw_is_valid_density(ctx->img1.density_x, ctx->img1.density_y, ctx->img1.density_code)) return 0;
	*px = ctx->img1.density_x; *py = ctx->img1.density_y; *pcode = ctx->img1.density_code;
	return 1;
}

void iw_set_output_density(struct iw_context *ctx, double x, double y, int code)
{
	ctx->img2.density_code = code;
	ctx->img2.density_x = x;
	ctx->img2.density_y = y;
}

// A "gamma" within 5e-6 of 1 is linear (src/imagew-api.c:513-520).
static void fix_gamma(struct iw_csdescr *cs)
{
	if(cs->cstype == IW_CSTYPE_GAMMA && cs->gamma >= 0.999995 && cs->gamma <= 1.000005) cs->cstype = IW_CSTYPE_LINEAR;
}

void iw_make_linear_csdescr(struct iw_csdescr *cs) { cs->cstype = IW_CSTYPE_LINEAR; cs->gamma = 0.0; cs->srgb_intent = 0; }
void iw_make_srgb_csdescr(struct iw_csdescr *cs, int intent) { cs->cstype = IW_CSTYPE_SRGB; cs->gamma = 0.0; cs->srgb_intent = intent; }
void iw_make_srgb_csdescr_2(struct iw_csdescr *cs) { cs->cstype = IW_CSTYPE_SRGB; cs->gamma = 0.0; }
void iw_make_rec709_csdescr(struct iw_csdescr *cs) { cs->cstype = IW_CSTYPE_REC709; cs->gamma = 0.0; }

void iw_make_gamma_csdescr(struct iw_csdescr *cs, double gamma)
{
	cs->cstype = IW_CSTYPE_GAMMA;
	cs->gamma = gamma < 0.1 ? 0.1 : (gamma > 10.0 ? 10.0 : gamma);
	cs->srgb_intent = 0;
	fix_gamma(cs);
}

void iw_set_output_colorspace(struct iw_context *ctx, const struct iw_csdescr *cs)
{
	ctx->cs_out_req = *cs;
	fix_gamma(&ctx->cs_out_req);
	ctx->cs_out_valid = 1;
}

void iw_set_input_colorspace(struct iw_context *ctx, const struct iw_csdescr *cs)
{
	ctx->cs_in = *cs;
	fix_gamma(&ctx->cs_in);
}

void iw_get_output_colorspace(struct iw_context *ctx, struct iw_csdescr *cs) { *cs = ctx->cs_out; }
const struct iw_palette *iw_get_output_palette(struct iw_context *ctx) { return ctx->opt.pal; }

void iw_set_random_seed(struct iw_context *ctx, int randomize, int seed)
{
	ctx->randomize = randomize;
	ctx->seed = seed;
}

void iw_set_allow_opt(struct iw_context *ctx, int opt, int n)
{
	iw_byte v = n ? 1 : 0;
	switch(opt) {
	case IW_OPT_GRAYSCALE: ctx->opt_gray = v; break;
	case IW_OPT_PALETTE: ctx->opt_pal = v; break;
	case IW_OPT_16_TO_8: ctx->opt_16to8 = v; break;
	case IW_OPT_STRIP_ALPHA: ctx->opt_strip = v; break;
	case IW_OPT_BINARY_TRNS: ctx->opt_bintrns = v; break;
	}
}

void iw_set_grayscale_weights(struct iw_context *ctx, double r, double g, double b)
{
	double tot = r + g + b;
	if(tot == 0.0) tot = 1.0;
	ctx->gsw[0] = r / tot;
	ctx->gsw[1] = g / tot;
	ctx->gsw[2] = b / tot;
}

void iw_set_resize_alg(struct iw_context *ctx, int dimension, int family, double blur, double p1, double p2)
{
	if(dimension < 0 || dimension > 1) dimension = 0;
	iwg::DimRequest &d = ctx->dim[dimension];
	d.family = family;
	d.blur = blur;
	d.p1 = p1;
	d.p2 = p2;
}

// Composes an orientation change with the current one (src/imagew-api.c:651-680).
void iw_reorient_image(struct iw_context *ctx, unsigned int x)
{
	static const unsigned int transposed[8] = {4, 6, 5, 7, 0, 2, 1, 3};
	x &= 7;
	if(x & 4) {
		ctx->img1.orient_transform = transposed[ctx->img1.orient_transform & 7];
		int t = ctx->img1.width; ctx->img1.width = ctx->img1.height; ctx->img1.height = t;
		double d = ctx->img1.density_x; ctx->img1.density_x = ctx->img1.density_y; ctx->img1.density_y = d;
	}
	ctx->img1.orient_transform ^= (x & 3);
}

// String options (src/imagew-api.c:996-1042).  At most 32 are kept.
void iw_set_option(struct iw_context *ctx, const char *name, const char *val)
{
	if(!val || !val[0]) val = "1";
	if(!ctx->opts) {
		ctx->opts = (iw_context::Option *)iw_mallocz(ctx, 32 * sizeof(iw_context::Option));
		if(!ctx->opts) return;
		ctx->nopts = 0;
	}
	for(int i = 0; i < ctx->nopts; i++) {
		if(ctx->opts[i].name && !strcmp(ctx->opts[i].name, name)) {
			iw_free(ctx, ctx->opts[i].val);
			ctx->opts[i].val = iw_strdup(ctx, val);
			return;
		}
	}
	if(ctx->nopts >= 32) return;
	ctx->opts[ctx->nopts].name = iw_strdup(ctx, name);
	ctx->opts[ctx->nopts].val = iw_strdup(ctx, val);
	ctx->nopts++;
}

const char *iw_get_option(struct iw_context *ctx, const char *name)
{
	for(int i = 0; i < ctx->nopts; i++)
		if(ctx->opts[i].name && !strcmp(ctx->opts[i].name, name)) return ctx->opts[i].val;
	return nullptr;
}

static void set_option_number(struct iw_context *ctx, const char *name, double v)
{
	char buf[100];
	iw_snprintf(buf, sizeof(buf), "%.20f", v);
	iw_set_option(ctx, name, buf);
}

// src/imagew-api.c:760-863
void iw_set_value(struct iw_context *ctx, int code, int n)
{
	switch(code) {
	case IW_VAL_API_VERSION: ctx->api_version = n; break;
	case IW_VAL_CVT_TO_GRAYSCALE: ctx->to_gray = n; break;
	case IW_VAL_DISABLE_GAMMA: ctx->no_gamma = n; break;
	case IW_VAL_NO_CSLABEL: ctx->no_cslabel = n; break;
	case IW_VAL_INT_CLAMP: ctx->intclamp = n; break;
	case IW_VAL_EDGE_POLICY_X: ctx->dim[IW_DIMENSION_H].edge = n; break;
	case IW_VAL_EDGE_POLICY_Y: ctx->dim[IW_DIMENSION_V].edge = n; break;
	case IW_VAL_PREF_UNITS: ctx->pref_units = n; break;
	case IW_VAL_GRAYSCALE_FORMULA: ctx->gsf = n; break;
	case IW_VAL_INPUT_NATIVE_GRAYSCALE: ctx->img1.native_grayscale = n; break;
	case IW_VAL_COMPRESSION: ctx->compression = n; break;
	case IW_VAL_PAGE_TO_READ: ctx->page = n; break;
	case IW_VAL_INCLUDE_SCREEN: ctx->include_screen = n; break;
	case IW_VAL_JPEG_QUALITY: set_option_number(ctx, "jpeg:quality", n); break;
	case IW_VAL_JPEG_SAMP_FACTOR_H: set_option_number(ctx, "jpeg:sampling-x", n); break;
	case IW_VAL_JPEG_SAMP_FACTOR_V: set_option_number(ctx, "jpeg:sampling-y", n); break;
	case IW_VAL_JPEG_ARITH_CODING: set_option_number(ctx, "jpeg:arith", n); break;
	case IW_VAL_DEFLATE_CMPR_LEVEL: set_option_number(ctx, "deflate:cmprlevel", n); break;
	case IW_VAL_OUTPUT_INTERLACED: ctx->interlaced = n; break;
	case IW_VAL_USE_BKGD_LABEL: ctx->use_file_label = n; break;
	case IW_VAL_BMP_NO_FILEHEADER: ctx->bmp_nofh = n; break;
	case IW_VAL_BMP_VERSION: set_option_number(ctx, "bmp:version", n); break;
	case IW_VAL_MAX_WIDTH: ctx->max_w = n; break;
	case IW_VAL_MAX_HEIGHT: ctx->max_h = n; break;
	case IW_VAL_NO_BKGD_LABEL: ctx->no_outlabel = n; break;
	case IW_VAL_INTENT: ctx->req_intent = n; break;
	case IW_VAL_OUTPUT_SAMPLE_TYPE: ctx->req_sampletype = n; break;
	case IW_VAL_OUTPUT_COLOR_TYPE:
		if(n == IW_COLORTYPE_RGB) iw_set_option(ctx, "deflate:colortype", "rgb");
		break;
	case IW_VAL_OUTPUT_FORMAT: ctx->out_fmt = n; break;
	case IW_VAL_NEGATE_TARGET: ctx->negate = n; break;
	}
}

int iw_get_value(struct iw_context *ctx, int code)
{
	switch(code) {
	case IW_VAL_API_VERSION: return ctx->api_version;
	case IW_VAL_CVT_TO_GRAYSCALE: return ctx->to_gray;
	case IW_VAL_DISABLE_GAMMA: return ctx->no_gamma;
	case IW_VAL_NO_CSLABEL: return ctx->no_cslabel;
	case IW_VAL_INT_CLAMP: return ctx->intclamp;
	case IW_VAL_EDGE_POLICY_X: return ctx->dim[IW_DIMENSION_H].edge;
	case IW_VAL_EDGE_POLICY_Y: return ctx->dim[IW_DIMENSION_V].edge;
	case IW_VAL_PREF_UNITS: return ctx->pref_units;
	case IW_VAL_GRAYSCALE_FORMULA: return ctx->gsf;
	case IW_VAL_INPUT_NATIVE_GRAYSCALE: return ctx->img1.native_grayscale;
	case IW_VAL_INPUT_WIDTH: return ctx->img1.width < 1 ? 1 : ctx->img1.width;
	case IW_VAL_INPUT_HEIGHT: return ctx->img1.height < 1 ? 1 : ctx->img1.height;
	case IW_VAL_INPUT_IMAGE_TYPE: return ctx->img1.imgtype;
	case IW_VAL_INPUT_DEPTH: return ctx->img1.bit_depth;
	case IW_VAL_COMPRESSION: return ctx->compression;
	case IW_VAL_PAGE_TO_READ: return ctx->page;
	case IW_VAL_INCLUDE_SCREEN: return ctx->include_screen;
	case IW_VAL_OUTPUT_PALETTE_GRAYSCALE: return ctx->opt.pal_is_gray;
	case IW_VAL_OUTPUT_INTERLACED: return ctx->interlaced;
	case IW_VAL_USE_BKGD_LABEL: return ctx->use_file_label;
	case IW_VAL_BMP_NO_FILEHEADER: return ctx->bmp_nofh;
	case IW_VAL_MAX_WIDTH: return ctx->max_w;
	case IW_VAL_MAX_HEIGHT: return ctx->max_h;
	case IW_VAL_PRECISION: return 32;
	case IW_VAL_NO_BKGD_LABEL: return ctx->no_outlabel;
	case IW_VAL_INTENT: return ctx->req_intent;
	case IW_VAL_OUTPUT_SAMPLE_TYPE: return ctx->req_sampletype;
	case IW_VAL_OUTPUT_FORMAT: return ctx->out_fmt;
	case IW_VAL_NEGATE_TARGET: return ctx->negate;
	}
	return 0;
}

void iw_set_value_dbl(struct iw_context *ctx, int code, double n)
{
	if(code == IW_VAL_WEBP_QUALITY) set_option_number(ctx, "webp:quality", n);
	else if(code == IW_VAL_TRANSLATE_X) ctx->dim[IW_DIMENSION_H].translate = n;
	else if(code == IW_VAL_TRANSLATE_Y) ctx->dim[IW_DIMENSION_V].translate = n;
}

double iw_get_value_dbl(struct iw_context *ctx, int code)
{
	if(code == IW_VAL_TRANSLATE_X) return ctx->dim[IW_DIMENSION_H].translate;
	if(code == IW_VAL_TRANSLATE_Y) return ctx->dim[IW_DIMENSION_V].translate;
	return 0.0;
}

double iw_convert_sample_to_linear(double v, const struct iw_csdescr *cs) { return iwg::to_linear(v, *cs); }
double iw_convert_sample_from_linear(double v, const struct iw_csdescr *cs) { return iwg::from_linear(v, *cs); }

// ===== processing (src/imagew-main.c:2250-2272) ============================

int iw_process_image(struct iw_context *ctx)
{
	if(ctx->use_count > 0) {
		iw_set_error(ctx, "Internal: Incorrect attempt to reprocess image");
		return 0;
	}
	ctx->use_count++;
	using Clk = std::chrono::steady_clock;
	auto ms = [](Clk::time_point a, Clk::time_point b) { return std::chrono::duration<double, std::milli>(b - a).count(); };
	const auto t0 = Clk::now();
	iwg::Plan P;
	if(!iwg::build_plan(ctx, P)) return 0;
	const auto t1 = Clk::now();
	if(!iwg::run_pipeline(ctx, P)) return 0;
	const auto t2 = Clk::now();
	iwg::bkgd_label(ctx, P);
	iwg::optimize(ctx);
	const auto t3 = Clk::now();
	ctx->stats.ms_phase[0] = ms(t0, t1);
	ctx->stats.ms_phase[4] = ms(t2, t3);
	ctx->stats.ms_phase[5] = ms(t1, t2);
	ctx->stats.ms_total = ms(t0, t3);
	return 1;
}

void iw_get_output_image(struct iw_context *ctx, struct iw_image *img)
{
	const iwg::OptState &o = ctx->opt;
	memset(img, 0, sizeof(*img));
	img->width = o.width;
	img->height = o.height;
	img->imgtype = o.imgtype;
	img->sampletype = ctx->img2.sampletype;
	img->bit_depth = o.bit_depth;
	img->pixels = (iw_byte *)o.pix;
	img->bpr = o.bpr;
	img->density_code = ctx->img2.density_code;
	img->density_x = ctx->img2.density_x;
	img->density_y = ctx->img2.density_y;
	img->rendering_intent = ctx->img2.rendering_intent;
	img->has_bkgdlabel = o.has_label;
	for(int k = 0; k < 4; k++) img->bkgdlabel.c[k] = ((double)o.label[k]) / (o.bit_depth == 8 ? 255.0 : 65535.0);
	img->has_colorkey_trns = o.has_ckey;
	for(int k = 0; k < 3; k++) img->colorkey[k] = o.ckey[k];
	if(ctx->reduced_out) {
		img->reduced_maxcolors = 1;
		if(IW_IMGTYPE_IS_GRAY(img->imgtype)) {
			img->maxcolorcode[IW_CHANNELTYPE_GRAY] = ctx->out_maxcc[0];
			if(IW_IMGTYPE_HAS_ALPHA(img->imgtype)) img->maxcolorcode[IW_CHANNELTYPE_ALPHA] = ctx->out_maxcc[1];
		}
		else {
			img->maxcolorcode[IW_CHANNELTYPE_RED] = ctx->out_maxcc[0];
			img->maxcolorcode[IW_CHANNELTYPE_GREEN] = ctx->out_maxcc[1];
			img->maxcolorcode[IW_CHANNELTYPE_BLUE] = ctx->out_maxcc[2];
			if(IW_IMGTYPE_HAS_ALPHA(img->imgtype)) img->maxcolorcode[IW_CHANNELTYPE_ALPHA] = ctx->out_maxcc[3];
		}
	}
}

// ===== stateless helpers (src/imagew-api.c:682-758, src/imagew-util.c) ====

int iw_get_sample_size(void) { return (int)sizeof(float); }
int iw_get_version_int(void) { return IW_VERSION_INT; }

char *iw_get_version_string(struct iw_context *, char *s, int n)
{
	iw_snprintf(s, n, "%d.%d.%d", (IW_VERSION_INT >> 16) & 0xff, (IW_VERSION_INT >> 8) & 0xff, IW_VERSION_INT & 0xff);
	return s;
}

char *iw_get_copyright_string(struct iw_context *ctx, char *s, int n)
{
	iw_translatef(ctx, 0, s, n, "Copyright \xc2\xa9 %s %s", "2011\xe2\x80\x93" "2022", "Jason Summers");
	return s;
}

unsigned int iw_color_get_int_sample(struct iw_color *clr, int ch, unsigned int maxcc)
{
	int n = (int)(0.5 + (clr->c[ch] * (double)maxcc));
	if(n < 0) n = 0;
	else if(n > (int)maxcc) n = (int)maxcc;
	return (unsigned int)n;
}

int iw_get_host_endianness(void)
{
	unsigned int x = 1;
	iw_byte b;
	memcpy(&b, &x, 1);
	return b == 0 ? IW_ENDIAN_BIG : IW_ENDIAN_LITTLE;
}

void iw_set_ui16le(iw_byte *b, unsigned int n) { b[0] = n & 0xff; b[1] = (n >> 8) & 0xff; }
void iw_set_ui32le(iw_byte *b, unsigned int n) { for(int i = 0; i < 4; i++) b[i] = (n >> (8 * i)) & 0xff; }
void iw_set_ui16be(iw_byte *b, unsigned int n) { b[0] = (n >> 8) & 0xff; b[1] = n & 0xff; }
void iw_set_ui32be(iw_byte *b, unsigned int n) { for(int i = 0; i < 4; i++) b[i] = (n >> (24 - 8 * i)) & 0xff; }
unsigned int iw_get_ui16le(const iw_byte *b) { return (unsigned int)b[0] | ((unsigned int)b[1] << 8); }
unsigned int iw_get_ui32le(const iw_byte *b) { return (unsigned int)b[0] | ((unsigned int)b[1] << 8) | ((unsigned int)b[2] << 16) | ((unsigned int)b[3] << 24); }
int iw_get_i32le(const iw_byte *b) { return (int32_t)iw_get_ui32le(b); }
unsigned int iw_get_ui16be(const iw_byte *b) { return ((unsigned int)b[0] << 8) | (unsigned int)b[1]; }
unsigned int iw_get_ui32be(const iw_byte *b) { return ((unsigned int)b[0] << 24) | ((unsigned int)b[1] << 16) | ((unsigned int)b[2] << 8) | (unsigned int)b[3]; }
unsigned int iw_get_ui16_e(const iw_byte *b, int e) { return e == IW_ENDIAN_LITTLE ? iw_get_ui16le(b) : iw_get_ui16be(b); }
unsigned int iw_get_ui32_e(const iw_byte *b, int e) { return e == IW_ENDIAN_LITTLE ? iw_get_ui32le(b) : iw_get_ui32be(b); }

int iw_max_color_to_bitdepth(unsigned int mc)
{
	for(unsigned int bd = 1; bd <= 15; bd++) if(mc < (1U << bd)) return (int)bd;
	return 16;
}

unsigned int iw_get_profile_by_fmt(int fmt)
{
	switch(fmt) {
	case IW_FORMAT_PNG:
		return IW_PROFILE_TRANSPARENCY | IW_PROFILE_GRAYSCALE | IW_PROFILE_PALETTETRNS | IW_PROFILE_GRAY1 |
			IW_PROFILE_GRAY2 | IW_PROFILE_GRAY4 | IW_PROFILE_16BPS | IW_PROFILE_BINARYTRNS | IW_PROFILE_PAL1 |
			IW_PROFILE_PAL2 | IW_PROFILE_PAL4 | IW_PROFILE_PAL8 | IW_PROFILE_REDUCEDBITDEPTHS | IW_PROFILE_PNG_BKGD;
	case IW_FORMAT_BMP: return IW_PROFILE_PAL1 | IW_PROFILE_PAL4 | IW_PROFILE_PAL8 | IW_PROFILE_REDUCEDBITDEPTHS;
	case IW_FORMAT_JPEG: return IW_PROFILE_GRAYSCALE;
	case IW_FORMAT_TIFF:
		return IW_PROFILE_TRANSPARENCY | IW_PROFILE_GRAYSCALE | IW_PROFILE_GRAY1 | IW_PROFILE_GRAY4 |
			IW_PROFILE_16BPS | IW_PROFILE_PAL4 | IW_PROFILE_PAL8;
	case IW_FORMAT_MIFF:
		return IW_PROFILE_TRANSPARENCY | IW_PROFILE_GRAYSCALE | IW_PROFILE_ALWAYSLINEAR | IW_PROFILE_HDRI | IW_PROFILE_RGB16_BKGD;
	case IW_FORMAT_WEBP: return IW_PROFILE_TRANSPARENCY;
	case IW_FORMAT_PAM:
		return IW_PROFILE_16BPS | IW_PROFILE_REDUCEDBITDEPTHS | IW_PROFILE_GRAYSCALE | IW_PROFILE_GRAY1 | IW_PROFILE_TRANSPARENCY;
	case IW_FORMAT_PNM: return IW_PROFILE_16BPS | IW_PROFILE_REDUCEDBITDEPTHS | IW_PROFILE_GRAYSCALE | IW_PROFILE_GRAY1;
	case IW_FORMAT_PPM: return IW_PROFILE_16BPS | IW_PROFILE_REDUCEDBITDEPTHS;
	case IW_FORMAT_PGM: return IW_PROFILE_16BPS | IW_PROFILE_REDUCEDBITDEPTHS | IW_PROFILE_GRAYSCALE;
	case IW_FORMAT_PBM: return IW_PROFILE_GRAY1;
	}
	return 0;
}

int iw_detect_fmt_from_filename(const char *fn)
{
	static const struct { const char *ext; int fmt; } t[] = {
		{"png", IW_FORMAT_PNG}, {"jpg", IW_FORMAT_JPEG}, {"jpeg", IW_FORMAT_JPEG}, {"bmp", IW_FORMAT_BMP},
		{"tif", IW_FORMAT_TIFF}, {"tiff", IW_FORMAT_TIFF}, {"miff", IW_FORMAT_MIFF}, {"webp", IW_FORMAT_WEBP},
		{"gif", IW_FORMAT_GIF}, {"pnm", IW_FORMAT_PNM}, {"pbm", IW_FORMAT_PBM}, {"pgm", IW_FORMAT_PGM},
		{"ppm", IW_FORMAT_PPM}, {"pam", IW_FORMAT_PAM}};
	const char *s = strrchr(fn, '.');
	if(!s) return IW_FORMAT_UNKNOWN;
	for(const auto &e : t) if(!iw_stricmp(s + 1, e.ext)) return e.fmt;
	return IW_FORMAT_UNKNOWN;
}

const char *iw_get_fmt_name(int fmt)
{
	switch(fmt) {
	case IW_FORMAT_PNG: return "PNG";
	case IW_FORMAT_JPEG: return "JPEG";
	case IW_FORMAT_BMP: return "BMP";
	case IW_FORMAT_TIFF: return "TIFF";
	case IW_FORMAT_MIFF: return "MIFF";
	case IW_FORMAT_WEBP: return "WebP";
	case IW_FORMAT_GIF: return "GIF";
	case IW_FORMAT_PNM: return "PNM";
	case IW_FORMAT_PBM: return "PBM";
	case IW_FORMAT_PGM: return "PGM";
	case IW_FORMAT_PPM: return "PPM";
	case IW_FORMAT_PAM: return "PAM";
	}
	return nullptr;
}

int iw_detect_fmt_of_file(const iw_byte *b, size_t n)
{
	if(n < 2) return IW_FORMAT_UNKNOWN;
	if(b[0] == 0x89 && b[1] == 0x50) return IW_FORMAT_PNG;
	if(n >= 3 && b[0] == 'G' && b[1] == 'I' && b[2] == 'F') return IW_FORMAT_GIF;
	if(b[0] == 0xff && b[1] == 0xd8) return IW_FORMAT_JPEG;
	if(b[0] == 'B' && (b[1] == 'M' || b[1] == 'A')) return IW_FORMAT_BMP;
	if((b[0] == 0x49 || b[0] == 0x4d) && b[1] == b[0]) return IW_FORMAT_TIFF;
	if(b[0] == 0x69 && b[1] == 0x64) return IW_FORMAT_MIFF;
	if(n >= 12 && !memcmp(b, "RIFF", 4) && !memcmp(b + 8, "WEBP", 4)) return IW_FORMAT_WEBP;
	if(b[0] == 'P' && b[1] >= '1' && b[1] <= '6') return IW_FORMAT_PNM;
	if(b[0] == 'P' && b[1] == '7' && n >= 3 && b[2] == 0x0a) return IW_FORMAT_PAM;
	return IW_FORMAT_UNKNOWN;
}

// This library has no file codecs; these report what the reference's
// pixel-format modules would accept.
int iw_is_input_fmt_supported(int fmt)
{
	return fmt == IW_FORMAT_MIFF || fmt == IW_FORMAT_GIF || fmt == IW_FORMAT_BMP || fmt == IW_FORMAT_PNM || fmt == IW_FORMAT_PAM;
}

int iw_is_output_fmt_supported(int fmt)
{
	switch(fmt) {
	case IW_FORMAT_BMP: case IW_FORMAT_TIFF: case IW_FORMAT_MIFF: case IW_FORMAT_PNM:
	case IW_FORMAT_PPM: case IW_FORMAT_PGM: case IW_FORMAT_PBM: case IW_FORMAT_PAM:
		return 1;
	}
	return 0;
}

void iw_utf8_to_ascii(const char *src, char *dst, int dstlen)
{
	static const struct { unsigned int code; const char *s; } map[] = {
		{0x00a9, "(c)"}, {0x00d7, "x"}, {0x2013, "-"}, {0x2018, "'"}, {0x2019, "'"},
		{0x201c, "\""}, {0x201d, "\""}, {0x2192, "->"}, {0xfeff, ""}};
	int dp = 0, need = 0;
	unsigned int cp = 0;
	auto emit = [&](char c) { if(dp <= dstlen - 2) dst[dp++] = c; };
	for(; *src; src++) {
		unsigned char c = (unsigned char)*src;
		if(c < 128) { emit((char)c); need = 0; continue; }
		if(c < 0xc0) {
			if(need > 0) {
				cp = (cp << 6) | (c & 0x3f);
				if(--need < 1) {
					const char *rep = "?";
					for(const auto &m : map) if(m.code == cp) { rep = m.s; break; }
					for(; *rep; rep++) emit(*rep);
				}
			}
		}
		else if(c < 0xe0) { cp = c & 0x1f; need = 1; }
		else if(c < 0xf0) { cp = c & 0x0f; need = 2; }
		else if(c < 0xf8) { cp = c & 0x07; need = 3; }
	}
	dst[dp] = '\0';
}

static int parse_one(const char *s, double *out, int *used)
{
	int slash = -1, len = 0;
	for(len = 0; s[len]; len++) {
		if(s[len] == '/') slash = len;
		if(s[len] == ',') break;
	}
	*out = 0.0;
	*used = 0;
	if(len < 1) return 0;
	*used = len;
	if(slash >= 0) {
		double num = atof(s), den = atof(s + slash + 1);
		*out = den == 0.0 ? 0.0 : num / den;
	}
	else *out = atof(s);
	return 1;
}

int iw_parse_number_list(const char *s, int maxn, double *res)
{
	int n, used, pos = 0;
	for(n = 0; n < maxn; n++) {
		if(!parse_one(s + pos, &res[n], &used)) break;
		pos += used;
		if(s[pos] != ',') return n + 1;
		pos++;
	}
	return n;
}

double iw_parse_number(const char *s)
{
	double r;
	int used;
	parse_one(s, &r, &used);
	return r;
}

int iw_round_to_int(double x) { return x < 0.0 ? -(int)(0.5 - x) : (int)(0.5 + x); }
int iw_parse_int(const char *s) { return iw_round_to_int(iw_parse_number(s)); }

}  // extern "C"

const char *iwg::get_option(iw_context *ctx, const char *name) { return iw_get_option(ctx, name); }

// ===== additive ABI: timed processing (include/imagew_gb300.h) =============

extern "C" int iwg_process_image_timed(struct iw_context *ctx, int warmup, int iters)
{
	if(ctx->use_count > 0) {
		iw_set_error(ctx, "Internal: Incorrect attempt to reprocess image");
		return 0;
	}
	ctx->use_count++;
	auto t0 = std::chrono::steady_clock::now();
	iwg::Plan P;
	if(!iwg::build_plan(ctx, P)) return 0;
	if(!iwg::run_pipeline(ctx, P, warmup < 0 ? 0 : warmup, iters < 1 ? 1 : iters)) return 0;
	iwg::bkgd_label(ctx, P);
	iwg::optimize(ctx);
	ctx->stats.ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
	return 1;
}

// ---- batches (include/imagew_gb300.h) ----

namespace {

// Runs fn(i) for i in [0, n) on up to hardware_concurrency threads.
template<class Fn>
void parallel_for(int n, Fn fn)
{
	int T = (int)std::thread::hardware_concurrency();
	T = std::max(1, std::min(T, std::min(n, 64)));
	if(T == 1) {
		for(int i = 0; i < n; i++) fn(i);
		return;
	}
	std::atomic<int> next(0);
	std::vector<std::thread> th;
	for(int t = 0; t < T; t++)
		th.emplace_back([&]() {
			for(int i = next++; i < n; i = next++) fn(i);
		});
	for(std::thread &x : th) x.join();
}

}  // namespace

// Output channels quantised by a serial scan (error-diffusion / random dither).
bool iwg::plan_needs_scan(const iwg::Plan &P)
{
	if(P.out_sampletype != IW_SAMPLETYPE_UINT) return false;
	for(int oc = 0; oc < P.out_n; oc++) {
		const int f = P.out[oc].q.dfam;
		if(f == IW_DITHERFAMILY_ERRDIFF || f == IW_DITHERFAMILY_RANDOM) return true;
	}
	return false;
}

// Device bytes one image of a batch holds while it runs (input, float
// intermediate, output, flag entries; scan buffers for serial dither).
size_t iwg::batch_device_bytes(const iwg::Plan &P)
{
	const size_t in = plan_in_bpr(P) * (size_t)(P.orient >= 4 ? P.img1_w : P.img1_h);
	const size_t mid = (size_t)P.mid_n * P.crop_w * P.out_h * sizeof(float);
	const size_t out = P.out_bpr * (size_t)P.out_h;
	size_t scan = 0;
	if(plan_needs_scan(P)) scan = (size_t)P.out_n * P.out_w * ((size_t)P.out_h + 4) * sizeof(double);
	return in + mid + out + scan + (size_t)P.out_w * P.out_h * 16 + 4096;
}

// Host wall time of iwg_process_batch's stages, process-wide sums (ms):
// planning, fast-form batches, plain-form batches, output post-pass.
static std::mutex g_bstage_mu;
static double g_bstage_ms[4] = {0, 0, 0, 0};

static void bstage_add(int k, std::chrono::steady_clock::time_point &t)
{
	const auto n = std::chrono::steady_clock::now();
	std::lock_guard<std::mutex> lk(g_bstage_mu);
	g_bstage_ms[k] += std::chrono::duration<double, std::milli>(n - t).count();
	t = n;
}

extern "C" int iwg_batch_phase_ms(double *out, int n)
{
	double v[4 + iwg::kBatchPhases];
	{
		std::lock_guard<std::mutex> lk(g_bstage_mu);
		for(int k = 0; k < 4; k++) v[k] = g_bstage_ms[k];
	}
	iwg::batch_phase_ms(v + 4);
	int m = 0;
	for(; out && m < n && m < 4 + iwg::kBatchPhases; m++) out[m] = v[m];
	return m;
}

extern "C" int iwg_process_batch(struct iw_context **ctxs, int n)
{
	if(!ctxs || n <= 0) return 0;
	auto t0 = std::chrono::steady_clock::now();
	auto ts = t0;
	std::vector<iwg::Plan> plans(n);
	std::vector<char> planned(n, 0);
	parallel_for(n, [&](int i) {
		iw_context *ctx = ctxs[i];
		if(!ctx) return;
		if(ctx->use_count > 0) {
			iw_set_error(ctx, "Internal: Incorrect attempt to reprocess image");
			return;
		}
		ctx->use_count++;
		planned[i] = iwg::build_plan(ctx, plans[i]) ? 1 : 0;
	});
	bstage_add(0, ts);
	// chunks of at most kBudget device bytes, in the callers' order
	const size_t kBudget = (size_t)8 << 30;
	std::vector<char> done(n, 0);
	std::vector<int> order;
	for(int i = 0; i < n; i++) if(planned[i]) order.push_back(i);
	std::vector<char> batched(n, 0);
	double dev_total = 0;
	size_t k = 0;
	while(k < order.size()) {
		std::vector<iw_context *> cc;
		std::vector<iwg::Plan *> pp;
		std::vector<int> idx;
		size_t bytes = 0;
		while(k < order.size()) {
			const int i = order[k];
			const size_t b = iwg::batch_device_bytes(plans[i]);
			if(!idx.empty() && bytes + b > kBudget) break;
			bytes += b;
			cc.push_back(ctxs[i]);
			pp.push_back(&plans[i]);
			idx.push_back(i);
			k++;
		}
		std::vector<int> status;
		double dev_ms = 0;
		ts = std::chrono::steady_clock::now();
		iwg::run_batch(cc, pp, status, dev_ms);
		bstage_add(1, ts);
		dev_total += dev_ms;
		// what the fast form did not take: one batch in the plain form
		std::vector<iw_context *> cc2;
		std::vector<iwg::Plan *> pp2;
		std::vector<int> idx2;
		for(size_t j = 0; j < idx.size(); j++) {
			const int i = idx[j];
			if(status[j] == 1) done[i] = batched[i] = 1;
			else if(status[j] == 0) {
				cc2.push_back(ctxs[i]);
				pp2.push_back(&plans[i]);
				idx2.push_back(i);
			}
		}
		if(!cc2.empty()) {
			std::vector<int> status2;
			iwg::run_batch_plain(cc2, pp2, status2, dev_ms);
			bstage_add(2, ts);
			dev_total += dev_ms;
			for(size_t j = 0; j < idx2.size(); j++) {
				const int i = idx2[j];
				if(status2[j] == 1) done[i] = batched[i] = 1;
				else if(status2[j] == 0) done[i] = iwg::run_pipeline(ctxs[i], plans[i]) ? 1 : 0;   // alone
			}
		}
	}
	ts = std::chrono::steady_clock::now();
	parallel_for(n, [&](int i) {
		if(!done[i]) return;
		iwg::bkgd_label(ctxs[i], plans[i]);
		iwg::optimize(ctxs[i]);
	});
	bstage_add(3, ts);
	const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
	int ok = 0;
	for(int i = 0; i < n; i++)
		if(done[i]) {
			ctxs[i]->stats.ms_total = ms;
			if(batched[i]) ctxs[i]->stats.ms_device = dev_total;
			ok++;
		}
	return ok;
}

