/*
 * iw_oracle.c -- CPU oracle: a plain-C restatement of ImageWorsener 1.3.5's
 * iw_process_image() path and the settings API that feeds it.
 *
 * TEST INFRASTRUCTURE ONLY (see iw_oracle.h).  Built with -ffp-contract=off:
 * every multiply and add below is a separately rounded IEEE double operation,
 * in the same order as the reference, which is what makes the output
 * byte-identical to the reference's.
 *
 * Where the reference walks the image column by column, the oracle walks it in
 * whatever order is convenient; the value computed for each sample, and the
 * order of the terms summed into it, are the reference's.
 */
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#include <stdarg.h>
#include <math.h>
#include <time.h>
#include <strings.h>

#include "iw_oracle.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ====================================================================== */
/* Allocation (src/imagew-util.c:24-137)                                  */
/* ====================================================================== */

static void *orc_default_malloc(void *ud, unsigned int flags, size_t n)
{
	return (flags & IW_MALLOCFLAG_ZEROMEM) ? calloc(n, 1) : malloc(n);
}

static void orc_default_free(void *ud, void *m)
{
	free(m);
}

void *iw_malloc_ex(struct iw_context *ctx, unsigned int flags, size_t n)
{
	void *m = NULL;
	if(n <= ctx->max_malloc) m = ctx->mallocfn(ctx->userdata, flags, n);
	if(!m && !(flags & IW_MALLOCFLAG_NOERRORS)) iw_set_error(ctx, "Out of memory");
	return m;
}

void *iw_malloc(struct iw_context *ctx, size_t n) { return iw_malloc_ex(ctx, 0, n); }
void *iw_mallocz(struct iw_context *ctx, size_t n) { return iw_malloc_ex(ctx, IW_MALLOCFLAG_ZEROMEM, n); }

void *iw_malloc_large(struct iw_context *ctx, size_t n1, size_t n2)
{
	if(n1 > ctx->max_malloc / n2) {
		iw_set_error(ctx, "Image too large to process");
		return NULL;
	}
	return iw_malloc_ex(ctx, 0, n1 * n2);
}

void *iw_realloc_ex(struct iw_context *ctx, unsigned int flags, void *old, size_t oldn, size_t n)
{
	void *m;
	if(!old) return iw_malloc_ex(ctx, flags, n);
	if(n > ctx->max_malloc) {
		if(!(flags & IW_MALLOCFLAG_NOERRORS)) iw_set_error(ctx, "Out of memory");
		return NULL;
	}
	/* Always a fresh block; the old one is freed even on failure. */
	m = ctx->mallocfn(ctx->userdata, flags, n);
	if(m) memcpy(m, old, oldn < n ? oldn : n);
	ctx->freefn(ctx->userdata, old);
	if(!m && !(flags & IW_MALLOCFLAG_NOERRORS)) iw_set_error(ctx, "Out of memory");
	return m;
}

void *iw_realloc(struct iw_context *ctx, void *m, size_t oldn, size_t n)
{
	return iw_realloc_ex(ctx, 0, m, oldn, n);
}

void iw_free(struct iw_context *ctx, void *m)
{
	if(m) ctx->freefn(ctx->userdata, m);
}

char *iw_strdup(struct iw_context *ctx, const char *s)
{
	size_t n;
	char *d;
	if(!s) return NULL;
	n = strlen(s) + 1;
	d = iw_malloc(ctx, n);
	if(d) memcpy(d, s, n);
	return d;
}

/* ====================================================================== */
/* Strings, translation, errors (src/imagew-api.c:15-162)                 */
/* ====================================================================== */

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

void iw_translatev(struct iw_context *ctx, unsigned int flags, char *dst, size_t dstlen,
	const char *fmt, va_list ap)
{
	char a[ORC_MSG_MAX], b[ORC_MSG_MAX];
	if(!ctx || !ctx->xlate) {
		iw_vsnprintf(dst, dstlen, fmt, ap);
		return;
	}
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

static void orc_record_error(struct iw_context *ctx, const char *msg)
{
	if(ctx->error_flag) return;
	ctx->error_flag = 1;
	if(!ctx->error_msg) {
		ctx->error_msg = iw_malloc_ex(ctx, IW_MALLOCFLAG_NOERRORS, ORC_MSG_MAX);
		if(!ctx->error_msg) return;
	}
	iw_strlcpy(ctx->error_msg, msg, ORC_MSG_MAX);
}

void iw_set_error(struct iw_context *ctx, const char *s)
{
	char buf[ORC_MSG_MAX];
	if(ctx->error_flag) return;
	iw_translate(ctx, IW_TRANSLATEFLAG_ERRORMSG, buf, sizeof(buf), s);
	orc_record_error(ctx, buf);
}

void iw_set_errorv(struct iw_context *ctx, const char *fmt, va_list ap)
{
	char buf[ORC_MSG_MAX];
	if(ctx->error_flag) return;
	iw_translatev(ctx, IW_TRANSLATEFLAG_ERRORMSG, buf, sizeof(buf), fmt, ap);
	orc_record_error(ctx, buf);
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
	char buf[ORC_MSG_MAX];
	if(!ctx->warn) return;
	iw_translate(ctx, IW_TRANSLATEFLAG_WARNINGMSG, buf, sizeof(buf), s);
	ctx->warn(ctx, buf);
}

void iw_warningv(struct iw_context *ctx, const char *fmt, va_list ap)
{
	char buf[ORC_MSG_MAX];
	if(!ctx->warn) return;
	iw_translatev(ctx, IW_TRANSLATEFLAG_WARNINGMSG, buf, sizeof(buf), fmt, ap);
	ctx->warn(ctx, buf);
}

void iw_warningf(struct iw_context *ctx, const char *fmt, ...)
{
	va_list ap;
	if(!ctx->warn) return;
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

/* ====================================================================== */
/* Small shared helpers (src/imagew-api.c:164-196)                        */
/* ====================================================================== */

int iw_imgtype_num_channels(int t)
{
	if(t == IW_IMGTYPE_RGBA) return 4;
	if(t == IW_IMGTYPE_RGB) return 3;
	if(t == IW_IMGTYPE_GRAYA) return 2;
	return 1;
}

static int orc_alpha_index(int t)
{
	if(t == IW_IMGTYPE_RGBA) return 3;
	if(t == IW_IMGTYPE_GRAYA) return 1;
	return 0;
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

/* ====================================================================== */
/* Context lifetime and settings (src/imagew-api.c:198-1042)              */
/* ====================================================================== */

static void orc_dim_defaults(struct orc_dim *d)
{
	memset(d, 0, sizeof(*d));
	d->family = IW_RESIZETYPE_AUTO;
	d->edge = IW_EDGE_POLICY_STANDARD;
	d->blur = 1.0;
}

struct iw_context *iw_create_context(struct iw_init_params *params)
{
	struct iw_context *ctx;
	int custom = params && params->mallocfn;

	ctx = custom ? params->mallocfn(params->userdata, IW_MALLOCFLAG_ZEROMEM, sizeof(*ctx))
	             : orc_default_malloc(NULL, IW_MALLOCFLAG_ZEROMEM, sizeof(*ctx));
	if(!ctx) return NULL;
	if(params) {
		ctx->userdata = params->userdata;
		ctx->api_version = params->api_version;
	}
	ctx->mallocfn = custom ? params->mallocfn : orc_default_malloc;
	ctx->freefn = custom ? params->freefn : orc_default_free;
	ctx->max_malloc = 2000000000;
	ctx->max_w = ctx->max_h = 40000;
	orc_dim_defaults(&ctx->dim[0]);
	orc_dim_defaults(&ctx->dim[1]);
	ctx->crop_w = ctx->crop_h = -1;
	iw_make_srgb_csdescr_2(&ctx->cs_in);
	iw_make_srgb_csdescr_2(&ctx->cs_out);
	ctx->gsf = IW_GSF_STANDARD;
	ctx->include_screen = 1;
	ctx->opt_gray = ctx->opt_pal = ctx->opt_16to8 = ctx->opt_strip = ctx->opt_bintrns = 1;
	return ctx;
}

void iw_destroy_context(struct iw_context *ctx)
{
	int i;
	if(!ctx) return;
	if(ctx->opts) {
		for(i = 0; i <= ctx->nopts; i++) {
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
	iw_free(ctx, ctx);
}

void iw_set_userdata(struct iw_context *ctx, void *u) { ctx->userdata = u; }
void *iw_get_userdata(struct iw_context *ctx) { return ctx->userdata; }
void iw_set_translate_fn(struct iw_context *ctx, iw_translatefn_type f) { ctx->xlate = f; }
void iw_set_warning_fn(struct iw_context *ctx, iw_warningfn_type f) { ctx->warn = f; }
void iw_set_max_malloc(struct iw_context *ctx, size_t n) { ctx->max_malloc = n; }

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
	if(ct >= 0 && ct < ORC_NCTYPES) ctx->req_maxcc[ct] = n;
}

/* Applies a per-channel-type setting, with the ALL / NONALPHA group codes of
 * src/imagew-api.c:391-433. */
static void orc_set_by_ctype(int *arr, int ct, int v)
{
	if(ct >= 0 && ct < ORC_NCTYPES) arr[ct] = v;
	if(ct == IW_CHANNELTYPE_ALL) arr[IW_CHANNELTYPE_ALPHA] = v;
	if(ct == IW_CHANNELTYPE_ALL || ct == IW_CHANNELTYPE_NONALPHA) {
		arr[IW_CHANNELTYPE_RED] = arr[IW_CHANNELTYPE_GREEN] = v;
		arr[IW_CHANNELTYPE_BLUE] = arr[IW_CHANNELTYPE_GRAY] = v;
	}
}

void iw_set_dither_type(struct iw_context *ctx, int ct, int f, int s)
{
	orc_set_by_ctype(ctx->dfam, ct, f);
	orc_set_by_ctype(ctx->dsub, ct, s);
}

void iw_set_color_count(struct iw_context *ctx, int ct, int c)
{
	orc_set_by_ctype(ctx->req_cc, ct, c);
}

void iw_set_channel_offset(struct iw_context *ctx, int ct, int dimension, double offs)
{
	if(ct < 0 || ct > 2) return;
	if(dimension < 0 || dimension > 1) dimension = 0;
	ctx->dim[dimension].chan_offset[ct] = offs;
}

void iw_set_input_max_color_code(struct iw_context *ctx, int ch, int c)
{
	if(ch >= 0 && ch < ORC_MAXCH) ctx->in_maxcc[ch] = c;
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

/* A gamma within 5e-6 of 1 is treated as linear (src/imagew-api.c:513-520). */
static void orc_fix_gamma(struct iw_csdescr *cs)
{
	if(cs->cstype == IW_CSTYPE_GAMMA && cs->gamma >= 0.999995 && cs->gamma <= 1.000005)
		cs->cstype = IW_CSTYPE_LINEAR;
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
	orc_fix_gamma(cs);
}

void iw_set_output_colorspace(struct iw_context *ctx, const struct iw_csdescr *cs)
{
	ctx->cs_out_req = *cs;
	orc_fix_gamma(&ctx->cs_out_req);
	ctx->cs_out_valid = 1;
}

void iw_set_input_colorspace(struct iw_context *ctx, const struct iw_csdescr *cs)
{
	ctx->cs_in = *cs;
	orc_fix_gamma(&ctx->cs_in);
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
	struct orc_dim *d;
	if(dimension < 0 || dimension > 1) dimension = 0;
	d = &ctx->dim[dimension];
	d->family = family;
	d->blur = blur;
	d->p1 = p1;
	d->p2 = p2;
}

/* Orientation change, composing with the current transform (src/imagew-api.c:651-680). */
void iw_reorient_image(struct iw_context *ctx, unsigned int x)
{
	static const unsigned int transposed[8] = {4, 6, 5, 7, 0, 2, 1, 3};
	x &= 7;
	if(x & 4) {
		int t;
		double td;
		ctx->img1.orient_transform = transposed[ctx->img1.orient_transform];
		t = ctx->img1.width; ctx->img1.width = ctx->img1.height; ctx->img1.height = t;
		td = ctx->img1.density_x; ctx->img1.density_x = ctx->img1.density_y; ctx->img1.density_y = td;
	}
	ctx->img1.orient_transform ^= (x & 3);
}

static char *orc_strdup_dbl(struct iw_context *ctx, double n)
{
	char buf[100];
	iw_snprintf(buf, sizeof(buf), "%.20f", n);
	return iw_strdup(ctx, buf);
}

void iw_set_option(struct iw_context *ctx, const char *name, const char *val)
{
	int i;
	if(!val || !val[0]) val = "1";
	if(!ctx->opts) {
		ctx->opts = iw_mallocz(ctx, 32 * sizeof(struct orc_option));
		if(!ctx->opts) return;
		ctx->nopts = 0;
	}
	for(i = 0; i < ctx->nopts; i++) {
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
	int i;
	for(i = 0; i < ctx->nopts; i++)
		if(ctx->opts[i].name && !strcmp(ctx->opts[i].name, name)) return ctx->opts[i].val;
	return NULL;
}

/* Settings that some codes only forward to iw_set_option (src/imagew-api.c:760-863).
 * The option string the reference stores leaks (it is duplicated again). */
static void orc_set_option_num(struct iw_context *ctx, const char *name, double v)
{
	iw_set_option(ctx, name, orc_strdup_dbl(ctx, v));
}

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
	case IW_VAL_JPEG_QUALITY: orc_set_option_num(ctx, "jpeg:quality", n); break;
	case IW_VAL_JPEG_SAMP_FACTOR_H: orc_set_option_num(ctx, "jpeg:sampling-x", n); break;
	case IW_VAL_JPEG_SAMP_FACTOR_V: orc_set_option_num(ctx, "jpeg:sampling-y", n); break;
	case IW_VAL_JPEG_ARITH_CODING: orc_set_option_num(ctx, "jpeg:arith", n); break;
	case IW_VAL_DEFLATE_CMPR_LEVEL: orc_set_option_num(ctx, "deflate:cmprlevel", n); break;
	case IW_VAL_OUTPUT_INTERLACED: ctx->interlaced = n; break;
	case IW_VAL_USE_BKGD_LABEL: ctx->use_file_label = n; break;
	case IW_VAL_BMP_NO_FILEHEADER: ctx->bmp_nofh = n; break;
	case IW_VAL_BMP_VERSION: orc_set_option_num(ctx, "bmp:version", n); break;
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
	if(code == IW_VAL_WEBP_QUALITY) orc_set_option_num(ctx, "webp:quality", n);
	else if(code == IW_VAL_TRANSLATE_X) ctx->dim[IW_DIMENSION_H].translate = n;
	else if(code == IW_VAL_TRANSLATE_Y) ctx->dim[IW_DIMENSION_V].translate = n;
}

double iw_get_value_dbl(struct iw_context *ctx, int code)
{
	if(code == IW_VAL_TRANSLATE_X) return ctx->dim[IW_DIMENSION_H].translate;
	if(code == IW_VAL_TRANSLATE_Y) return ctx->dim[IW_DIMENSION_V].translate;
	return 0.0;
}

/* ====================================================================== */
/* Colour transfer functions (src/imagew-main.c:28-96, :427-446)          */
/* ====================================================================== */

static double orc_to_linear(double v, const struct iw_csdescr *cs)
{
	switch(cs->cstype) {
	case IW_CSTYPE_LINEAR:
		return v;
	case IW_CSTYPE_GAMMA:
		return pow(v, cs->gamma);
	case IW_CSTYPE_REC709:
		if(v < 4.5 * 0.020) return v / 4.5;
		return pow((v + 0.099) / 1.099, 1.0 / 0.45);
	default: /* sRGB, also for unknown types */
		if(v <= 0.04045) return v / 12.92;
		return pow((v + 0.055) / (1.055), 2.4);
	}
}

static double orc_from_linear(double v, const struct iw_csdescr *cs)
{
	/* Values this close to 1 map to exactly 1. */
	if(v > 0.999999999) return 1.0;
	switch(cs->cstype) {
	case IW_CSTYPE_LINEAR:
		return v;
	case IW_CSTYPE_GAMMA:
		return pow(v, 1.0 / cs->gamma);
	case IW_CSTYPE_REC709:
		if(v < 0.020) return 4.5 * v;
		return 1.099 * pow(v, 0.45) - 0.099;
	default:
		if(v <= 0.0031308) return 12.92 * v;
		return 1.055 * pow(v, 1.0 / 2.4) - 0.055;
	}
}

double iw_convert_sample_to_linear(double v, const struct iw_csdescr *cs) { return orc_to_linear(v, cs); }
double iw_convert_sample_from_linear(double v, const struct iw_csdescr *cs) { return orc_from_linear(v, cs); }

/* ====================================================================== */
/* Resampling filters and weight lists (src/imagew-resize.c)              */
/* ====================================================================== */

enum { ORC_ROW_STD, ORC_ROW_NEAREST, ORC_ROW_NULL };

struct orc_weights {
	int kind;           /* ORC_ROW_* */
	int n_in, n_out;
	double offset;      /* used by ORC_ROW_NEAREST */
	double edge_value;  /* value of virtual (transparent-edge) pixels */
	int n;              /* number of (src,dst,w) triples */
	int *src, *dst;
	double *w;
};

struct orc_filter {
	int family;
	double radius, b, c, mix;
};

static double orc_sinc(double x)
{
	if(x <= 0.000000005) return 1.0;
	return sin(M_PI * x) / (M_PI * x);
}

/* Kernel value at distance x >= 0 (src/imagew-resize.c:62-185). */
static double orc_kernel(const struct orc_filter *f, double x)
{
	double r = f->radius;
	switch(f->family) {
	case IW_RESIZETYPE_LANCZOS:
		return x < r ? orc_sinc(x) * orc_sinc(x / r) : 0.0;
	case IW_RESIZETYPE_HANNING:
		return x < r ? orc_sinc(x) * (0.5 * cos(M_PI * x / r) + 0.5) : 0.0;
	case IW_RESIZETYPE_BLACKMAN:
		if(x >= r) return 0.0;
		return orc_sinc(x) * (0.5 * cos(M_PI * x / r) + 0.08 * cos(2.0 * M_PI * x / r) + 0.42);
	case IW_RESIZETYPE_SINC:
		return x < r ? orc_sinc(x) : 0.0;
	case IW_RESIZETYPE_GAUSSIAN: {
		double g;
		if(x >= 2.0) return 0.0;
		g = exp(-2.0 * x * x) * 0.79788456080286535587989;
		if(x <= 1.999) return g;
		return 1000.0 * (2.0 - x) * g; /* taper to zero just before 2 */
	}
	case IW_RESIZETYPE_TRIANGLE:
		return x < 1.0 ? 1.0 - x : 0.0;
	case IW_RESIZETYPE_QUADRATIC:
		if(x < 0.5) return 0.75 - x * x;
		if(x < 1.5) return 0.50 * (x - 1.5) * (x - 1.5);
		return 0.0;
	case IW_RESIZETYPE_CUBIC: {
		double b = f->b, c = f->c;
		if(x < 1.0)
			return ((12.0 - 9.0 * b - 6.0 * c) * x * x * x + (-18.0 + 12.0 * b + 6.0 * c) * x * x + (6.0 - 2.0 * b)) / 6.0;
		if(x < 2.0)
			return ((-b - 6.0 * c) * x * x * x + (6.0 * b + 30.0 * c) * x * x + (-12.0 * b - 48.0 * c) * x + (8.0 * b + 24.0 * c)) / 6.0;
		return 0.0;
	}
	case IW_RESIZETYPE_HERMITE:
		return x < 1.0 ? 2.0 * x * x * x - 3.0 * x * x + 1.0 : 0.0;
	case IW_RESIZETYPE_BOX:
		return x <= 0.5 ? 1.0 : 0.0;
	case IW_RESIZETYPE_BOXAVG:
		if(x < 0.4999999) return 1.0;
		return x <= 0.5000001 ? 0.5 : 0.0;
	case IW_RESIZETYPE_MIX:
		if(x < (0.5 - f->mix / 2.0)) return 1.0;
		if(x < (0.5 + f->mix / 2.0)) return 0.5 - (x - 0.5) / f->mix;
		return 0.0;
	}
	return 0.0;
}

static void orc_weights_free(struct iw_context *ctx, struct orc_weights *wt)
{
	iw_free(ctx, wt->src);
	iw_free(ctx, wt->dst);
	iw_free(ctx, wt->w);
	memset(wt, 0, sizeof(*wt));
}

/* Builds the weight list for one dimension and one channel type
 * (iwpvt_resize_rows_init + iw_create_weightlist_std, src/imagew-resize.c:240-556).
 * Returns 0 on error. */
static int orc_weights_build(struct iw_context *ctx, struct orc_weights *wt, const struct orc_dim *d,
	int ctype, int n_in, int n_out, double edge_bkgd_value)
{
	struct orc_filter f;
	int standard = 1, boxhack = 0, sincfam = 0;
	double rf, est;
	int cap, o;

	memset(wt, 0, sizeof(*wt));
	memset(&f, 0, sizeof(f));
	wt->n_in = n_in;
	wt->n_out = n_out;
	wt->kind = ORC_ROW_STD;
	f.family = d->family;

	switch(d->family) {
	case IW_RESIZETYPE_NULL: wt->kind = ORC_ROW_NULL; standard = 0; break;
	case IW_RESIZETYPE_NEAREST: wt->kind = ORC_ROW_NEAREST; standard = 0; boxhack = 1; break;
	case IW_RESIZETYPE_MIX:
		f.mix = ((double)n_out) / n_in;
		if(f.mix > 1.0) f.mix = 1.0 / f.mix;
		f.radius = 0.5 + f.mix;
		break;
	case IW_RESIZETYPE_BOX: f.radius = 0.501; boxhack = 1; break;
	case IW_RESIZETYPE_BOXAVG: f.radius = 0.501; break;
	case IW_RESIZETYPE_TRIANGLE: f.radius = 1.0; break;
	case IW_RESIZETYPE_QUADRATIC: f.radius = 1.5; break;
	case IW_RESIZETYPE_GAUSSIAN: f.radius = 2.0; break;
	case IW_RESIZETYPE_HERMITE: f.radius = 1.0; break;
	case IW_RESIZETYPE_CUBIC:
		f.radius = 2.0;
		f.b = d->p1 < -100.0 ? -100.0 : (d->p1 > 100.0 ? 100.0 : d->p1);
		f.c = d->p2 < -100.0 ? -100.0 : (d->p2 > 100.0 ? 100.0 : d->p2);
		break;
	case IW_RESIZETYPE_LANCZOS: case IW_RESIZETYPE_HANNING:
	case IW_RESIZETYPE_BLACKMAN: case IW_RESIZETYPE_SINC:
		sincfam = 1;
		break;
	default:
		iw_set_error(ctx, "Internal: Unknown resize algorithm");
		return 0;
	}
	if(sincfam) {
		f.radius = floor(d->p1 + 0.5);
		if(f.radius < 2.0) f.radius = 2.0;
		if(f.radius > 100.0) f.radius = 100.0;
	}

	wt->edge_value = 0.0;
	if(d->edge == IW_EDGE_POLICY_TRANSPARENT) wt->edge_value = edge_bkgd_value;

	wt->offset = d->translate;
	if(boxhack) wt->offset -= 0.00000000001;
	if(d->use_offset && ctype >= 0 && ctype <= 2) wt->offset += d->chan_offset[ctype];

	if(!standard) return 1;

	{
		double blur = d->blur;
		if(blur < 0.0001) blur = 0.0001;
		if(blur > 10000.0) blur = 10000.0;
		rf = (d->true_size < (double)n_in) ? ((double)n_in) / d->true_size : 1.0;
		rf *= blur;
	}

	/* The reference sizes its first allocation from this estimate. */
	est = 2.0 * f.radius * rf * n_out;
	if(((size_t)(int)est + 32) * 16 > ctx->max_malloc) {
		iw_set_error(ctx, "Out of memory");
		return 0;
	}
	cap = (int)est + 32;
	if(cap < 64) cap = 64;
	wt->src = iw_malloc(ctx, sizeof(int) * (size_t)cap);
	wt->dst = iw_malloc(ctx, sizeof(int) * (size_t)cap);
	wt->w = iw_malloc(ctx, sizeof(double) * (size_t)cap);
	if(!wt->src || !wt->dst || !wt->w) return 0;

	for(o = 0; o < n_out; o++) {
		double center = (0.5 + (double)o - wt->offset) / d->true_size;
		double pos = center * (double)n_in - 0.5;
		int first = (int)ceil(pos - f.radius * rf - 0.0001);
		int last = (int)floor(pos + f.radius * rf + 0.0001);
		int start = wt->n, count = 0, ip, k;
		double sum = 0.0;

		for(ip = first; ip <= last; ip++) {
			double x, v;
			int src;
			if(d->edge == IW_EDGE_POLICY_STANDARD && (ip < 0 || ip >= n_in)) continue;
			x = (((double)ip) - pos) / rf;
			v = orc_kernel(&f, x < 0 ? -x : x);
			if(v == 0.0) continue;
			sum += v;
			count++;
			if(ip < 0 || ip > n_in - 1) {
				if(d->edge == IW_EDGE_POLICY_TRANSPARENT) src = -1;
				else src = ip < 0 ? 0 : n_in - 1;
			}
			else src = ip;
			if(wt->n >= cap) {
				int ncap = cap * 2;
				wt->src = iw_realloc(ctx, wt->src, sizeof(int) * (size_t)cap, sizeof(int) * (size_t)ncap);
				wt->dst = iw_realloc(ctx, wt->dst, sizeof(int) * (size_t)cap, sizeof(int) * (size_t)ncap);
				wt->w = iw_realloc(ctx, wt->w, sizeof(double) * (size_t)cap, sizeof(double) * (size_t)ncap);
				if(!wt->src || !wt->dst || !wt->w) return 0;
				cap = ncap;
			}
			wt->src[wt->n] = src;
			wt->dst[wt->n] = o;
			wt->w[wt->n] = v;
			wt->n++;
		}
		if(count > 0) {
			for(k = start; k < wt->n; k++) wt->w[k] = (sum != 0.0) ? wt->w[k] / sum : 0.0;
		}
	}
	return 1;
}

/* Resamples one line (src/imagew-resize.c:346-410). */
static void orc_resample(const struct orc_weights *wt, const double *in, double *out)
{
	int i;
	if(wt->kind == ORC_ROW_NULL) {
		for(i = 0; i < wt->n_out; i++) out[i] = i < wt->n_in ? in[i] : 0.0;
		return;
	}
	if(wt->kind == ORC_ROW_NEAREST) {
		for(i = 0; i < wt->n_out; i++) {
			double c = (0.5 + (double)i - wt->offset) / (double)wt->n_out;
			int p = (int)floor(c * (double)wt->n_in);
			if(p < 0) p = 0;
			if(p > wt->n_in - 1) p = wt->n_in - 1;
			out[i] = in[p];
		}
		return;
	}
	for(i = 0; i < wt->n_out; i++) out[i] = 0.0;
	for(i = 0; i < wt->n; i++) {
		double s = wt->src[i] >= 0 ? in[wt->src[i]] : wt->edge_value;
		out[wt->dst[i]] += s * wt->w[i];
	}
}

/* ====================================================================== */
/* Planning (src/imagew-main.c:1463-2248)                                 */
/* ====================================================================== */

enum { BK_EARLY = 1, BK_LATE = 2 };
enum { BKSRC_NONE = 0, BKSRC_FILE = 1, BKSRC_REQ = 2 };

struct orc_midch {       /* one intermediate channel */
	int ctype;
	int in_ch;           /* first input channel read */
	int to_gray;         /* combine in_ch..in_ch+2 into gray */
	int out_ch;          /* output channel, -1 if dropped */
	double bk_early;     /* background for early compositing (linear) */
	int unassoc;         /* colour channel of an image with alpha */
};

struct orc_outch {
	int ctype, dfam, dsub, cc, maxcc;
	double maxcc_d;
	double bk1, bk2;     /* late background colours (linear) */
};

struct orc_plan {
	int in_nphys, in_nlog, in_logtype, in_alpha;
	int in_maxcc[ORC_MAXCH];
	double in_maxcc_d[ORC_MAXCH];
	int in_slow[ORC_MAXCH];      /* per-sample path without the input table */
	int in_max; double in_max_d;
	int reduced_in;
	double *in_tab;              /* input code -> linear, or NULL */
	int crop_x, crop_y, crop_w, crop_h;

	int mid_type, mid_n, mid_alpha;
	struct orc_midch mid[ORC_MAXCH];

	int out_n;
	struct orc_outch out[ORC_MAXCH];
	int no_out_tables;
	int errdiff;

	int apply_bk, bk_strategy, bk_checker, bk_source;
	double bk1_alpha, bk2_alpha;
	struct iw_color inlabel_lin;
};

static int orc_ctype_of(int imgtype, int ch)
{
	switch(imgtype) {
	case IW_IMGTYPE_GRAY: return ch == 0 ? IW_CHANNELTYPE_GRAY : 0;
	case IW_IMGTYPE_GRAYA: return ch == 0 ? IW_CHANNELTYPE_GRAY : (ch == 1 ? IW_CHANNELTYPE_ALPHA : 0);
	case IW_IMGTYPE_RGB: return ch <= 2 ? ch : 0;
	case IW_IMGTYPE_RGBA: return ch <= 3 ? ch : 0;
	}
	return 0;
}

static double orc_gray_of(const struct iw_context *ctx, double r, double g, double b)
{
	if(ctx->gsf == IW_GSF_WEIGHTED)
		return ctx->gsw[0] * r + ctx->gsw[1] * g + ctx->gsw[2] * b;
	if(ctx->gsf == IW_GSF_ORDERBYVALUE) {
		/* weights applied to the values sorted from largest to smallest */
		double hi, mid, lo;
		if(g <= r) { hi = r; mid = g; } else { hi = g; mid = r; }
		if(b <= mid) lo = b;
		else {
			lo = mid;
			if(b <= hi) mid = b;
			else { mid = hi; hi = b; }
		}
		return ctx->gsw[0] * hi + ctx->gsw[1] * mid + ctx->gsw[2] * lo;
	}
	return 0.0;
}

static int orc_bkgd_has_trns(const struct iw_context *ctx, const struct orc_plan *P)
{
	if(!P->apply_bk) return 0;
	if(!(ctx->profile & IW_PROFILE_TRANSPARENCY)) return 0;
	if(P->bk_strategy == BK_EARLY) return 0;
	if(P->bk_source == BKSRC_FILE) return ctx->inlabel.c[3] < 1.0;
	if(P->bk_source == BKSRC_REQ) {
		if(P->bk_checker && ctx->bkgd2.c[3] < 1.0) return 1;
		return ctx->bkgd.c[3] < 1.0;
	}
	return 0;
}

/* Decides whether/when to composite a background (src/imagew-main.c:1734-1823). */
static void orc_decide_bkgd(struct iw_context *ctx, struct orc_plan *P)
{
	if(!IW_IMGTYPE_HAS_ALPHA(P->in_logtype)) {
		P->apply_bk = 0;
		return;
	}
	if(ctx->inlabel_set && (ctx->use_file_label || !ctx->bkgd_valid)) P->bk_source = BKSRC_FILE;
	else if(ctx->bkgd_valid) {
		P->bk_source = BKSRC_REQ;
		P->bk_checker = ctx->bkgd_checker;
	}
	else P->bk_source = BKSRC_NONE;

	if(P->bk_checker && ctx->check_size < 1) ctx->check_size = 1;
	if(ctx->bkgd_valid) P->apply_bk = 1;

	if(!(ctx->profile & IW_PROFILE_TRANSPARENCY)) {
		if(!ctx->bkgd_valid && !P->apply_bk)
			iw_warning(ctx, "This image may have transparency, which is incompatible with the output format. A background color will be applied.");
		P->apply_bk = 1;
	}

	if(ctx->dim[0].use_offset || ctx->dim[1].use_offset) {
		if(!ctx->bkgd_valid && !P->apply_bk)
			iw_warning(ctx, "This image may have transparency, which is incompatible with a channel offset. A background color will be applied.");
		P->apply_bk = 1;
		if(P->bk_checker && ctx->bkgd_checker) {
			iw_warning(ctx, "Checkerboard backgrounds are not supported when using a channel offset.");
			P->bk_checker = 0;
		}
		P->bk_strategy = BK_EARLY;
		return;
	}
	if(!P->apply_bk) return;
	P->bk_strategy = BK_LATE;
}

/* Channel-layout strategy codes: 0xSIO with S=stage, I=input type, O=output
 * type, where 1=G, 2=GA, 3=RGB, 4=RGBA (src/imagew-main.c:1613-1631). */
#define ST(i, o) (((i) << 4) | (o))

static void orc_decide_strategy(struct iw_context *ctx, struct orc_plan *P, int *s1, int *s2)
{
	int in;
	switch(P->in_logtype) {
	case IW_IMGTYPE_RGBA: in = 4; break;
	case IW_IMGTYPE_RGB: in = 3; break;
	case IW_IMGTYPE_GRAYA: in = 2; break;
	default: in = 1; break;
	}
	if(ctx->to_gray) {
		*s1 = ST(in, (in == 2 || in == 4) ? 2 : 1);
		*s2 = (in == 2 || in == 4) ? ST(2, 2) : ST(1, 1);
	}
	else {
		*s1 = ST(in, (in == 2 || in == 4) ? 4 : 3);
		*s2 = (in == 2 || in == 4) ? ST(4, 4) : ST(3, 3);
	}

	if(P->apply_bk && P->bk_strategy == BK_EARLY) {
		if(*s1 == ST(4, 4)) { *s1 = ST(4, 3); *s2 = ST(3, 3); }
		else if(*s1 == ST(2, 2)) { *s1 = ST(2, 1); *s2 = ST(1, 1); }
		else if(*s1 == ST(2, 4)) { *s1 = ST(2, 3); *s2 = ST(3, 3); }
		else if(*s1 == ST(4, 2)) { *s1 = ST(4, 1); *s2 = ST(1, 1); }
	}
	if(P->apply_bk && !orc_bkgd_has_trns(ctx, P)) {
		if(*s2 == ST(2, 2)) *s2 = ST(2, 1);
		else if(*s2 == ST(4, 4)) *s2 = ST(4, 3);
	}
}

static void orc_prepare_bkgd(struct iw_context *ctx, struct orc_plan *P, int out_type)
{
	struct iw_color b1 = {{1.0, 0.0, 1.0, 1.0}}, b2 = {{0.0, 0.0, 0.0, 1.0}};
	int i;
	if(P->bk_source == BKSRC_FILE) {
		b1 = P->inlabel_lin;
		P->bk_checker = 0;
	}
	else if(P->bk_source == BKSRC_REQ) {
		b1 = ctx->bkgd;
		if(ctx->bkgd_checker) b2 = ctx->bkgd2;
	}
	if(P->bk_strategy == BK_EARLY) P->bk1_alpha = 1.0;
	else {
		P->bk1_alpha = b1.c[3];
		P->bk2_alpha = b2.c[3];
	}
	if(P->bk_strategy == BK_LATE && (out_type == IW_IMGTYPE_RGB || out_type == IW_IMGTYPE_RGBA)) {
		for(i = 0; i < 3; i++) {
			P->out[i].bk1 = b1.c[i];
			if(P->bk_checker) P->out[i].bk2 = b2.c[i];
		}
	}
	else if(P->bk_strategy == BK_LATE && (out_type == IW_IMGTYPE_GRAY || out_type == IW_IMGTYPE_GRAYA)) {
		P->out[0].bk1 = orc_gray_of(ctx, b1.c[0], b1.c[1], b1.c[2]);
		if(P->bk_checker) P->out[0].bk2 = orc_gray_of(ctx, b2.c[0], b2.c[1], b2.c[2]);
	}
	else if(P->bk_strategy == BK_EARLY && out_type == IW_IMGTYPE_RGB) {
		for(i = 0; i < 3; i++) P->mid[i].bk_early = b1.c[i];
	}
	else if(P->bk_strategy == BK_EARLY && out_type == IW_IMGTYPE_GRAY) {
		P->mid[0].bk_early = orc_gray_of(ctx, b1.c[0], b1.c[1], b1.c[2]);
	}
}

/* Table of linear values for every code of an 8-bit-or-less image, when the
 * reference builds one (src/imagew-main.c:1172-1195).  Table and per-sample
 * conversion give identical values; the table matters because the reference
 * only uses it in the "fast" sample path. */
static double *orc_make_lin_table(struct iw_context *ctx, const struct iw_image *img, const struct iw_csdescr *cs)
{
	int n, i;
	double *t;
	if(cs->cstype == IW_CSTYPE_LINEAR) return NULL;
	if(img->bit_depth > 16) return NULL; /* float output: never consulted */
	n = 1 << img->bit_depth;
	if(n > 256) return NULL;
	if(((size_t)img->width) * img->height <= 512) return NULL;
	t = iw_malloc(ctx, n * sizeof(double));
	if(!t) return NULL;
	for(i = 0; i < n; i++) t[i] = orc_to_linear(((double)i) / (n - 1), cs);
	return t;
}

static void orc_set_auto_family(struct iw_context *ctx, int n_in, int n_out, int dim)
{
	if(n_out == n_in && !ctx->dim[dim].use_offset && !ctx->true_valid && ctx->dim[dim].translate == 0.0)
		iw_set_resize_alg(ctx, dim, IW_RESIZETYPE_NULL, 1.0, 0.0, 0.0);
	else
		iw_set_resize_alg(ctx, dim, IW_RESIZETYPE_CUBIC, 1.0, 0.0, 0.5); /* Catmull-Rom */
}

static int orc_prepare(struct iw_context *ctx, struct orc_plan *P)
{
	int w = ctx->canvas_w, h = ctx->canvas_h;
	int i, j, s1, s2, out_max = 0;

	memset(P, 0, sizeof(*P));
	if(!ctx->profile) {
		iw_set_error(ctx, "Output profile not set");
		return 0;
	}
	if(ctx->randomize) ctx->seed = (int)time(NULL);

	ctx->dim[0].true_size = ctx->true_valid ? ctx->true_w : (double)w;
	ctx->dim[1].true_size = ctx->true_valid ? ctx->true_h : (double)h;

	if(!iw_check_image_dimensions(ctx, ctx->img1.width, ctx->img1.height)) return 0;
	if(!iw_check_image_dimensions(ctx, w, h)) return 0;

	if(ctx->to_gray) {
		if(ctx->gsf == IW_GSF_STANDARD) {
			ctx->gsf = IW_GSF_WEIGHTED;
			iw_set_grayscale_weights(ctx, 0.212655, 0.715158, 0.072187);
		}
		else if(ctx->gsf == IW_GSF_COMPATIBLE) {
			ctx->gsf = IW_GSF_WEIGHTED;
			iw_set_grayscale_weights(ctx, 0.299, 0.587, 0.114);
		}
	}

	/* Logical input type: a transparent edge adds a virtual alpha channel. */
	P->in_logtype = ctx->img1.imgtype;
	if(ctx->dim[0].edge == IW_EDGE_POLICY_TRANSPARENT || ctx->dim[1].edge == IW_EDGE_POLICY_TRANSPARENT) {
		if(ctx->img1.imgtype == IW_IMGTYPE_GRAY) P->in_logtype = IW_IMGTYPE_GRAYA;
		else if(ctx->img1.imgtype == IW_IMGTYPE_RGB) P->in_logtype = IW_IMGTYPE_RGBA;
	}
	P->in_nphys = iw_imgtype_num_channels(ctx->img1.imgtype);
	P->in_nlog = iw_imgtype_num_channels(P->in_logtype);
	P->in_alpha = orc_alpha_index(P->in_logtype);
	for(i = 0; i < P->in_nlog; i++) {
		P->mid[i].ctype = orc_ctype_of(P->in_logtype, i);
		P->mid[i].in_ch = i;
		if(i >= P->in_nphys) P->in_slow[i] = 1;
	}
	ctx->img2.width = w;
	ctx->img2.height = h;

	/* Crop rectangle, clamped as the reference does (including its use of
	 * the x origin when the y origin is past the bottom). */
	P->crop_x = ctx->crop_x; P->crop_y = ctx->crop_y;
	P->crop_w = ctx->crop_w; P->crop_h = ctx->crop_h;
	if(P->crop_x < 0) P->crop_x = 0;
	if(P->crop_y < 0) P->crop_y = 0;
	if(P->crop_x > ctx->img1.width - 1) P->crop_x = ctx->img1.width - 1;
	if(P->crop_y > ctx->img1.height - 1) P->crop_x = ctx->img1.height - 1;
	if(P->crop_w < 0) P->crop_w = ctx->img1.width - P->crop_x;
	if(P->crop_h < 0) P->crop_h = ctx->img1.height - P->crop_y;
	if(P->crop_w < 1) P->crop_w = 1;
	if(P->crop_h < 1) P->crop_h = 1;
	if(P->crop_w > ctx->img1.width - P->crop_x) P->crop_w = ctx->img1.width - P->crop_x;
	if(P->crop_h > ctx->img1.height - P->crop_y) P->crop_h = ctx->img1.height - P->crop_y;
	/* The reference writes the clamped crop back into its settings. */
	ctx->crop_x = P->crop_x; ctx->crop_y = P->crop_y;
	ctx->crop_w = P->crop_w; ctx->crop_h = P->crop_h;

	/* Output colour space. */
	if(ctx->cs_out_valid) {
		ctx->cs_out = ctx->cs_out_req;
		if((ctx->profile & IW_PROFILE_ALWAYSLINEAR) && ctx->cs_out.cstype != IW_CSTYPE_LINEAR) {
			iw_warning(ctx, "Forcing output colorspace to linear; required by the output format.");
			iw_make_linear_csdescr(&ctx->cs_out);
		}
	}
	else if(ctx->profile & IW_PROFILE_ALWAYSLINEAR) iw_make_linear_csdescr(&ctx->cs_out);
	else iw_make_srgb_csdescr_2(&ctx->cs_out);

	/* Input max colour codes. */
	if(ctx->img1.sampletype != IW_SAMPLETYPE_FLOATINGPOINT) {
		P->in_max = (1 << ctx->img1.bit_depth) - 1;
		P->in_max_d = (double)P->in_max;
		for(i = 0; i < ORC_MAXCH; i++) {
			if(ctx->in_maxcc[i] <= 0) ctx->in_maxcc[i] = P->in_max;
			P->in_maxcc[i] = ctx->in_maxcc[i];
			P->in_maxcc_d[i] = (double)ctx->in_maxcc[i];
			if(ctx->in_maxcc[i] != P->in_max) P->reduced_in = 1;
		}
	}
	if(P->reduced_in || ctx->img1.sampletype == IW_SAMPLETYPE_FLOATINGPOINT)
		for(i = 0; i < P->in_nphys; i++) P->in_slow[i] = 1;

	for(i = 0; i < 2; i++)
		for(j = 0; j < 3; j++)
			if(fabs(ctx->dim[i].chan_offset[j]) > 0.00001) ctx->dim[i].use_offset = 1;
	if(ctx->to_gray && (ctx->dim[0].use_offset || ctx->dim[1].use_offset)) {
		iw_warning(ctx, "Disabling channel offset, due to grayscale output.");
		ctx->dim[0].use_offset = ctx->dim[1].use_offset = 0;
	}

	orc_decide_bkgd(ctx, P);

	for(i = 0; i < 2; i++) {
		if(ctx->dim[i].use_offset ||
			(P->apply_bk && P->bk_strategy == BK_EARLY && ctx->dim[i].edge == IW_EDGE_POLICY_TRANSPARENT))
			ctx->dim[i].no_cache = 1;
	}

	orc_decide_strategy(ctx, P, &s1, &s2);

	switch(s1) {
	case ST(4, 4): P->mid_type = IW_IMGTYPE_RGBA; break;
	case ST(2, 4):
		P->mid_type = IW_IMGTYPE_RGBA;
		P->mid[0].in_ch = P->mid[1].in_ch = P->mid[2].in_ch = 0;
		P->mid[3].in_ch = 1;
		break;
	case ST(3, 3): case ST(4, 3): P->mid_type = IW_IMGTYPE_RGB; break;
	case ST(1, 3): case ST(2, 3):
		P->mid_type = IW_IMGTYPE_RGB;
		P->mid[0].in_ch = P->mid[1].in_ch = P->mid[2].in_ch = 0;
		break;
	case ST(4, 2):
		P->mid_type = IW_IMGTYPE_GRAYA;
		P->mid[0].to_gray = 1;
		P->mid[0].in_ch = 0;
		P->mid[1].in_ch = 3;
		break;
	case ST(2, 2): P->mid_type = IW_IMGTYPE_GRAYA; break;
	case ST(3, 1):
		P->mid_type = IW_IMGTYPE_GRAY;
		P->mid[0].to_gray = 1;
		P->mid[0].in_ch = 0;
		break;
	case ST(1, 1): P->mid_type = IW_IMGTYPE_GRAY; P->mid[0].in_ch = 0; break;
	default: /* includes GA->G and RGBA->G, which the reference also rejects */
		iw_set_errorf(ctx, "Internal error, unknown strategy %d", s1);
		return 0;
	}
	P->mid_n = iw_imgtype_num_channels(P->mid_type);
	P->mid_alpha = orc_alpha_index(P->mid_type);
	for(i = 0; i < P->mid_n; i++) P->mid[i].out_ch = i;

	switch(s2) {
	case ST(4, 4): ctx->img2.imgtype = IW_IMGTYPE_RGBA; break;
	case ST(3, 3): ctx->img2.imgtype = IW_IMGTYPE_RGB; break;
	case ST(4, 3): ctx->img2.imgtype = IW_IMGTYPE_RGB; P->mid[3].out_ch = -1; break;
	case ST(2, 2): ctx->img2.imgtype = IW_IMGTYPE_GRAYA; break;
	case ST(1, 1): ctx->img2.imgtype = IW_IMGTYPE_GRAY; break;
	case ST(2, 1): ctx->img2.imgtype = IW_IMGTYPE_GRAY; P->mid[1].out_ch = -1; break;
	default:
		iw_set_error(ctx, "Internal error");
		return 0;
	}
	P->out_n = iw_imgtype_num_channels(ctx->img2.imgtype);
	for(i = 0; i < P->mid_n; i++) P->mid[i].ctype = orc_ctype_of(P->mid_type, i);
	for(i = 0; i < P->out_n; i++) P->out[i].ctype = orc_ctype_of(ctx->img2.imgtype, i);
	if(IW_IMGTYPE_HAS_ALPHA(P->mid_type))
		for(i = 0; i < P->mid_n; i++)
			if(P->mid[i].ctype != IW_CHANNELTYPE_ALPHA) P->mid[i].unassoc = 1;

	/* Output sample type and depth (src/imagew-main.c:1514-1541). */
	if(ctx->profile & IW_PROFILE_HDRI) {
		ctx->img2.sampletype = IW_SAMPLETYPE_FLOATINGPOINT;
		ctx->img2.bit_depth = 32;
	}
	else {
		ctx->img2.sampletype = IW_SAMPLETYPE_UINT;
		if(ctx->req_depth > 8 && (ctx->profile & IW_PROFILE_16BPS)) ctx->img2.bit_depth = 16;
		else {
			if(ctx->req_depth > 8) iw_warning(ctx, "Reducing depth to 8; required by the output format.");
			ctx->img2.bit_depth = 8;
		}
	}

	if(ctx->img2.sampletype == IW_SAMPLETYPE_FLOATINGPOINT) {
		int any = 0;
		for(i = 0; i < ORC_NCTYPES; i++) if(ctx->req_cc[i]) any = 1;
		if(any) iw_warning(ctx, "Posterization is not supported with floating point output.");
	}
	else {
		out_max = (1 << ctx->img2.bit_depth) - 1;
		for(i = 0; i < P->out_n; i++) P->out[i].maxcc = out_max;
		if(ctx->profile & IW_PROFILE_REDUCEDBITDEPTHS) {
			for(i = 0; i < P->out_n; i++) {
				int m = ctx->req_maxcc[P->out[i].ctype];
				if(m > 0) P->out[i].maxcc = m > out_max ? out_max : m;
			}
		}
		for(i = 0; i < P->out_n; i++) {
			if(P->out[i].maxcc != out_max) {
				ctx->reduced_out = 1;
				P->no_out_tables = 1;
			}
			P->out[i].maxcc_d = (double)P->out[i].maxcc;
		}
	}
	for(i = 0; i < P->out_n; i++) {
		struct orc_outch *o = &P->out[i];
		o->cc = ctx->req_cc[o->ctype];
		if(o->cc) {
			if(o->cc < 2) o->cc = 2;
			else if(o->cc > o->maxcc) o->cc = o->maxcc;
		}
		if(o->cc == 1 + o->maxcc) o->cc = 0;
		o->dfam = ctx->dfam[o->ctype];
		o->dsub = ctx->dsub[o->ctype];
		if(o->dfam == IW_DITHERFAMILY_ERRDIFF) P->errdiff = 1;
		ctx->out_maxcc[i] = o->maxcc;
	}

	if(!P->reduced_in && ctx->img1.sampletype == IW_SAMPLETYPE_UINT)
		P->in_tab = orc_make_lin_table(ctx, &ctx->img1, &ctx->cs_in);

	if(ctx->inlabel_set) {
		for(i = 0; i < 3; i++) P->inlabel_lin.c[i] = orc_to_linear(ctx->inlabel.c[i], &ctx->cs_in);
		P->inlabel_lin.c[3] = ctx->inlabel.c[3];
	}
	if(P->apply_bk) orc_prepare_bkgd(ctx, P, ctx->img2.imgtype);

	ctx->img2.rendering_intent = ctx->req_intent == IW_INTENT_UNKNOWN ? ctx->img1.rendering_intent : ctx->req_intent;

	if(ctx->dim[0].family == IW_RESIZETYPE_AUTO) orc_set_auto_family(ctx, P->crop_w, ctx->img2.width, 0);
	if(ctx->dim[1].family == IW_RESIZETYPE_AUTO) orc_set_auto_family(ctx, P->crop_h, ctx->img2.height, 1);

	if(IW_IMGTYPE_HAS_ALPHA(ctx->img2.imgtype) && !ctx->opt_strip) {
		ctx->opt_pal = 0;
		ctx->opt_bintrns = 0;
	}
	return 1;
}
#undef ST

/* ====================================================================== */
/* Reading input samples (src/imagew-main.c:129-383)                      */
/* ====================================================================== */

/* Logical (x,y) of the crop-relative image -> physical pixel coordinates. */
static void orc_phys_xy(const struct iw_context *ctx, const struct orc_plan *P, int x, int y, int *px, int *py)
{
	int lx = P->crop_x + x, ly = P->crop_y + y;
	int W = ctx->img1.width, H = ctx->img1.height;
	switch(ctx->img1.orient_transform) {
	case 0: *px = lx; *py = ly; break;
	case 1: *px = W - 1 - lx; *py = ly; break;
	case 2: *px = lx; *py = H - 1 - ly; break;
	case 3: *px = W - 1 - lx; *py = H - 1 - ly; break;
	case 4: *px = ly; *py = lx; break;
	case 5: *px = ly; *py = W - 1 - lx; break;
	case 6: *px = H - 1 - ly; *py = lx; break;
	case 7: *px = H - 1 - ly; *py = W - 1 - lx; break;
	default: *px = 0; *py = 0; break;
	}
}

static unsigned int orc_raw_int(const struct iw_context *ctx, const struct orc_plan *P, int x, int y, int ch)
{
	int px, py;
	const iw_byte *row;
	orc_phys_xy(ctx, P, x, y, &px, &py);
	row = ctx->img1.pixels + (size_t)py * ctx->img1.bpr;
	switch(ctx->img1.bit_depth) {
	case 8: return row[P->in_nphys * px + ch];
	case 16: {
		const iw_byte *p = row + (size_t)(P->in_nphys * px + ch) * 2;
		return ((unsigned int)p[0] << 8) | p[1];
	}
	case 4: return (px & 1) ? (row[px / 2] & 0x0f) : (row[px / 2] >> 4);
	case 2: return (row[px / 4] >> ((3 - px % 4) * 2)) & 0x03;
	case 1: return (row[px / 8] & (1 << (7 - px % 8))) ? 1 : 0;
	}
	return 0;
}

/* Sample value in [0,1] before any colour conversion (get_raw_sample). */
static double orc_raw(const struct iw_context *ctx, const struct orc_plan *P, int x, int y, int ch)
{
	if(ch >= P->in_nphys) return 1.0; /* virtual alpha: opaque */
	if(ctx->img1.sampletype == IW_SAMPLETYPE_FLOATINGPOINT) {
		int px, py;
		float f;
		orc_phys_xy(ctx, P, x, y, &px, &py);
		if(ctx->img1.bit_depth != 32) return 0.0;
		memcpy(&f, ctx->img1.pixels + (size_t)py * ctx->img1.bpr + (size_t)(P->in_nphys * px + ch) * 4, 4);
		return (double)f;
	}
	return ((double)orc_raw_int(ctx, P, x, y, ch)) / P->in_maxcc_d[ch];
}

static double orc_int_to_linear(const struct orc_plan *P, unsigned int v, const struct iw_csdescr *cs)
{
	if(cs->cstype == IW_CSTYPE_LINEAR) return ((double)v) / P->in_max_d;
	if(P->in_tab) return P->in_tab[v];
	return orc_to_linear(((double)v) / P->in_max_d, cs);
}

/* Linear-light value of intermediate channel m at (x,y) (get_sample_cvt_to_linear). */
static double orc_sample_linear(const struct iw_context *ctx, const struct orc_plan *P, int x, int y,
	int m, const struct iw_csdescr *cs)
{
	const struct orc_midch *mc = &P->mid[m];
	int ch = mc->in_ch;
	if(P->in_slow[ch]) {
		if(mc->to_gray) {
			double r = orc_to_linear(orc_raw(ctx, P, x, y, ch + 0), cs);
			double g = orc_to_linear(orc_raw(ctx, P, x, y, ch + 1), cs);
			double b = orc_to_linear(orc_raw(ctx, P, x, y, ch + 2), cs);
			return orc_gray_of(ctx, r, g, b);
		}
		return orc_to_linear(orc_raw(ctx, P, x, y, ch), cs);
	}
	if(mc->to_gray) {
		double r = orc_int_to_linear(P, orc_raw_int(ctx, P, x, y, ch + 0), cs);
		double g = orc_int_to_linear(P, orc_raw_int(ctx, P, x, y, ch + 1), cs);
		double b = orc_int_to_linear(P, orc_raw_int(ctx, P, x, y, ch + 2), cs);
		return orc_gray_of(ctx, r, g, b);
	}
	return orc_int_to_linear(P, orc_raw_int(ctx, P, x, y, ch), cs);
}

/* ====================================================================== */
/* Output quantisation (src/imagew-main.c:457-765)                        */
/* ====================================================================== */

/* 8x8 threshold ranks: dispersed (Bayer) and clustered "halftone" patterns;
 * the threshold of rank r is (r + 0.5)/64 (src/imagew-main.c:461-483). */
static const unsigned char orc_dither_rank[2][64] = {
	{ 0,48,12,60, 3,51,15,63, 32,16,44,28,35,19,47,31,  8,56, 4,52,11,59, 7,55, 40,24,36,20,43,27,39,23,
	  2,50,14,62, 1,49,13,61, 34,18,46,30,33,17,45,29, 10,58, 6,54, 9,57, 5,53, 42,26,38,22,41,25,37,21 },
	{ 3, 9,17,27,25,15, 7, 1, 11,29,37,45,43,35,23, 5, 19,39,51,57,55,49,33,13, 31,47,59,63,61,53,41,21,
	 30,46,58,62,60,52,40,20, 18,38,50,56,54,48,32,12, 10,28,36,44,42,34,22, 4,  2, 8,16,26,24,14, 6, 0 }
};

/* Error-diffusion kernels as numerator/denominator.  Positions:
 *        x  0  1
 *  2  3  4  5  6
 *  7  8  9 10 11        (src/imagew-main.c:505-535) */
static const signed char orc_ed_num[8][12] = {
	{7,0, 0,3,5,1,0, 0,0,0,0,0},
	{7,5, 3,5,7,5,3, 1,3,5,3,1},
	{8,4, 2,4,8,4,2, 1,2,4,2,1},
	{8,4, 2,4,8,4,2, 0,0,0,0,0},
	{5,3, 2,4,5,4,2, 0,2,3,2,0},
	{4,3, 1,2,3,2,1, 0,0,0,0,0},
	{2,0, 0,1,1,0,0, 0,0,0,0,0},
	{1,1, 0,1,1,1,0, 0,0,1,0,0}
};
static const double orc_ed_den[8] = {16.0, 48.0, 42.0, 32.0, 32.0, 16.0, 4.0, 8.0};

struct orc_tail {
	const struct iw_csdescr *cs;
	double *rev;        /* output code -> linear for 8-bit output, or NULL */
	double *nc;         /* nearest-colour midpoints, or NULL */
	double *err[3];     /* error-diffusion rows; 0 = current row */
	struct { unsigned int mult, carry; } prng;
	int no_tables;
};

static unsigned int orc_prng_next(struct orc_tail *T)
{
	unsigned long long x = 0xfff0bf23ULL * T->prng.mult + T->prng.carry;
	T->prng.carry = (unsigned int)(x >> 32);
	T->prng.mult = 0xffffffffU - (unsigned int)(x & 0xffffffffULL);
	return T->prng.mult;
}

static void orc_prng_seed(struct orc_tail *T, int s)
{
	T->prng.mult = 0x03333333U + (unsigned int)s;
	T->prng.carry = 0x05555555U + (unsigned int)s;
}

static double orc_code_to_linear(const struct orc_tail *T, unsigned int v, const struct iw_csdescr *cs, double maxcc)
{
	if(cs->cstype == IW_CSTYPE_LINEAR) return ((double)v) / maxcc;
	if(T->rev) return T->rev[v];
	return orc_to_linear(((double)v) / maxcc, cs);
}

/* The two representable codes around v, and their linear values
 * (get_nearest_valid_colors).  Returns 1 if v maps exactly onto one code. */
static int orc_bracket(const struct orc_tail *T, double v, const struct iw_csdescr *cs, double maxcc, int cc,
	double *lin_lo, double *lin_hi, double *code_lo, double *code_hi)
{
	double t = orc_from_linear(v, cs);
	unsigned int lo, hi;
	if(cc == 0) {
		double e = t * maxcc;
		if(e > maxcc) e = maxcc;
		if(e < 0.0) e = 0.0;
		*code_lo = floor(e);
		*code_hi = ceil(e);
	}
	else {
		double steps = (double)(cc - 1);
		double e = t * steps;
		if(e > steps) e = steps;
		if(e < 0.0) e = 0.0;
		*code_lo = floor(0.5000000001 + floor(e) * (maxcc / steps));
		*code_hi = floor(0.5000000001 + ceil(e) * (maxcc / steps));
	}
	lo = (unsigned int)*code_lo;
	hi = (unsigned int)*code_hi;
	if(lo == hi) return 1;
	*lin_lo = orc_code_to_linear(T, lo, cs, maxcc);
	*lin_hi = orc_code_to_linear(T, hi, cs, maxcc);
	return 0;
}

static void orc_diffuse(struct orc_tail *T, int sub, double err, int x, int y, int width)
{
	const signed char *n = orc_ed_num[sub <= 7 ? sub : 0];
	double den = orc_ed_den[sub <= 7 ? sub : 0];
	int f = (y % 2) ? -1 : 1;
	double c[12];
	int k;
	for(k = 0; k < 12; k++) c[k] = ((double)n[k]) / den;

	if(x - f >= 0 && x - f < width) {
		if(x - 2 * f >= 0 && x - 2 * f < width) {
			T->err[1][x - 2 * f] += err * c[2];
			T->err[2][x - 2 * f] += err * c[7];
		}
		T->err[1][x - f] += err * c[3];
		T->err[2][x - f] += err * c[8];
	}
	T->err[1][x] += err * c[4];
	T->err[2][x] += err * c[9];
	if(x + f >= 0 && x + f < width) {
		T->err[0][x + f] += err * c[0];
		T->err[1][x + f] += err * c[5];
		T->err[2][x + f] += err * c[10];
		if(x + 2 * f >= 0 && x + 2 * f < width) {
			T->err[0][x + 2 * f] += err * c[1];
			T->err[1][x + 2 * f] += err * c[6];
			T->err[2][x + 2 * f] += err * c[11];
		}
	}
}

/* Quantise one linear sample to the output code (put_sample_convert_from_linear). */
static double orc_quantize(struct orc_tail *T, const struct orc_outch *o, int use_nc, double v, int x, int y, int width)
{
	double lin_lo = 0, lin_hi = 0, code_lo, code_hi, d_lo, d_hi;

	if(v < 0.0) v = 0.0;
	if(v > 1.0) v = 1.0;

	if(use_nc) {
		/* smallest index whose midpoint exceeds v */
		int lo = 0, hi = 255;
		while(lo < hi) {
			int mid = (lo + hi) / 2;
			if(T->nc[mid] > v) hi = mid; else lo = mid + 1;
		}
		return (double)lo;
	}
	if(o->dfam == IW_DITHERFAMILY_ERRDIFF) {
		v += T->err[0][x];
		if(v > 1.0) v = 1.0;
		else if(v < 0.0) v = 0.0;
	}
	if(orc_bracket(T, v, T->cs, o->maxcc_d, o->cc, &lin_lo, &lin_hi, &code_lo, &code_hi)) {
		if(o->dfam == IW_DITHERFAMILY_RANDOM) (void)orc_prng_next(T); /* one draw per sample */
		return code_lo;
	}
	d_lo = v - lin_lo;
	d_hi = lin_hi - v;
	switch(o->dfam) {
	case IW_DITHERFAMILY_NONE:
		return d_hi <= d_lo ? code_hi : code_lo;
	case IW_DITHERFAMILY_ERRDIFF:
		if(d_hi <= d_lo) {
			orc_diffuse(T, o->dsub, -d_hi, x, y, width);
			return code_hi;
		}
		orc_diffuse(T, o->dsub, d_lo, x, y, width);
		return code_lo;
	case IW_DITHERFAMILY_ORDERED: {
		double thr = ((double)orc_dither_rank[o->dsub ? 1 : 0][(x % 8) + 8 * (y % 8)] + 0.5) / 64.0;
		return (d_lo / (d_lo + d_hi) >= thr) ? code_hi : code_lo;
	}
	case IW_DITHERFAMILY_RANDOM: {
		double thr = ((double)orc_prng_next(T)) / (double)0xffffffff;
		return (d_lo / (d_lo + d_hi) >= thr) ? code_hi : code_lo;
	}
	}
	return 0.0;
}

static void orc_put(struct iw_context *ctx, int ch, int x, int y, double s, int nch)
{
	iw_byte *row = ctx->img2.pixels + (size_t)y * ctx->img2.bpr;
	if(ctx->img2.bit_depth == 8) {
		row[nch * x + ch] = (iw_byte)(0.5 + s);
	}
	else if(ctx->img2.bit_depth == 16) {
		unsigned short u = (unsigned short)(0.5 + s);
		row[(nch * x + ch) * 2] = (iw_byte)(u >> 8);
		row[(nch * x + ch) * 2 + 1] = (iw_byte)(u & 0xff);
	}
}

static void orc_put_float(struct iw_context *ctx, int ch, int x, int y, double s, int nch)
{
	float f = (float)s;
	memcpy(ctx->img2.pixels + (size_t)y * ctx->img2.bpr + (size_t)(nch * x + ch) * 4, &f, 4);
}

/* ====================================================================== */
/* The two passes (src/imagew-main.c:831-1169)                            */
/* ====================================================================== */

struct orc_run {
	struct orc_plan *P;
	struct orc_tail T;
	float *mid;        /* intermediate colour channel, mid_w x mid_h */
	float *mid_alpha;
	float *fin_alpha;  /* resampled alpha, img2 size */
	int mid_w, mid_h;
};

static int orc_vertical(struct iw_context *ctx, struct orc_run *R, int m, const struct iw_csdescr *cs)
{
	struct orc_plan *P = R->P;
	const struct orc_midch *mc = &P->mid[m];
	struct orc_weights wt;
	int is_alpha = mc->ctype == IW_CHANNELTYPE_ALPHA;
	float *dst = is_alpha ? R->mid_alpha : R->mid;
	double *in, *out;
	int x, y, ok = 0;
	int nin = P->crop_h, nout = R->mid_h;

	if(!orc_weights_build(ctx, &wt, &ctx->dim[IW_DIMENSION_V], mc->ctype, nin, nout,
		(P->apply_bk && P->bk_strategy == BK_EARLY) ? P->mid[mc->ctype < ORC_MAXCH ? mc->ctype : 0].bk_early : 0.0))
		goto done;
	in = iw_malloc(ctx, nin * sizeof(double));
	out = iw_malloc(ctx, nout * sizeof(double));
	if(!in || !out) { iw_free(ctx, in); iw_free(ctx, out); goto done; }

	for(x = 0; x < P->crop_w; x++) {
		for(y = 0; y < nin; y++) {
			double s = orc_sample_linear(ctx, P, x, y, m, cs);
			if(mc->unassoc) {
				s *= orc_raw(ctx, P, x, y, P->in_alpha);
			}
			else if(P->apply_bk && P->bk_strategy == BK_EARLY) {
				double a = orc_raw(ctx, P, x, y, P->in_alpha);
				s = (a) * (s) + (1.0 - a) * (mc->bk_early);
			}
			in[y] = s;
		}
		orc_resample(&wt, in, out);
		if(ctx->intclamp)
			for(y = 0; y < nout; y++) out[y] = out[y] < 0.0 ? 0.0 : (out[y] > 1.0 ? 1.0 : out[y]);
		for(y = 0; y < nout; y++) dst[(size_t)y * R->mid_w + x] = (float)out[y];
	}
	iw_free(ctx, in);
	iw_free(ctx, out);
	ok = 1;
done:
	orc_weights_free(ctx, &wt);
	return ok;
}

static int orc_horizontal(struct iw_context *ctx, struct orc_run *R, int m, const struct iw_csdescr *cs)
{
	struct orc_plan *P = R->P;
	const struct orc_midch *mc = &P->mid[m];
	struct orc_outch none, *o;
	struct orc_weights wt;
	int is_alpha = mc->ctype == IW_CHANNELTYPE_ALPHA;
	int och = mc->out_ch, W = ctx->img2.width;
	int bk_trns = orc_bkgd_has_trns(ctx, P);
	int use_nc, errdiff = 0;
	const float *src = is_alpha ? R->mid_alpha : R->mid;
	double *in, *out;
	int x, y, z, k, ok = 0;

	if(och >= 0) o = &P->out[och];
	else {
		memset(&none, 0, sizeof(none));
		none.ctype = IW_CHANNELTYPE_NONALPHA;
		o = &none;
	}
	use_nc = R->T.nc && !is_alpha && o->dfam == IW_DITHERFAMILY_NONE && o->cc == 0;
	R->T.cs = cs;

	if(o->dfam == IW_DITHERFAMILY_RANDOM) {
		if(o->dsub == IW_DITHERSUBTYPE_SAMEPATTERN && o->ctype != IW_CHANNELTYPE_ALPHA)
			orc_prng_seed(&R->T, ctx->seed);
		else
			orc_prng_seed(&R->T, ctx->seed + o->ctype);
	}
	if(och >= 0 && o->dfam == IW_DITHERFAMILY_ERRDIFF) {
		errdiff = 1;
		for(k = 0; k < 3; k++) memset(R->T.err[k], 0, W * sizeof(double));
	}

	if(!orc_weights_build(ctx, &wt, &ctx->dim[IW_DIMENSION_H], mc->ctype, R->mid_w, W,
		(P->apply_bk && P->bk_strategy == BK_EARLY) ? P->mid[mc->ctype < ORC_MAXCH ? mc->ctype : 0].bk_early : 0.0))
		goto done;
	in = iw_malloc(ctx, R->mid_w * sizeof(double));
	out = iw_malloc(ctx, W * sizeof(double));
	if(!in || !out) { iw_free(ctx, in); iw_free(ctx, out); goto done; }

	for(y = 0; y < R->mid_h; y++) {
		for(x = 0; x < R->mid_w; x++) in[x] = src[(size_t)y * R->mid_w + x];
		orc_resample(&wt, in, out);
		if(ctx->intclamp)
			for(x = 0; x < W; x++) out[x] = out[x] < 0.0 ? 0.0 : (out[x] > 1.0 ? 1.0 : out[x]);
		if(is_alpha && R->fin_alpha)
			for(x = 0; x < W; x++) R->fin_alpha[(size_t)y * W + x] = (float)out[x];
		if(och < 0) continue;

		for(z = 0; z < W; z++) {
			int alt = 0;
			double s, a, bka = 0.0;
			x = (errdiff && (y % 2)) ? W - 1 - z : z;
			s = out[x];
			if(P->bk_checker)
				alt = (((ctx->check_origin[0] + x) / ctx->check_size) % 2) !=
				      (((ctx->check_origin[1] + y) / ctx->check_size) % 2);
			if(bk_trns) bka = alt ? P->bk2_alpha : P->bk1_alpha;
			if(mc->unassoc) {
				a = R->fin_alpha[(size_t)y * W + x];
				if(a != 0.0) s /= a;
				if(P->apply_bk && P->bk_strategy == BK_LATE) {
					double bc = alt ? o->bk2 : o->bk1;
					if(bk_trns) s = s * a + bc * bka * (1.0 - a);
					else s = s * a + bc * (1.0 - a);
				}
			}
			else if(is_alpha && bk_trns) {
				s = s + bka * (1.0 - s);
			}
			if(ctx->img2.sampletype == IW_SAMPLETYPE_FLOATINGPOINT)
				orc_put_float(ctx, och, x, y, s, P->out_n);
			else
				orc_put(ctx, och, x, y, orc_quantize(&R->T, o, use_nc, s, x, y, W), P->out_n);
		}
		if(errdiff) {
			for(x = 0; x < W; x++) {
				R->T.err[0][x] = R->T.err[1][x];
				R->T.err[1][x] = R->T.err[2][x];
				R->T.err[2][x] = 0.0;
			}
		}
	}
	iw_free(ctx, in);
	iw_free(ctx, out);
	ok = 1;
done:
	orc_weights_free(ctx, &wt);
	return ok;
}

static int orc_one_channel(struct iw_context *ctx, struct orc_run *R, int m,
	const struct iw_csdescr *cs_in, const struct iw_csdescr *cs_out)
{
	return orc_vertical(ctx, R, m, cs_in) && orc_horizontal(ctx, R, m, cs_out);
}

/* Output background label (src/imagew-main.c:1238-1322). */
static unsigned int orc_quantize_plain(struct orc_tail *T, double v, const struct iw_csdescr *cs, double maxcc)
{
	double lin_lo = 0, lin_hi = 0, code_lo, code_hi, s;
	if(v < 0.0) v = 0.0;
	if(v > 1.0) v = 1.0;
	if(orc_bracket(T, v, cs, maxcc, 0, &lin_lo, &lin_hi, &code_lo, &code_hi)) s = code_lo;
	else s = (lin_hi - v <= v - lin_lo) ? code_hi : code_lo;
	return (unsigned int)(0.5 + s);
}

static void orc_bkgd_label(struct iw_context *ctx, struct orc_run *R)
{
	struct iw_color c = {{1.0, 0.0, 1.0, 1.0}};
	double maxc;
	unsigned int u;
	int k;
	if(!(ctx->profile & (IW_PROFILE_PNG_BKGD | IW_PROFILE_RGB8_BKGD | IW_PROFILE_RGB16_BKGD))) return;
	if(ctx->no_outlabel) return;
	if(ctx->outlabel_valid) c = ctx->outlabel;
	else if(ctx->inlabel_set) c = R->P->inlabel_lin;
	else return;
	if(ctx->to_gray) {
		double g = orc_gray_of(ctx, c.c[0], c.c[1], c.c[2]);
		c.c[0] = c.c[1] = c.c[2] = g;
	}
	if(ctx->profile & IW_PROFILE_RGB8_BKGD) maxc = 255.0;
	else if(ctx->profile & IW_PROFILE_RGB16_BKGD) maxc = 65535.0;
	else if(ctx->img2.bit_depth == 8) maxc = 255.0;
	else if(ctx->img2.bit_depth == 16) maxc = 65535.0;
	else return;
	for(k = 0; k < 3; k++) {
		u = orc_quantize_plain(&R->T, c.c[k], &ctx->cs_out, maxc);
		ctx->img2.bkgdlabel.c[k] = ((double)u) / maxc;
	}
	if(c.c[3] <= 0.0) u = 0;
	else if(c.c[3] >= 1.0) u = (unsigned int)maxc;
	else u = (unsigned int)(0.5 + c.c[3] * (unsigned int)maxc);
	ctx->img2.bkgdlabel.c[3] = ((double)u) / maxc;
	ctx->img2.has_bkgdlabel = 1;
}

static void orc_negate(struct iw_context *ctx, struct orc_plan *P)
{
	int ch, x, y, n = P->out_n;
	for(ch = 0; ch < n; ch++) {
		if(P->out[ch].ctype == IW_CHANNELTYPE_ALPHA) continue;
		for(y = 0; y < ctx->img2.height; y++) {
			iw_byte *row = ctx->img2.pixels + (size_t)y * ctx->img2.bpr;
			for(x = 0; x < ctx->img2.width; x++) {
				if(ctx->img2.sampletype == IW_SAMPLETYPE_FLOATINGPOINT) {
					float f;
					memcpy(&f, row + (size_t)(n * x + ch) * 4, 4);
					f = ((float)1.0) - f;
					memcpy(row + (size_t)(n * x + ch) * 4, &f, 4);
				}
				else if(ctx->img2.bit_depth == 8) {
					row[n * x + ch] = (iw_byte)(P->out[ch].maxcc - row[n * x + ch]);
				}
				else if(ctx->img2.bit_depth == 16) {
					iw_byte *p = row + (size_t)(n * x + ch) * 2;
					unsigned int v = (unsigned int)P->out[ch].maxcc - (p[0] * 256u + p[1]);
					p[0] = (iw_byte)((v & 0xff00) >> 8);
					p[1] = (iw_byte)(v & 0xff);
				}
			}
		}
	}
}

static int orc_process(struct iw_context *ctx, struct orc_plan *P)
{
	struct orc_run R;
	struct iw_csdescr lin;
	int ok = 0, m, k;

	memset(&R, 0, sizeof(R));
	R.P = P;
	R.mid_w = P->crop_w;
	R.mid_h = ctx->img2.height;
	iw_make_linear_csdescr(&lin);

	ctx->img2.bpr = iw_calc_bytesperrow(ctx->img2.width, ctx->img2.bit_depth * P->out_n);
	ctx->img2.pixels = iw_malloc_large(ctx, ctx->img2.bpr, ctx->img2.height);
	if(!ctx->img2.pixels) goto done;
	R.mid = iw_malloc_large(ctx, (size_t)R.mid_w * R.mid_h, sizeof(float));
	if(!R.mid) goto done;
	if(P->errdiff) {
		for(k = 0; k < 3; k++) {
			R.T.err[k] = iw_malloc(ctx, ctx->img2.width * sizeof(double));
			if(!R.T.err[k]) goto done;
		}
	}
	if(!P->no_out_tables) {
		R.T.rev = orc_make_lin_table(ctx, &ctx->img2, &ctx->cs_out);
		if(!ctx->no_gamma && ctx->cs_out.cstype != IW_CSTYPE_LINEAR &&
			ctx->img2.sampletype != IW_SAMPLETYPE_FLOATINGPOINT && ctx->img2.bit_depth <= 8 &&
			((size_t)ctx->img2.width) * ctx->img2.height > 512)
		{
			int n = (1 << ctx->img2.bit_depth) - 1, i;
			double prev = 0.0;
			R.T.nc = iw_malloc(ctx, n * sizeof(double));
			if(R.T.nc) {
				for(i = 0; i < n; i++) {
					double cur = orc_to_linear(((double)(i + 1)) / n, &ctx->cs_out);
					R.T.nc[i] = (prev + cur) / 2.0;
					prev = cur;
				}
			}
		}
	}

	if(IW_IMGTYPE_HAS_ALPHA(P->mid_type)) {
		R.mid_alpha = iw_malloc_large(ctx, (size_t)R.mid_w * R.mid_h, sizeof(float));
		if(!R.mid_alpha) goto done;
		R.fin_alpha = iw_malloc_large(ctx, (size_t)ctx->img2.width * ctx->img2.height, sizeof(float));
		if(!R.fin_alpha) goto done;
		if(!orc_one_channel(ctx, &R, P->mid_alpha, &lin, &lin)) goto done;
	}
	for(m = 0; m < P->mid_n; m++) {
		if(P->mid[m].ctype == IW_CHANNELTYPE_ALPHA) continue;
		if(ctx->no_gamma) {
			if(!orc_one_channel(ctx, &R, m, &lin, &lin)) goto done;
		}
		else if(!orc_one_channel(ctx, &R, m, &ctx->cs_in, &ctx->cs_out)) goto done;
	}
	orc_bkgd_label(ctx, &R);
	if(ctx->negate) orc_negate(ctx, P);
	ok = 1;
done:
	iw_free(ctx, R.mid);
	iw_free(ctx, R.mid_alpha);
	iw_free(ctx, R.fin_alpha);
	for(k = 0; k < 3; k++) iw_free(ctx, R.T.err[k]);
	iw_free(ctx, R.T.rev);
	iw_free(ctx, R.T.nc);
	return ok;
}

int iw_process_image(struct iw_context *ctx)
{
	struct orc_plan P;
	int ok;
	if(ctx->use_count > 0) {
		iw_set_error(ctx, "Internal: Incorrect attempt to reprocess image");
		return 0;
	}
	ctx->use_count++;
	memset(&P, 0, sizeof(P));
	ok = orc_prepare(ctx, &P) && orc_process(ctx, &P);
	iw_free(ctx, P.in_tab);
	if(!ok) return 0;
	orc_optimize(ctx);
	return 1;
}

void iw_get_output_image(struct iw_context *ctx, struct iw_image *img)
{
	const struct orc_opt *o = &ctx->opt;
	int k;
	memset(img, 0, sizeof(*img));
	img->width = o->width;
	img->height = o->height;
	img->imgtype = o->imgtype;
	img->sampletype = ctx->img2.sampletype;
	img->bit_depth = o->bit_depth;
	img->pixels = (iw_byte *)o->pix;
	img->bpr = o->bpr;
	img->density_code = ctx->img2.density_code;
	img->density_x = ctx->img2.density_x;
	img->density_y = ctx->img2.density_y;
	img->rendering_intent = ctx->img2.rendering_intent;
	img->has_bkgdlabel = o->has_label;
	for(k = 0; k < 4; k++)
		img->bkgdlabel.c[k] = ((double)o->label[k]) / (o->bit_depth == 8 ? 255.0 : 65535.0);
	img->has_colorkey_trns = o->has_ckey;
	img->colorkey[0] = o->ckey[0];
	img->colorkey[1] = o->ckey[1];
	img->colorkey[2] = o->ckey[2];
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

/* ====================================================================== */
/* Stateless helpers (src/imagew-api.c:682-758, src/imagew-util.c)       */
/* ====================================================================== */

int iw_get_sample_size(void) { return (int)sizeof(float); }
int iw_get_version_int(void) { return IW_VERSION_INT; }

char *iw_get_version_string(struct iw_context *ctx, char *s, int n)
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
void iw_set_ui32le(iw_byte *b, unsigned int n) { b[0] = n & 0xff; b[1] = (n >> 8) & 0xff; b[2] = (n >> 16) & 0xff; b[3] = (n >> 24) & 0xff; }
void iw_set_ui16be(iw_byte *b, unsigned int n) { b[0] = (n >> 8) & 0xff; b[1] = n & 0xff; }
void iw_set_ui32be(iw_byte *b, unsigned int n) { b[0] = (n >> 24) & 0xff; b[1] = (n >> 16) & 0xff; b[2] = (n >> 8) & 0xff; b[3] = n & 0xff; }
unsigned int iw_get_ui16le(const iw_byte *b) { return (unsigned int)b[0] | ((unsigned int)b[1] << 8); }
unsigned int iw_get_ui32le(const iw_byte *b) { return (unsigned int)b[0] | ((unsigned int)b[1] << 8) | ((unsigned int)b[2] << 16) | ((unsigned int)b[3] << 24); }
int iw_get_i32le(const iw_byte *b) { return (int32_t)iw_get_ui32le(b); }
unsigned int iw_get_ui16be(const iw_byte *b) { return ((unsigned int)b[0] << 8) | (unsigned int)b[1]; }
unsigned int iw_get_ui32be(const iw_byte *b) { return ((unsigned int)b[0] << 24) | ((unsigned int)b[1] << 16) | ((unsigned int)b[2] << 8) | (unsigned int)b[3]; }
unsigned int iw_get_ui16_e(const iw_byte *b, int e) { return e == IW_ENDIAN_LITTLE ? iw_get_ui16le(b) : iw_get_ui16be(b); }
unsigned int iw_get_ui32_e(const iw_byte *b, int e) { return e == IW_ENDIAN_LITTLE ? iw_get_ui32le(b) : iw_get_ui32be(b); }

int iw_max_color_to_bitdepth(unsigned int mc)
{
	unsigned int bd;
	for(bd = 1; bd <= 15; bd++) if(mc < (1U << bd)) return (int)bd;
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
		{"ppm", IW_FORMAT_PPM}, {"pam", IW_FORMAT_PAM}, {NULL, 0}};
	const char *s = strrchr(fn, '.');
	int i;
	if(!s) return IW_FORMAT_UNKNOWN;
	for(i = 0; t[i].ext; i++) if(!iw_stricmp(s + 1, t[i].ext)) return t[i].fmt;
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
	return NULL;
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
	if(b[0] == 'P' && b[1] == '7' && b[2] == 0x0a) return IW_FORMAT_PAM;
	return IW_FORMAT_UNKNOWN;
}

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
		{0x201c, "\""}, {0x201d, "\""}, {0x2192, "->"}, {0xfeff, ""}, {0, NULL}};
	int dp = 0, need = 0, i;
	unsigned int cp = 0;
	for(; *src; src++) {
		unsigned char c = (unsigned char)*src;
		const char *rep = NULL;
		if(c < 128) {
			if(dp <= dstlen - 2) dst[dp++] = (char)c;
			need = 0;
			continue;
		}
		if(c < 0xc0) {
			if(need > 0) {
				cp = (cp << 6) | (c & 0x3f);
				if(--need < 1) {
					rep = "?";
					for(i = 0; map[i].s; i++) if(map[i].code == cp) { rep = map[i].s; break; }
					for(i = 0; rep[i]; i++) if(dp <= dstlen - 2) dst[dp++] = rep[i];
				}
			}
		}
		else if(c < 0xe0) { cp = c & 0x1f; need = 1; }
		else if(c < 0xf0) { cp = c & 0x0f; need = 2; }
		else if(c < 0xf8) { cp = c & 0x07; need = 3; }
	}
	dst[dp] = '\0';
}

static int orc_number_len(const char *s, int *slash)
{
	int i;
	for(i = 0; s[i]; i++) {
		if(s[i] == '/') *slash = i;
		if(s[i] == ',') return i;
	}
	return i;
}

static int orc_parse_one(const char *s, double *out, int *used)
{
	int slash = -1, len = orc_number_len(s, &slash);
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
		if(!orc_parse_one(s + pos, &res[n], &used)) break;
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
	orc_parse_one(s, &r, &used);
	return r;
}

int iw_round_to_int(double x)
{
	return x < 0.0 ? -(int)(0.5 - x) : (int)(0.5 + x);
}

int iw_parse_int(const char *s)
{
	return iw_round_to_int(iw_parse_number(s));
}
