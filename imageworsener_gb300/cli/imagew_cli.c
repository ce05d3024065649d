/*
 * imagew_cli.c -- imagew_gb300, a command-line front end of libimagew_gb300
 * for PNM (PGM/PPM, binary) and PAM files.
 *
 *   imagew_gb300 [options] <infile> <outfile>
 *
 * It reads the input with pnm.c, configures a context through the libimagew
 * API, runs iw_process_image() (the GPU pipeline when linked against
 * libimagew_gb300) and writes the output; for these formats the written file
 * is the one the reference's imagew would write (ImageWorsener 1.3.5
 * src/imagew-cmd.c, iwcmd_run :1046-1479).
 *
 * Options (the reference's names and meanings, src/imagew-cmd.c:2107-2197):
 *   -w, -width N|xF; -h, -height N|xF   output size in pixels or relative to
 *                                   the input (x1.5); one of them alone keeps
 *                                   the aspect ratio
 *   -s W,H; -S W,H                  fit inside W x H; exactly W x H
 *   -bestfit, -nobestfit            fit -w x -h inside, or not; -noresize
 *   -filter, -filterx, -filtery F   resampling filter: mix nearest point linear
 *                                   triangle quadratic hermite box boxavg
 *                                   gaussian auto null lanczos[N] hann[N]
 *                                   hanning[N] blackman[N] sinc[N] catrom
 *                                   mitchell bspline cubicB,C keys[A]
 *   -blur, -blurx, -blury X|x[F]    filter blur factor (alone: gaussian); "x":
 *                                   interpolate (sharpened when downscaling)
 *   -edge, -edgex, -edgey s|r|t     edge policy (standard, replicate, transparent)
 *   -translate [s]X,Y               shift the image (s: in input pixels)
 *   -imagesize W,H                  size of the image within the canvas
 *   -offsetred|green|blue|rb X      channel offsets, horizontal (rb: red by X,
 *   -offsetvred|vgreen|vblue|vrb X  blue by -X) and vertical
 *   -depth N|R,G,B,A; -depthgray N; -depthalpha N; -depthcc N   output depths
 *   -sampletype u|f
 *   -cc N|R,G,B,A; -cccolor, -ccalpha, -ccred, -ccgreen, -ccblue, -ccgray N
 *   -dither D; -dithercolor, -ditheralpha, -ditherred, -dithergreen,
 *     -ditherblue, -dithergray D    f fs o halftone r r2 jjn stucki burkes
 *                                   sierra sierra3 sierra2 sierralite atkinson none
 *   -grayscale, -condgrayscale      convert to grayscale (conditional: only
 *                                   if the input is gray)
 *   -gsf, -grayscaleformula s|c|wR,G,B|vA[,B,C]
 *   -cs, -inputcs gammaG|linear|srgb[p|r|s|a]|rec709
 *   -intent p|r|s|a|perceptual|relative|saturation|absolute|default|none
 *   -nogamma, -intclamp, -negate, -nocslabel
 *   -noopt all|grayscale|palette|reduceto8|stripalpha|binarytrns
 *   -randseed N|r
 *   -bkgd C[,C2]; -checkersize N; -checkerorigin X,Y   background (RGB hex)
 *   -bkgdlabel C; -usebkgdlabel; -nobkgdlabel
 *   -reorient fliph|flipv|rotate90|rotate180|rotate270|transpose|transverse|N
 *   -crop X,Y[,W,H]                 use part of the input
 *   -infmt, -outfmt pam|ppm|pgm|pbm|pnm   file formats (default: from the
 *                                   file's contents / name)
 *   -opt NAME=VALUE                 iw_set_option(), e.g. gpu:precision=fp64
 *   -noinfo, -quiet, -nowarn        messages
 * Options that only concern other file formats (-compress, -colortype,
 * -page, -jpegquality, -jpegsampling, -webpquality, -zipcmprlevel,
 * -pngcmprlevel, -bmpversion, -density, -encoding, -precision, -interlace,
 * -jpegarith, -bmptrns, -includescreen, -noincludescreen, -msgstostdout,
 * -msgstostderr) are accepted and change nothing in PNM/PAM files.
 */
#define IW_INCLUDE_UTIL_FUNCTIONS
#include "imagew.h"
#include "pnm.h"

#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

struct opt_kv { char *name, *val; };

struct dither_req { int fam, sub; };   /* fam < 0: not given */

struct params {
	const char *in, *out;
	int infmt, outfmt;
	int dst_w_req, dst_h_req;
	int rel_flag[2];             /* size given relative to the input: rel[k] x */
	double rel[2];
	int bestfit, bestfit_option, noresize;
	int fam[2];                  /* resize family per dimension (0: library default) */
	double p1[2], p2[2], blur[2];
	int blur_set[2], blur_interp[2];
	int edge[2];
	int translate_set, translate_src;
	double translate_x, translate_y;
	int imagesize_set;
	double imagesize_x, imagesize_y;
	double offset_h[3], offset_v[3];
	int depth, depthcc, channel_depth[5];
	int sample_type;
	int cc_all, cc_nonalpha, cc[5];
	struct dither_req dither_all, dither_nonalpha, dither[5];
	int grayscale, condgrayscale, gsf;
	double gsf_w[3];
	int cs_in_set, cs_out_set, intent;
	struct iw_csdescr cs_in, cs_out;
	int nogamma, intclamp, negate, nocslabel;
	int noopt[6];                /* indexed by IW_OPT_* */
	int randomize, random_seed;
	int apply_bkgd, checkerboard, check_size, check_x, check_y;
	struct iw_color bkgd, bkgd2;
	int bkgd_label_set, use_bkgd_label, no_bkgd_label;
	struct iw_color bkgd_label;
	unsigned int reorient;
	int use_crop, crop_x, crop_y, crop_w, crop_h;
	int noinfo, nowarn;
	struct opt_kv opts[32];
	int nopts;
};

static int name_len(const char *s)
{
	int i;
	for(i = 0; s[i]; i++)
		if(!((s[i] >= 'a' && s[i] <= 'z') || (s[i] >= 'A' && s[i] <= 'Z'))) return i;
	return i;
}

/* Resize-algorithm names (src/imagew-cmd.c:1622-1735). */
static int decode_filter(const char *s, int *fam, double *p1, double *p2)
{
	static const struct { const char *name; int fam; } tab[] = {
		{"mix", IW_RESIZETYPE_MIX}, {"nearest", IW_RESIZETYPE_NEAREST}, {"point", IW_RESIZETYPE_NEAREST},
		{"linear", IW_RESIZETYPE_TRIANGLE}, {"triangle", IW_RESIZETYPE_TRIANGLE},
		{"quadratic", IW_RESIZETYPE_QUADRATIC}, {"hermite", IW_RESIZETYPE_HERMITE}, {"box", IW_RESIZETYPE_BOX},
		{"boxavg", IW_RESIZETYPE_BOXAVG}, {"gaussian", IW_RESIZETYPE_GAUSSIAN}, {"auto", IW_RESIZETYPE_AUTO},
		{"null", IW_RESIZETYPE_NULL}, {NULL, 0}};
	int i, len = (int)strlen(s), nl = name_len(s);
	*p1 = *p2 = 0.0;
	for(i = 0; tab[i].name; i++)
		if(!strcmp(s, tab[i].name)) { *fam = tab[i].fam; return 1; }
	if(nl == 7 && !strncmp(s, "lanczos", 7)) { *p1 = len > nl ? atof(s + nl) : 3.0; *fam = IW_RESIZETYPE_LANCZOS; return 1; }
	if((nl == 4 && !strncmp(s, "hann", 4)) || (nl == 7 && !strncmp(s, "hanning", 7))) {
		*p1 = len > nl ? atof(s + nl) : 4.0; *fam = IW_RESIZETYPE_HANNING; return 1;
	}
	if(nl == 8 && !strncmp(s, "blackman", 8)) { *p1 = len > nl ? atof(s + nl) : 4.0; *fam = IW_RESIZETYPE_BLACKMAN; return 1; }
	if(nl == 4 && !strncmp(s, "sinc", 4)) { *p1 = len > nl ? atof(s + nl) : 4.0; *fam = IW_RESIZETYPE_SINC; return 1; }
	if(!strcmp(s, "catrom")) { *fam = IW_RESIZETYPE_CUBIC; *p1 = 0.0; *p2 = 0.5; return 1; }
	if(!strcmp(s, "mitchell")) { *fam = IW_RESIZETYPE_CUBIC; *p1 = 1.0 / 3; *p2 = 1.0 / 3; return 1; }
	if(!strcmp(s, "bspline")) { *fam = IW_RESIZETYPE_CUBIC; *p1 = 1.0; *p2 = 0.0; return 1; }
	if(nl == 5 && !strncmp(s, "cubic", 5)) {
		const char *comma = strchr(s, ',');
		if(len < nl + 3 || !comma) return 0;
		*p1 = atof(s + nl);
		*p2 = atof(comma + 1);
		*fam = IW_RESIZETYPE_CUBIC;
		return 1;
	}
	if(nl == 4 && !strncmp(s, "keys", 4)) {
		*p2 = len > nl ? atof(s + nl) : 0.5;
		*p1 = 1.0 - 2.0 * *p2;
		*fam = IW_RESIZETYPE_CUBIC;
		return 1;
	}
	return 0;
}

/* Dither names (src/imagew-cmd.c:1762-1799). */
static int decode_dither(const char *s, int *fam, int *sub)
{
	static const struct { const char *name; int fam, sub; } tab[] = {
		{"f", IW_DITHERFAMILY_ERRDIFF, IW_DITHERSUBTYPE_FS}, {"fs", IW_DITHERFAMILY_ERRDIFF, IW_DITHERSUBTYPE_FS},
		{"o", IW_DITHERFAMILY_ORDERED, IW_DITHERSUBTYPE_DEFAULT},
		{"halftone", IW_DITHERFAMILY_ORDERED, IW_DITHERSUBTYPE_HALFTONE},
		{"r", IW_DITHERFAMILY_RANDOM, IW_DITHERSUBTYPE_DEFAULT},
		{"r2", IW_DITHERFAMILY_RANDOM, IW_DITHERSUBTYPE_SAMEPATTERN},
		{"jjn", IW_DITHERFAMILY_ERRDIFF, IW_DITHERSUBTYPE_JJN}, {"stucki", IW_DITHERFAMILY_ERRDIFF, IW_DITHERSUBTYPE_STUCKI},
		{"burkes", IW_DITHERFAMILY_ERRDIFF, IW_DITHERSUBTYPE_BURKES},
		{"sierra", IW_DITHERFAMILY_ERRDIFF, IW_DITHERSUBTYPE_SIERRA3},
		{"sierra3", IW_DITHERFAMILY_ERRDIFF, IW_DITHERSUBTYPE_SIERRA3},
		{"sierra2", IW_DITHERFAMILY_ERRDIFF, IW_DITHERSUBTYPE_SIERRA2},
		{"sierralite", IW_DITHERFAMILY_ERRDIFF, IW_DITHERSUBTYPE_SIERRA42A},
		{"atkinson", IW_DITHERFAMILY_ERRDIFF, IW_DITHERSUBTYPE_ATKINSON},
		{"none", IW_DITHERFAMILY_NONE, IW_DITHERSUBTYPE_DEFAULT}, {NULL, 0, 0}};
	int i;
	for(i = 0; tab[i].name; i++)
		if(!strcmp(s, tab[i].name)) { *fam = tab[i].fam; *sub = tab[i].sub; return 1; }
	return 0;
}

/* Format names (src/imagew-cmd.c:393-410); only the PNM family is read and
 * written here, the others are known names that the run refuses. */
static int decode_fmt(const char *s)
{
	static const struct { const char *name; int fmt; } tab[] = {
		{"png", IW_FORMAT_PNG}, {"jpg", IW_FORMAT_JPEG}, {"jpeg", IW_FORMAT_JPEG}, {"bmp", IW_FORMAT_BMP},
		{"tif", IW_FORMAT_TIFF}, {"tiff", IW_FORMAT_TIFF}, {"miff", IW_FORMAT_MIFF}, {"webp", IW_FORMAT_WEBP},
		{"gif", IW_FORMAT_GIF}, {"pnm", IW_FORMAT_PNM}, {"ppm", IW_FORMAT_PPM}, {"pgm", IW_FORMAT_PGM},
		{"pbm", IW_FORMAT_PBM}, {"pam", IW_FORMAT_PAM}, {NULL, 0}};
	int i;
	for(i = 0; tab[i].name; i++)
		if(!strcmp(s, tab[i].name)) return tab[i].fmt;
	return IW_FORMAT_UNKNOWN;
}

static int is_pnm_family(int fmt)
{
	return fmt == IW_FORMAT_PNM || fmt == IW_FORMAT_PPM || fmt == IW_FORMAT_PGM || fmt == IW_FORMAT_PBM ||
	       fmt == IW_FORMAT_PAM;
}

/* Colour-space names (src/imagew-cmd.c:1802-1836): gammaG, linear,
 * srgb with an optional rendering-intent letter, rec709. */
static int decode_cs(const char *s, struct iw_csdescr *cs, int *intent)
{
	const int len = (int)strlen(s), nl = name_len(s);
	if(nl == 5 && len > 5 && !strncmp(s, "gamma", 5)) { iw_make_gamma_csdescr(cs, iw_parse_number(s + 5)); return 1; }
	if(!strcmp(s, "linear")) { iw_make_linear_csdescr(cs); return 1; }
	if(len >= 4 && !strncmp(s, "srgb", 4)) {
		if(s[4] == 'p') *intent = IW_INTENT_PERCEPTUAL;
		else if(s[4] == 'r') *intent = IW_INTENT_RELATIVE;
		else if(s[4] == 's') *intent = IW_INTENT_SATURATION;
		else if(s[4] == 'a') *intent = IW_INTENT_ABSOLUTE;
		iw_make_srgb_csdescr_2(cs);
		return 1;
	}
	if(!strcmp(s, "rec709")) { iw_make_rec709_csdescr(cs); return 1; }
	return 0;
}

/* Rendering intents (src/imagew-cmd.c:1971-1997). */
static int decode_intent(const char *s, int *intent)
{
	static const struct { const char *a, *b; int v; } tab[] = {
		{"p", "perceptual", IW_INTENT_PERCEPTUAL}, {"r", "relative", IW_INTENT_RELATIVE},
		{"s", "saturation", IW_INTENT_SATURATION}, {"a", "absolute", IW_INTENT_ABSOLUTE},
		{"", "default", IW_INTENT_DEFAULT}, {"", "none", IW_INTENT_NONE}, {NULL, NULL, 0}};   /* no short forms */
	int i;
	for(i = 0; tab[i].a; i++)
		if((tab[i].a[0] && !strcmp(s, tab[i].a)) || !strcmp(s, tab[i].b)) { *intent = tab[i].v; return 1; }
	return 0;
}

/* Grayscale formulas (src/imagew-cmd.c:1939-1969): s(tandard), c(ompatible),
 * w<r>,<g>,<b> (weighted, three weights), v<a>[,<b>,<c>] (weights by value
 * order, at least one). */
static int decode_gsf(const char *s, int *gsf, double w[3])
{
	const int nl = name_len(s);
	if(!strcmp(s, "s")) { *gsf = IW_GSF_STANDARD; return 1; }
	if(!strcmp(s, "c")) { *gsf = IW_GSF_COMPATIBLE; return 1; }
	if(nl == 1 && s[0] == 'w') {
		if(iw_parse_number_list(s + 1, 3, w) != 3) return 0;
		*gsf = IW_GSF_WEIGHTED;
		return 1;
	}
	if(nl == 1 && s[0] == 'v') {
		if(iw_parse_number_list(s + 1, 3, w) < 1) return 0;
		*gsf = IW_GSF_ORDERBYVALUE;
		return 1;
	}
	return 0;
}

static int decode_noopt(const char *s, int noopt[6])
{
	static const struct { const char *name; int opt; } tab[] = {
		{"grayscale", IW_OPT_GRAYSCALE}, {"palette", IW_OPT_PALETTE}, {"reduceto8", IW_OPT_16_TO_8},
		{"stripalpha", IW_OPT_STRIP_ALPHA}, {"binarytrns", IW_OPT_BINARY_TRNS}, {NULL, 0}};
	int i;
	for(i = 0; tab[i].name; i++) {
		if(!strcmp(s, "all")) noopt[tab[i].opt] = 1;
		else if(!strcmp(s, tab[i].name)) { noopt[tab[i].opt] = 1; return 1; }
	}
	return !strcmp(s, "all");
}

/* Orientation transforms (src/imagew-cmd.c:1999-2018); a number is passed as is. */
static int decode_reorient(const char *s, unsigned int *r)
{
	static const struct { const char *name; unsigned int v; } tab[] = {
		{"fliph", IW_REORIENT_FLIP_H}, {"flipv", IW_REORIENT_FLIP_V}, {"rotate90", IW_REORIENT_ROTATE_90},
		{"rotate180", IW_REORIENT_ROTATE_180}, {"rotate270", IW_REORIENT_ROTATE_270},
		{"transpose", IW_REORIENT_TRANSPOSE}, {"transverse", IW_REORIENT_TRANSVERSE}, {NULL, 0}};
	int i;
	if(s[0] >= '0' && s[0] <= '9') { *r = (unsigned int)iw_parse_int(s); return 1; }
	for(i = 0; tab[i].name; i++)
		if(!strcmp(s, tab[i].name)) { *r = tab[i].v; return 1; }
	return 0;
}

/* A background colour of 3, 4, 6, 8, 12 or 16 hex digits: 1, 2 or 4 digits
 * per channel, RGB or RGBA; any other length gives magenta
 * (src/imagew-cmd.c:1547-1577).  Alpha is 1 unless given. */
static int hexd(char d)
{
	if(d >= '0' && d <= '9') return d - '0';
	if(d >= 'a' && d <= 'f') return d - 'a' + 10;
	if(d >= 'A' && d <= 'F') return d - 'A' + 10;
	return 0;
}

static void parse_color(struct iw_color *clr, const char *s, size_t len)
{
	int digits = 0, nch = 0, k, i;
	clr->c[IW_CHANNELTYPE_ALPHA] = 1.0;
	switch(len) {
	case 3: digits = 1; nch = 3; break;
	case 4: digits = 1; nch = 4; break;
	case 6: digits = 2; nch = 3; break;
	case 8: digits = 2; nch = 4; break;
	case 12: digits = 4; nch = 3; break;
	case 16: digits = 4; nch = 4; break;
	default:
		clr->c[0] = 1.0; clr->c[1] = 0.0; clr->c[2] = 1.0;
		return;
	}
	for(k = 0; k < nch; k++) {
		int v = 0;
		for(i = 0; i < digits; i++) v = 16 * v + hexd(s[k * digits + i]);
		clr->c[k] = (double)v / (double)((1 << (4 * digits)) - 1);
	}
}

/* Channel-name suffix of -cc<name>, -dither<name>, -offset<name>: the
 * IW_CHANNELTYPE_* index, -1 if none. */
static int channel_suffix(const char *s)
{
	if(!strcmp(s, "red")) return IW_CHANNELTYPE_RED;
	if(!strcmp(s, "green")) return IW_CHANNELTYPE_GREEN;
	if(!strcmp(s, "blue")) return IW_CHANNELTYPE_BLUE;
	if(!strcmp(s, "alpha")) return IW_CHANNELTYPE_ALPHA;
	if(!strcmp(s, "gray")) return IW_CHANNELTYPE_GRAY;
	return -1;
}

/* Up to four comma-separated numbers rounded to integers; the ones not
 * given are left as they are. */
static void parse_ints(const char *s, int *out, int n)
{
	double v[4];
	const int c = iw_parse_number_list(s, n, v);
	int k;
	for(k = 0; k < c && k < n; k++) out[k] = iw_round_to_int(v[k]);
}

static void parse_dbl_pair(const char *s, double *a, double *b)
{
	double v[2];
	const int c = iw_parse_number_list(s, 2, v);
	if(c >= 1) *a = v[0];
	if(c >= 2) *b = v[1];
}

static void warn_fn(struct iw_context *ctx, const char *msg)
{
	struct params *p = (struct params *)iw_get_userdata(ctx);
	if(!p || !p->nowarn) fprintf(stderr, "Warning: %s\n", msg);
}

/* The reference's fit of the source into dst_w x dst_h keeping the aspect
 * ratio (src/imagew-cmd.c:427-454); returns 1 if it fitted to the height. */
static int bestfit(int src_w, int src_h, int *dst_w, int *dst_h)
{
	int x, r = 0;
	double f = (double)*dst_w / src_w;
	x = (int)(0.5 + (double)src_h * f);
	if(x <= *dst_h) *dst_h = x;
	else {
		r = 1;
		f = (double)*dst_h / src_h;
		x = (int)(0.5 + (double)src_w * f);
		if(x < *dst_w) *dst_w = x;
	}
	if(*dst_w < 1) *dst_w = 1;
	if(*dst_h < 1) *dst_h = 1;
	return r;
}

/* Output depths (src/imagew-cmd.c:984-1044): -depthcc alone sets the maximum
 * code of every channel; otherwise the overall depth is the largest of -depth
 * and the per-channel depths, rounded up to 8 or 16, and every channel whose
 * depth is below it gets the maximum code 2^depth - 1. */
static void set_depths(struct params *p, struct iw_context *ctx)
{
	int k, overall = p->depth;
	if(p->depthcc >= 2) {
		for(k = 0; k < 5; k++) iw_set_output_max_color_code(ctx, k, p->depthcc - 1);
		return;
	}
	for(k = 0; k < 5; k++)
		if(overall < p->channel_depth[k]) overall = p->channel_depth[k];
	if(!overall) return;
	overall = overall <= 8 ? 8 : 16;
	iw_set_output_depth(ctx, overall);
	for(k = 0; k < 5; k++) {
		const int d = p->channel_depth[k] ? p->channel_depth[k] : p->depth;
		if(d > 0 && d < overall) iw_set_output_max_color_code(ctx, k, (1 << d) - 1);
	}
}

/* Output size (src/imagew-cmd.c:805-982; PNM files carry no density, so no
 * density adjustment applies). */
static void output_size(struct params *p, int src_w, int src_h, int *dst_w, int *dst_h)
{
	if(p->noresize) {
		p->dst_w_req = src_w;
		p->dst_h_req = src_h;
		p->rel_flag[0] = p->rel_flag[1] = 0;
		p->bestfit = 0;
	}
	*dst_w = p->dst_w_req < 0 ? -1 : (p->dst_w_req == 0 ? 1 : p->dst_w_req);
	*dst_h = p->dst_h_req < 0 ? -1 : (p->dst_h_req == 0 ? 1 : p->dst_h_req);
	if(p->rel_flag[0]) { *dst_w = (int)(0.5 + p->rel[0] * src_w); if(*dst_w < 1) *dst_w = 1; }
	if(p->rel_flag[1]) { *dst_h = (int)(0.5 + p->rel[1] * src_h); if(*dst_h < 1) *dst_h = 1; }
	if(*dst_w == -1 && *dst_h == -1) { *dst_w = src_w; *dst_h = src_h; }
	else if(*dst_h == -1) { *dst_h = 1000000; bestfit(src_w, src_h, dst_w, dst_h); }
	else if(*dst_w == -1) { *dst_w = 1000000; bestfit(src_w, src_h, dst_w, dst_h); }
	else if(p->bestfit) bestfit(src_w, src_h, dst_w, dst_h);
	if(*dst_w < 1) *dst_w = 1;
	if(*dst_h < 1) *dst_h = 1;
}

/* The reference's order of calls (src/imagew-cmd.c:1046-1479): options and
 * processing values, read, reorient, output profile and depths, colour
 * spaces, dither, colour counts, grayscale, channel offsets, background,
 * crop, size, translation, filters, canvas, process, write. */
static int run(struct params *p)
{
	struct iw_init_params ip;
	struct iw_context *ctx;
	FILE *f = NULL;
	int ok = 0, k, src_w, src_h, dst_w, dst_h;
	char msg[200];

	memset(&ip, 0, sizeof(ip));
	ip.api_version = IW_VERSION_INT;
	ip.userdata = p;
	ctx = iw_create_context(&ip);
	if(!ctx) { fprintf(stderr, "imagew error: cannot create a context\n"); return 0; }
	iw_set_warning_fn(ctx, warn_fn);

	if(p->outfmt == IW_FORMAT_UNKNOWN) p->outfmt = iw_detect_fmt_from_filename(p->out);
	if(!is_pnm_family(p->outfmt)) {
		iw_set_error(ctx, p->outfmt == IW_FORMAT_UNKNOWN ? "Unknown output format; use -outfmt." :
		                                                     "Writing this format is not supported by imagew_gb300.");
		goto done;
	}
	for(k = 0; k < p->nopts; k++) iw_set_option(ctx, p->opts[k].name, p->opts[k].val);
	if(p->random_seed != 0 || p->randomize) iw_set_random_seed(ctx, p->randomize, p->random_seed);
	if(p->sample_type >= 0) iw_set_value(ctx, IW_VAL_OUTPUT_SAMPLE_TYPE, p->sample_type);
	if(p->nogamma) iw_set_value(ctx, IW_VAL_DISABLE_GAMMA, 1);
	if(p->intclamp) iw_set_value(ctx, IW_VAL_INT_CLAMP, 1);
	if(p->nocslabel) iw_set_value(ctx, IW_VAL_NO_CSLABEL, 1);
	for(k = IW_OPT_GRAYSCALE; k <= IW_OPT_BINARY_TRNS; k++)
		if(p->noopt[k]) iw_set_allow_opt(ctx, k, 0);
	if(p->edge[0] >= 0) iw_set_value(ctx, IW_VAL_EDGE_POLICY_X, p->edge[0]);
	if(p->edge[1] >= 0) iw_set_value(ctx, IW_VAL_EDGE_POLICY_Y, p->edge[1]);
	if(p->gsf >= 0) {
		iw_set_value(ctx, IW_VAL_GRAYSCALE_FORMULA, p->gsf);
		if(p->gsf == IW_GSF_WEIGHTED || p->gsf == IW_GSF_ORDERBYVALUE)
			iw_set_grayscale_weights(ctx, p->gsf_w[0], p->gsf_w[1], p->gsf_w[2]);
	}
	if(p->negate) iw_set_value(ctx, IW_VAL_NEGATE_TARGET, 1);

	/* a forced input format: the reference's reader dispatch takes "pnm"
	 * and "pam" for these files and no other PNM name (src/imagew-allfmts.c:55-85) */
	if(p->infmt == IW_FORMAT_PPM || p->infmt == IW_FORMAT_PGM || p->infmt == IW_FORMAT_PBM) {
		iw_set_errorf(ctx, "Attempt to read unknown file format (%d)", p->infmt);
		goto done;
	}
	if(p->infmt != IW_FORMAT_UNKNOWN && !is_pnm_family(p->infmt)) {
		iw_set_error(ctx, "Reading this format is not supported by imagew_gb300.");
		goto done;
	}
	f = fopen(p->in, "rb");
	if(!f) { iw_set_errorf(ctx, "Failed to open %s for reading", p->in); goto done; }
	if(!pnm_read(ctx, f)) goto done;
	fclose(f);
	f = NULL;
	if(p->reorient) iw_reorient_image(ctx, p->reorient);

	iw_set_output_profile(ctx, iw_get_profile_by_fmt(p->outfmt));
	set_depths(p, ctx);
	if(p->cs_in_set) iw_set_input_colorspace(ctx, &p->cs_in);
	if(p->cs_out_set) iw_set_output_colorspace(ctx, &p->cs_out);
	if(p->intent != IW_INTENT_UNKNOWN) iw_set_value(ctx, IW_VAL_INTENT, p->intent);
	if(p->dither_all.fam >= 0) iw_set_dither_type(ctx, IW_CHANNELTYPE_ALL, p->dither_all.fam, p->dither_all.sub);
	if(p->dither_nonalpha.fam >= 0)
		iw_set_dither_type(ctx, IW_CHANNELTYPE_NONALPHA, p->dither_nonalpha.fam, p->dither_nonalpha.sub);
	for(k = 0; k < 5; k++)
		if(p->dither[k].fam >= 0) iw_set_dither_type(ctx, k, p->dither[k].fam, p->dither[k].sub);
	if(p->outfmt == IW_FORMAT_PBM) p->cc_all = 2;   /* bi-level */
	if(p->cc_all) iw_set_color_count(ctx, IW_CHANNELTYPE_ALL, p->cc_all);
	if(p->cc_nonalpha) iw_set_color_count(ctx, IW_CHANNELTYPE_NONALPHA, p->cc_nonalpha);
	for(k = 0; k < 5; k++)
		if(p->cc[k]) iw_set_color_count(ctx, k, p->cc[k]);
	if(p->outfmt == IW_FORMAT_PGM || p->outfmt == IW_FORMAT_PBM) { p->grayscale = 1; p->condgrayscale = 0; }
	if(p->condgrayscale) {
		if(iw_get_value(ctx, IW_VAL_INPUT_NATIVE_GRAYSCALE)) iw_set_value(ctx, IW_VAL_CVT_TO_GRAYSCALE, 1);
	}
	else if(p->grayscale) iw_set_value(ctx, IW_VAL_CVT_TO_GRAYSCALE, 1);
	for(k = 0; k < 3; k++) {
		if(p->offset_h[k] != 0.0) iw_set_channel_offset(ctx, k, IW_DIMENSION_H, p->offset_h[k]);
		if(p->offset_v[k] != 0.0) iw_set_channel_offset(ctx, k, IW_DIMENSION_V, p->offset_v[k]);
	}
	if(p->apply_bkgd) {   /* the colours are given in sRGB; the library takes linear ones */
		if(!p->nogamma) {
			struct iw_csdescr srgb;
			iw_make_srgb_csdescr_2(&srgb);
			for(k = 0; k < 3; k++) {
				p->bkgd.c[k] = iw_convert_sample_to_linear(p->bkgd.c[k], &srgb);
				if(p->checkerboard) p->bkgd2.c[k] = iw_convert_sample_to_linear(p->bkgd2.c[k], &srgb);
			}
		}
		iw_set_apply_bkgd_2(ctx, &p->bkgd);
		if(p->checkerboard) {
			iw_set_bkgd_checkerboard_2(ctx, p->check_size, &p->bkgd2);
			iw_set_bkgd_checkerboard_origin(ctx, p->check_x, p->check_y);
		}
	}
	if(p->use_bkgd_label) iw_set_value(ctx, IW_VAL_USE_BKGD_LABEL, 1);
	if(p->no_bkgd_label) iw_set_value(ctx, IW_VAL_NO_BKGD_LABEL, 1);
	else if(p->bkgd_label_set) iw_set_output_bkgd_label_2(ctx, &p->bkgd_label);

	src_w = iw_get_value(ctx, IW_VAL_INPUT_WIDTH);
	src_h = iw_get_value(ctx, IW_VAL_INPUT_HEIGHT);
	if(p->use_crop) {   /* src/imagew-cmd.c:1311-1325 */
		if(p->crop_x < 0) p->crop_x = 0;
		if(p->crop_y < 0) p->crop_y = 0;
		if(p->crop_x > src_w - 1) p->crop_x = src_w - 1;
		if(p->crop_y > src_h - 1) p->crop_y = src_h - 1;
		if(p->crop_w < 0 || p->crop_w > src_w - p->crop_x) p->crop_w = src_w - p->crop_x;
		if(p->crop_h < 0 || p->crop_h > src_h - p->crop_y) p->crop_h = src_h - p->crop_y;
		if(p->crop_w < 1) p->crop_w = 1;
		if(p->crop_h < 1) p->crop_h = 1;
		src_w = p->crop_w;
		src_h = p->crop_h;
	}
	output_size(p, src_w, src_h, &dst_w, &dst_h);

	if((p->edge[0] != IW_EDGE_POLICY_REPLICATE && p->edge[0] != IW_EDGE_POLICY_TRANSPARENT) ||
	   (p->edge[1] != IW_EDGE_POLICY_REPLICATE && p->edge[1] != IW_EDGE_POLICY_TRANSPARENT)) {
		if(p->imagesize_set) iw_warning(ctx, "\xe2\x80\x9c-edge t\xe2\x80\x9d is recommended when using -imagesize");
		else if(p->translate_set) iw_warning(ctx, "\xe2\x80\x9c-edge t\xe2\x80\x9d is recommended when using -translate");
	}
	if(p->translate_set) {
		if(p->translate_src) {   /* given in input pixels */
			if(p->translate_x != 0.0) p->translate_x *= (double)dst_w / src_w;
			if(p->translate_y != 0.0) p->translate_y *= (double)dst_h / src_h;
		}
		iw_set_value_dbl(ctx, IW_VAL_TRANSLATE_X, p->translate_x);
		iw_set_value_dbl(ctx, IW_VAL_TRANSLATE_Y, p->translate_y);
	}

	{
		int told = 0;   /* the notice is printed once */
		for(k = 0; k < 2; k++)
			if(p->blur_set[k] && !p->fam[k]) {
				if(!p->nowarn && !told) fprintf(stderr, "Notice: Selecting gaussian filter for blurring\n");
				told = 1;
				p->fam[k] = IW_RESIZETYPE_GAUSSIAN;
			}
	}
	for(k = 0; k < 2; k++) {   /* k = 0: horizontal, 1: vertical */
		const int s = k == 0 ? src_w : src_h, d = k == 0 ? dst_w : dst_h;
		if(!p->fam[k]) continue;
		if(p->blur_interp[k] && d < s) p->blur[k] *= (double)d / s;   /* interpolation: sharpen when downscaling */
		iw_set_resize_alg(ctx, k == 0 ? IW_DIMENSION_H : IW_DIMENSION_V, p->fam[k], p->blur[k], p->p1[k], p->p2[k]);
	}
	if(!p->noinfo) {
		if(dst_w == src_w && dst_h == src_h) printf("Processing: %d\xc3\x97%d\n", dst_w, dst_h);
		else printf("Resizing: %d\xc3\x97%d \xe2\x86\x92 %d\xc3\x97%d\n", src_w, src_h, dst_w, dst_h);
	}
	iw_set_output_canvas_size(ctx, dst_w, dst_h);
	if(p->imagesize_set) iw_set_output_image_size(ctx, p->imagesize_x, p->imagesize_y);
	if(p->use_crop) iw_set_input_crop(ctx, p->crop_x, p->crop_y, p->crop_w, p->crop_h);

	if(!iw_process_image(ctx)) goto done;

	f = fopen(p->out, "wb");
	if(!f) { iw_set_errorf(ctx, "Failed to open %s for writing", p->out); goto done; }
	if(!pnm_write(ctx, f, p->outfmt)) goto done;
	if(fclose(f) != 0) { f = NULL; iw_set_error(ctx, "Failed to write file"); goto done; }
	f = NULL;
	ok = 1;

done:
	if(f) fclose(f);
	if(iw_get_errorflag(ctx)) fprintf(stderr, "imagew error: %s\n", iw_get_errormsg(ctx, msg, sizeof(msg)));
	iw_destroy_context(ctx);
	return ok;
}

static int usage(void)
{
	fprintf(stderr, "Usage: imagew_gb300 [options] <infile> <outfile>\n"
		"PNM (PGM/PPM, binary) and PAM files; see the source header for the options.\n");
	return 1;
}

/* A width or height: pixels, or "x<factor>" relative to the input
 * (src/imagew-cmd.c:2302-2315). */
static void parse_w_or_h(struct params *p, const char *v, int k)
{
	if(v[0] == 'x') { p->rel_flag[k] = 1; p->rel[k] = iw_parse_number(v + 1); }
	else if(k == 0) p->dst_w_req = iw_parse_int(v);
	else p->dst_h_req = iw_parse_int(v);
}

static int flag_option(struct params *p, const char *o)
{
	static const char *const no_effect[] = {"interlace", "jpegarith", "bmptrns", "includescreen", "noincludescreen",
	                                        "msgstostdout", "msgstostderr", NULL};
	int k;
	if(!strcmp(o, "bestfit")) p->bestfit_option = 1;
	else if(!strcmp(o, "nobestfit")) p->bestfit_option = 0;
	else if(!strcmp(o, "noresize")) p->noresize = 1;
	else if(!strcmp(o, "grayscale")) p->grayscale = 1;
	else if(!strcmp(o, "condgrayscale")) p->condgrayscale = 1;
	else if(!strcmp(o, "nogamma")) p->nogamma = 1;
	else if(!strcmp(o, "intclamp")) p->intclamp = 1;
	else if(!strcmp(o, "nocslabel")) p->nocslabel = 1;
	else if(!strcmp(o, "usebkgdlabel")) p->use_bkgd_label = 1;
	else if(!strcmp(o, "nobkgdlabel")) p->no_bkgd_label = 1;
	else if(!strcmp(o, "negate")) p->negate = 1;
	else if(!strcmp(o, "noinfo")) p->noinfo = 1;
	else if(!strcmp(o, "nowarn")) p->nowarn = 1;
	else if(!strcmp(o, "quiet")) p->noinfo = p->nowarn = 1;
	else {
		for(k = 0; no_effect[k]; k++)
			if(!strcmp(o, no_effect[k])) return 1;
		return 0;
	}
	return 1;
}

/* An option with a value; 0 after printing an error. */
static int value_option(struct params *p, const char *o, const char *v)
{
	static const char *const no_effect[] = {"precision", "colortype", "page", "jpegquality", "jpegsampling",
	                                        "webpquality", "zipcmprlevel", "pngcmprlevel", "bmpversion", NULL};
	int k;
	if(!strcmp(o, "w") || !strcmp(o, "width")) parse_w_or_h(p, v, 0);
	else if(!strcmp(o, "h") || !strcmp(o, "height")) parse_w_or_h(p, v, 1);
	else if(!strcmp(o, "s") || !strcmp(o, "S")) {
		const char *comma = strchr(v, ',');
		if(!comma) { fprintf(stderr, "Bad size option\n"); return 0; }
		parse_w_or_h(p, v, 0);
		parse_w_or_h(p, comma + 1, 1);
		p->bestfit = o[0] == 's';
	}
	else if(!strncmp(o, "filter", 6) && (!o[6] || ((o[6] == 'x' || o[6] == 'y') && !o[7]))) {
		int fam = 0;
		double a1, a2;
		if(!decode_filter(v, &fam, &a1, &a2)) { fprintf(stderr, "Unknown resize type \xe2\x80\x9c%s\xe2\x80\x9d\n", v); return 0; }
		for(k = 0; k < 2; k++)
			if(o[6] == '\0' || (o[6] == 'x' && k == 0) || (o[6] == 'y' && k == 1)) {
				p->fam[k] = fam;
				p->p1[k] = a1;
				p->p2[k] = a2;
			}
	}
	else if(!strncmp(o, "blur", 4) && (!o[4] || ((o[4] == 'x' || o[4] == 'y') && !o[5]))) {
		const int interp = name_len(v) == 1 && v[0] == 'x';   /* "x[F]": interpolate */
		const double b = interp ? (v[1] ? iw_parse_number(v + 1) : 1.0) : iw_parse_number(v);
		for(k = 0; k < 2; k++)
			if(o[4] == '\0' || (o[4] == 'x' && k == 0) || (o[4] == 'y' && k == 1)) {
				p->blur[k] = b;
				p->blur_set[k] = 1;
				p->blur_interp[k] = interp;
			}
	}
	else if(!strncmp(o, "edge", 4) && (!o[4] || ((o[4] == 'x' || o[4] == 'y') && !o[5]))) {
		const int e = v[0] == 's' ? IW_EDGE_POLICY_STANDARD : (v[0] == 'r' ? IW_EDGE_POLICY_REPLICATE :
			(v[0] == 't' ? IW_EDGE_POLICY_TRANSPARENT : -1));
		if(e < 0) { fprintf(stderr, "Unknown edge policy\n"); return 0; }
		if(o[4] != 'y') p->edge[0] = e;
		if(o[4] != 'x') p->edge[1] = e;
	}
	else if(!strcmp(o, "translate")) {
		p->translate_src = v[0] == 's';
		parse_dbl_pair(v + p->translate_src, &p->translate_x, &p->translate_y);
		p->translate_set = 1;
	}
	else if(!strcmp(o, "imagesize")) {
		parse_dbl_pair(v, &p->imagesize_x, &p->imagesize_y);
		if(p->imagesize_x > 0.0 && p->imagesize_y > 0.0) p->imagesize_set = 1;
	}
	else if(!strncmp(o, "offset", 6)) {
		const int vert = o[6] == 'v';
		double *off = vert ? p->offset_v : p->offset_h;
		const char *ch = o + 6 + vert;
		if(!strcmp(ch, "rb")) { off[IW_CHANNELTYPE_RED] = iw_parse_number(v); off[IW_CHANNELTYPE_BLUE] = -off[IW_CHANNELTYPE_RED]; }
		else {
			k = channel_suffix(ch);
			if(k < 0 || k > IW_CHANNELTYPE_BLUE) { fprintf(stderr, "Unknown option \xe2\x80\x9c%s\xe2\x80\x9d\n", o); return 0; }
			off[k] = iw_parse_number(v);
		}
	}
	else if(!strcmp(o, "depth")) {
		if(strchr(v, ',')) parse_ints(v, p->channel_depth, 4);   /* R,G,B,A */
		else p->depth = iw_parse_int(v);
	}
	else if(!strcmp(o, "depthcc")) p->depthcc = iw_parse_int(v);
	else if(!strcmp(o, "depthgray")) p->channel_depth[IW_CHANNELTYPE_GRAY] = iw_parse_int(v);
	else if(!strcmp(o, "depthalpha")) p->channel_depth[IW_CHANNELTYPE_ALPHA] = iw_parse_int(v);
	else if(!strcmp(o, "sampletype")) {
		if(v[0] == 'u') p->sample_type = IW_SAMPLETYPE_UINT;
		else if(v[0] == 'f') p->sample_type = IW_SAMPLETYPE_FLOATINGPOINT;
		else { fprintf(stderr, "Unknown sample type \xe2\x80\x9c%s\xe2\x80\x9d\n", v); return 0; }
	}
	else if(!strcmp(o, "cc")) {
		if(strchr(v, ',')) parse_ints(v, p->cc, 4);   /* R,G,B,A */
		else p->cc_all = iw_parse_int(v);
	}
	else if(!strcmp(o, "cccolor")) p->cc_nonalpha = iw_parse_int(v);
	else if(!strncmp(o, "cc", 2) && channel_suffix(o + 2) >= 0) p->cc[channel_suffix(o + 2)] = iw_parse_int(v);
	else if(!strncmp(o, "dither", 6)) {
		struct dither_req *d = !o[6] ? &p->dither_all : (!strcmp(o + 6, "color") ? &p->dither_nonalpha :
			(channel_suffix(o + 6) >= 0 ? &p->dither[channel_suffix(o + 6)] : NULL));
		if(!d) { fprintf(stderr, "Unknown option \xe2\x80\x9c%s\xe2\x80\x9d\n", o); return 0; }
		if(!decode_dither(v, &d->fam, &d->sub)) { fprintf(stderr, "Unknown dither type \xe2\x80\x9c%s\xe2\x80\x9d\n", v); return 0; }
	}
	else if(!strcmp(o, "gsf") || !strcmp(o, "grayscaleformula")) {
		if(!decode_gsf(v, &p->gsf, p->gsf_w)) { fprintf(stderr, "Invalid grayscale formula\n"); return 0; }
		p->grayscale = 1;
	}
	else if(!strcmp(o, "cs") || !strcmp(o, "inputcs")) {
		const int in = o[0] == 'i';
		if(!decode_cs(v, in ? &p->cs_in : &p->cs_out, &p->intent)) {
			fprintf(stderr, "Unknown color space \xe2\x80\x9c%s\xe2\x80\x9d\n", v);
			return 0;
		}
		if(in) p->cs_in_set = 1;
		else p->cs_out_set = 1;
	}
	else if(!strcmp(o, "intent")) {
		if(!decode_intent(v, &p->intent)) { fprintf(stderr, "Unknown intent \xe2\x80\x9c%s\xe2\x80\x9d\n", v); return 0; }
	}
	else if(!strcmp(o, "noopt")) {
		if(!decode_noopt(v, p->noopt)) { fprintf(stderr, "Unknown optimization \xe2\x80\x9c%s\xe2\x80\x9d\n", v); return 0; }
	}
	else if(!strcmp(o, "randseed")) {
		if(v[0] == 'r') p->randomize = 1;
		else p->random_seed = iw_parse_int(v);
	}
	else if(!strcmp(o, "bkgd")) {
		const char *comma = strchr(v, ',');
		p->apply_bkgd = 1;
		if(!comma) parse_color(&p->bkgd, v, strlen(v));
		else {   /* two colours: a checkerboard */
			p->checkerboard = 1;
			parse_color(&p->bkgd, v, (size_t)(comma - v));
			parse_color(&p->bkgd2, comma + 1, strlen(comma + 1));
		}
	}
	else if(!strcmp(o, "bkgdlabel")) {
		struct iw_csdescr srgb;
		parse_color(&p->bkgd_label, v, strlen(v));
		iw_make_srgb_csdescr_2(&srgb);
		for(k = 0; k < 3; k++) p->bkgd_label.c[k] = iw_convert_sample_to_linear(p->bkgd_label.c[k], &srgb);
		p->bkgd_label_set = 1;
	}
	else if(!strcmp(o, "checkersize")) p->check_size = iw_parse_int(v);
	else if(!strcmp(o, "checkerorigin")) {
		int xy[2] = {p->check_x, p->check_y};
		parse_ints(v, xy, 2);
		p->check_x = xy[0];
		p->check_y = xy[1];
	}
	else if(!strcmp(o, "reorient")) {
		if(!decode_reorient(v, &p->reorient)) {
			fprintf(stderr, "Unknown orientation transform \xe2\x80\x9c%s\xe2\x80\x9d\n", v);
			return 0;
		}
	}
	else if(!strcmp(o, "crop")) {
		int c[4] = {0, 0, -1, -1};
		parse_ints(v, c, 4);
		p->crop_x = c[0]; p->crop_y = c[1]; p->crop_w = c[2]; p->crop_h = c[3];
		p->use_crop = 1;
	}
	else if(!strcmp(o, "infmt") || !strcmp(o, "outfmt")) {
		const int fmt = decode_fmt(v);
		if(fmt == IW_FORMAT_UNKNOWN) { fprintf(stderr, "Unknown format \xe2\x80\x9c%s\xe2\x80\x9d\n", v); return 0; }
		if(o[0] == 'i') p->infmt = fmt;
		else p->outfmt = fmt;
	}
	else if(!strcmp(o, "compress")) {
		if(strcmp(v, "none") && strcmp(v, "zip") && strcmp(v, "lzw") && strcmp(v, "jpeg") && strcmp(v, "rle")) {
			fprintf(stderr, "Unknown compression \xe2\x80\x9c%s\xe2\x80\x9d\n", v);
			return 0;
		}
	}
	else if(!strcmp(o, "density")) {
		const int nl = name_len(v);
		if(!(nl == 1 && (v[0] == 'i' || v[0] == 'c')) && strcmp(v, "auto") && strcmp(v, "none") && strcmp(v, "keep") &&
		   strcmp(v, "adjust")) {
			fprintf(stderr, "Invalid density \xe2\x80\x9c%s\xe2\x80\x9d\n", v);
			return 0;
		}
	}
	else if(!strcmp(o, "encoding")) {
		if(strcmp(v, "auto") && strcmp(v, "ascii") && strcmp(v, "utf8")) {
			fprintf(stderr, "Unknown encoding \xe2\x80\x9c%s\xe2\x80\x9d\n", v);
			return 0;
		}
	}
	else if(!strcmp(o, "opt")) {   /* NAME=VALUE; NAME alone: an empty value */
		const char *eq = strchr(v, '=');
		if(p->nopts >= 32) { fprintf(stderr, "Too many -opt options\n"); return 0; }
		p->opts[p->nopts].name = strdup(v);
		if(eq) { p->opts[p->nopts].name[eq - v] = '\0'; p->opts[p->nopts].val = strdup(eq + 1); }
		else p->opts[p->nopts].val = strdup("");
		p->nopts++;
	}
	else {
		for(k = 0; no_effect[k]; k++)
			if(!strcmp(o, no_effect[k])) return 1;
		fprintf(stderr, "Unknown option \xe2\x80\x9c%s\xe2\x80\x9d\n", o);
		return 0;
	}
	return 1;
}

/* Options with a value, by name (src/imagew-cmd.c:2107-2198). */
static int takes_value(const char *o)
{
	static const char *const names[] = {
		"w", "width", "h", "height", "s", "S", "opt", "precision", "depth", "depthcc", "depthgray", "depthalpha",
		"sampletype", "inputcs", "cs", "filter", "filterx", "filtery", "blur", "blurx", "blury", "dither",
		"dithercolor", "ditheralpha", "ditherred", "dithergreen", "ditherblue", "dithergray", "cc", "cccolor",
		"ccalpha", "ccred", "ccgreen", "ccblue", "ccgray", "bkgd", "bkgdlabel", "checkersize", "checkerorigin",
		"crop", "reorient", "offsetred", "offsetgreen", "offsetblue", "offsetrb", "offsetvred", "offsetvgreen",
		"offsetvblue", "offsetvrb", "translate", "imagesize", "compress", "colortype", "page", "jpegquality",
		"jpegsampling", "webpquality", "zipcmprlevel", "pngcmprlevel", "bmpversion", "randseed", "infmt", "outfmt",
		"edge", "edgex", "edgey", "density", "gsf", "grayscaleformula", "intent", "noopt", "encoding", NULL};
	int k;
	for(k = 0; names[k]; k++)
		if(!strcmp(o, names[k])) return 1;
	return 0;
}

int main(int argc, char **argv)
{
	struct params p;
	int i, k, nfiles = 0;
	memset(&p, 0, sizeof(p));
	p.infmt = p.outfmt = IW_FORMAT_UNKNOWN;
	p.dst_w_req = p.dst_h_req = -1;
	p.edge[0] = p.edge[1] = -1;
	p.blur[0] = p.blur[1] = 1.0;
	p.bestfit_option = -1;
	p.sample_type = -1;
	p.gsf = -1;
	p.check_size = 16;
	p.dither_all.fam = p.dither_nonalpha.fam = -1;
	for(k = 0; k < 5; k++) p.dither[k].fam = -1;
	for(i = 1; i < argc; i++) {
		const char *a = argv[i];
		if(a[0] == '-' && a[1]) {
			const char *o = a + 1;
			if(o[0] == '-') o++;
			if(!strcmp(o, "help")) { printf("Usage: imagew_gb300 [-w <width>] [-h <height>] [options] <in-file> <out-file>\n"); return 0; }
			if(!strcmp(o, "version")) {
				char ver[32];
				iw_get_version_string(NULL, ver, (int)sizeof(ver));
				printf("imagew_gb300 (ImageWorsener %s interface)\n", ver);
				return 0;
			}
			if(takes_value(o)) {
				if(i + 1 >= argc) return usage();
				if(!value_option(&p, o, argv[++i])) return 1;
			}
			else if(!flag_option(&p, o)) { fprintf(stderr, "Unknown option \xe2\x80\x9c%s\xe2\x80\x9d\n", o); return 1; }
			continue;
		}
		if(nfiles == 0) p.in = a;
		else if(nfiles == 1) p.out = a;
		nfiles++;
	}
	if(nfiles != 2) return usage();
	if(p.bestfit_option >= 0) p.bestfit = p.bestfit_option;   /* wherever -bestfit / -nobestfit stood */
	if(!p.noinfo) printf("%s \xe2\x86\x92 %s\n", p.in, p.out);
	k = run(&p) ? 0 : 1;
	for(i = 0; i < p.nopts; i++) { free(p.opts[i].name); free(p.opts[i].val); }
	return k;
}
