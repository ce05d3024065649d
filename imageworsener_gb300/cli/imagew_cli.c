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
 *   -w, -width N; -h, -height N     output size (one of them: keep the aspect
 *                                   ratio); -bestfit: fit inside N x M;
 *                                   -noresize: keep the input size
 *   -filter, -filterx, -filtery F   resampling filter: mix nearest point linear
 *                                   triangle quadratic hermite box boxavg
 *                                   gaussian auto null lanczos[N] hann[N]
 *                                   hanning[N] blackman[N] sinc[N] catrom
 *                                   mitchell bspline cubicB,C keys[A]
 *   -blur, -blurx, -blury X         filter blur factor (alone: gaussian)
 *   -edge, -edgex, -edgey s|r|t     edge policy (standard, replicate, transparent)
 *   -depth N                        output bits per sample
 *   -cc N                           colours per channel
 *   -dither D                       f fs o halftone r r2 jjn stucki burkes
 *                                   sierra sierra3 sierra2 sierralite atkinson none
 *   -grayscale                      convert to grayscale
 *   -crop X,Y[,W,H]                 use part of the input
 *   -outfmt pam|ppm|pgm|pnm         output format (default: from the file name)
 *   -opt NAME=VALUE                 iw_set_option(), e.g. gpu:precision=fp64
 *   -noinfo, -quiet, -nowarn        messages
 */
#define IW_INCLUDE_UTIL_FUNCTIONS
#include "imagew.h"
#include "pnm.h"

#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

struct opt_kv { char *name, *val; };

struct params {
	const char *in, *out;
	int outfmt;
	int dst_w_req, dst_h_req, bestfit, noresize;
	int fam[2];                  /* resize family per dimension (0: library default) */
	double p1[2], p2[2], blur[2];
	int blur_set[2];
	int edge[2];
	int depth, cc, grayscale;
	int dither_fam, dither_sub;
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

/* Resize-algorithm names (src/imagew-cmd.c:1622-1736). */
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

/* Dither names (src/imagew-cmd.c:1769-1786). */
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

static int decode_outfmt(const char *s)
{
	if(!strcmp(s, "pam")) return IW_FORMAT_PAM;
	if(!strcmp(s, "ppm")) return IW_FORMAT_PPM;
	if(!strcmp(s, "pgm")) return IW_FORMAT_PGM;
	if(!strcmp(s, "pnm")) return IW_FORMAT_PNM;
	return IW_FORMAT_UNKNOWN;
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
	if(p->outfmt != IW_FORMAT_PNM && p->outfmt != IW_FORMAT_PPM && p->outfmt != IW_FORMAT_PGM && p->outfmt != IW_FORMAT_PAM) {
		iw_set_error(ctx, p->outfmt == IW_FORMAT_UNKNOWN ? "Unknown output format; use -outfmt." :
		                                                     "Writing this format is not supported by imagew_gb300.");
		goto done;
	}
	for(k = 0; k < p->nopts; k++) iw_set_option(ctx, p->opts[k].name, p->opts[k].val);

	f = fopen(p->in, "rb");
	if(!f) { iw_set_errorf(ctx, "Failed to open %s for reading", p->in); goto done; }
	if(!pnm_read(ctx, f)) goto done;
	fclose(f);
	f = NULL;

	iw_set_output_profile(ctx, iw_get_profile_by_fmt(p->outfmt));
	if(p->depth) {   /* src/imagew-cmd.c:984-1040, -depth alone */
		const int overall = p->depth <= 8 ? 8 : 16;
		iw_set_output_depth(ctx, overall);
		if(p->depth < overall)
			for(k = 0; k < 5; k++) iw_set_output_max_color_code(ctx, k, (1 << p->depth) - 1);
	}
	if(p->dither_fam >= 0) iw_set_dither_type(ctx, IW_CHANNELTYPE_ALL, p->dither_fam, p->dither_sub);
	if(p->cc) iw_set_color_count(ctx, IW_CHANNELTYPE_ALL, p->cc);
	if(p->outfmt == IW_FORMAT_PGM) p->grayscale = 1;
	if(p->grayscale) iw_set_value(ctx, IW_VAL_CVT_TO_GRAYSCALE, 1);
	if(p->edge[0] >= 0) iw_set_value(ctx, IW_VAL_EDGE_POLICY_X, p->edge[0]);
	if(p->edge[1] >= 0) iw_set_value(ctx, IW_VAL_EDGE_POLICY_Y, p->edge[1]);

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

	/* output size (src/imagew-cmd.c:805-880; PNM files carry no density) */
	if(p->noresize) { p->dst_w_req = src_w; p->dst_h_req = src_h; p->bestfit = 0; }
	dst_w = p->dst_w_req < 0 ? -1 : (p->dst_w_req == 0 ? 1 : p->dst_w_req);
	dst_h = p->dst_h_req < 0 ? -1 : (p->dst_h_req == 0 ? 1 : p->dst_h_req);
	if(dst_w == -1 && dst_h == -1) { dst_w = src_w; dst_h = src_h; }
	else if(dst_h == -1) { dst_h = 1000000; bestfit(src_w, src_h, &dst_w, &dst_h); }
	else if(dst_w == -1) { dst_w = 1000000; bestfit(src_w, src_h, &dst_w, &dst_h); }
	else if(p->bestfit) bestfit(src_w, src_h, &dst_w, &dst_h);

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
		if(p->fam[k]) iw_set_resize_alg(ctx, k == 0 ? IW_DIMENSION_H : IW_DIMENSION_V, p->fam[k], p->blur[k], p->p1[k], p->p2[k]);
	}
	if(!p->noinfo) {
		if(dst_w == src_w && dst_h == src_h) printf("Processing: %d\xc3\x97%d\n", dst_w, dst_h);
		else printf("Resizing: %d\xc3\x97%d \xe2\x86\x92 %d\xc3\x97%d\n", src_w, src_h, dst_w, dst_h);
	}
	iw_set_output_canvas_size(ctx, dst_w, dst_h);
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

int main(int argc, char **argv)
{
	struct params p;
	int i, k, nfiles = 0;
	memset(&p, 0, sizeof(p));
	p.outfmt = IW_FORMAT_UNKNOWN;
	p.dst_w_req = p.dst_h_req = -1;
	p.edge[0] = p.edge[1] = -1;
	p.blur[0] = p.blur[1] = 1.0;
	p.dither_fam = -1;
	for(i = 1; i < argc; i++) {
		const char *a = argv[i];
		if(a[0] == '-' && a[1]) {
			const char *o = a + 1, *v = NULL;
			if(o[0] == '-') o++;
			/* options without a value */
			if(!strcmp(o, "bestfit")) { p.bestfit = 1; continue; }
			if(!strcmp(o, "noresize")) { p.noresize = 1; continue; }
			if(!strcmp(o, "grayscale")) { p.grayscale = 1; continue; }
			if(!strcmp(o, "noinfo") || !strcmp(o, "quiet")) { p.noinfo = 1; if(o[0] == 'q') p.nowarn = 1; continue; }
			if(!strcmp(o, "nowarn")) { p.nowarn = 1; continue; }
			if(i + 1 >= argc) { fprintf(stderr, "Option %s needs a value\n", a); return 1; }
			v = argv[++i];
			if(!strcmp(o, "w") || !strcmp(o, "width")) p.dst_w_req = atoi(v);
			else if(!strcmp(o, "h") || !strcmp(o, "height")) p.dst_h_req = atoi(v);
			else if(!strcmp(o, "filter") || !strcmp(o, "filterx") || !strcmp(o, "filtery")) {
				int fam = 0;
				double a1, a2;
				if(!decode_filter(v, &fam, &a1, &a2)) {
					fprintf(stderr, "Unknown resize type \xe2\x80\x9c%s\xe2\x80\x9d\n", v);
					return 1;
				}
				for(k = 0; k < 2; k++)
					if(o[6] == '\0' || (o[6] == 'x' && k == 0) || (o[6] == 'y' && k == 1)) {
						p.fam[k] = fam;
						p.p1[k] = a1;
						p.p2[k] = a2;
					}
			}
			else if(!strcmp(o, "blur") || !strcmp(o, "blurx") || !strcmp(o, "blury")) {
				for(k = 0; k < 2; k++)
					if(o[4] == '\0' || (o[4] == 'x' && k == 0) || (o[4] == 'y' && k == 1)) {
						p.blur[k] = atof(v);
						p.blur_set[k] = 1;
					}
			}
			else if(!strcmp(o, "edge") || !strcmp(o, "edgex") || !strcmp(o, "edgey")) {
				const int e = v[0] == 's' ? IW_EDGE_POLICY_STANDARD : (v[0] == 'r' ? IW_EDGE_POLICY_REPLICATE :
					(v[0] == 't' ? IW_EDGE_POLICY_TRANSPARENT : -1));
				if(e < 0) { fprintf(stderr, "Unknown edge policy\n"); return 1; }
				if(o[4] != 'y') p.edge[0] = e;
				if(o[4] != 'x') p.edge[1] = e;
			}
			else if(!strcmp(o, "depth")) p.depth = atoi(v);
			else if(!strcmp(o, "cc")) p.cc = atoi(v);
			else if(!strcmp(o, "dither")) {
				if(!decode_dither(v, &p.dither_fam, &p.dither_sub)) { fprintf(stderr, "Unknown dither type\n"); return 1; }
			}
			else if(!strcmp(o, "crop")) {
				double n[4];
				const int c = iw_parse_number_list(v, 4, n);
				p.crop_x = p.crop_y = 0;
				p.crop_w = p.crop_h = -1;
				if(c >= 1) p.crop_x = iw_round_to_int(n[0]);
				if(c >= 2) p.crop_y = iw_round_to_int(n[1]);
				if(c >= 3) p.crop_w = iw_round_to_int(n[2]);
				if(c >= 4) p.crop_h = iw_round_to_int(n[3]);
				p.use_crop = 1;
			}
			else if(!strcmp(o, "outfmt")) {
				p.outfmt = decode_outfmt(v);
				if(p.outfmt == IW_FORMAT_UNKNOWN) { fprintf(stderr, "Unknown format \xe2\x80\x9c%s\xe2\x80\x9d\n", v); return 1; }
			}
			else if(!strcmp(o, "opt")) {
				const char *eq = strchr(v, '=');
				if(p.nopts >= 32) { fprintf(stderr, "Too many -opt options\n"); return 1; }
				p.opts[p.nopts].name = strdup(v);
				if(eq) { p.opts[p.nopts].name[eq - v] = '\0'; p.opts[p.nopts].val = strdup(eq + 1); }
				else p.opts[p.nopts].val = strdup("1");
				p.nopts++;
			}
			else { fprintf(stderr, "Unknown option \xe2\x80\x9c%s\xe2\x80\x9d\n", a); return 1; }
			continue;
		}
		if(nfiles == 0) p.in = a;
		else if(nfiles == 1) p.out = a;
		nfiles++;
	}
	if(nfiles != 2) return usage();
	if(!p.noinfo) printf("%s \xe2\x86\x92 %s\n", p.in, p.out);
	k = run(&p) ? 0 : 1;
	for(i = 0; i < p.nopts; i++) { free(p.opts[i].name); free(p.opts[i].val); }
	return k;
}
