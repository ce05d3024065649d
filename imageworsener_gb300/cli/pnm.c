/*
 * pnm.c -- PNM (PBM/PGM/PPM, binary forms) and PAM image files for the
 * imagew_gb300 command-line tool, over the libimagew API only.
 *
 * Behaviour follows the reference's codec, ImageWorsener 1.3.5
 * src/imagew-pnm.c (a PNM output holding a two-entry gray palette is
 * written as PBM, :867-954):
 *   reading   P4, P5, P6 and P7 (PAM with DEPTH 1-4); MAXVAL below 256 gives
 *             8-bit samples, else 16-bit big-endian; a MAXVAL other than 255 or
 *             65535 becomes the input's max colour code (:109-222, :224-437);
 *   writing   P5 / P6 headers "P5\n<w> <h>\n<maxval>\n", PAM headers with
 *             WIDTH, HEIGHT, DEPTH, MAXVAL, TUPLTYPE, ENDHDR lines; reduced bit
 *             depths must be equal over the written channels; gray images
 *             written as PPM repeat the gray sample (:494-958).
 * The file layouts are the Netpbm formats; the code is this project's own.
 */
#include "pnm.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static int is_ws(int c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f'; }

/* Next whitespace-delimited token of a PNM header; '#' starts a comment that
 * runs to the end of the line.  The delimiter after the token is consumed. */
static int pnm_token(FILE *f, char *buf, int cap)
{
	int c, n = 0;
	for(;;) {
		c = fgetc(f);
		if(c == EOF) return 0;
		if(c == '#') {
			while(c != '\n' && c != EOF) c = fgetc(f);
			if(c == EOF) return 0;
			continue;
		}
		if(!is_ws(c)) break;
	}
	while(c != EOF && !is_ws(c)) {
		if(c == '#') {   /* a comment ends the token too */
			while(c != '\n' && c != EOF) c = fgetc(f);
			break;
		}
		if(n >= cap - 1) return 0;
		buf[n++] = (char)c;
		c = fgetc(f);
	}
	buf[n] = '\0';
	return n > 0;
}

/* One PAM header line (without its newline), truncated to cap-1 bytes. */
static int pam_line(FILE *f, char *buf, int cap)
{
	int c, n = 0;
	for(;;) {
		c = fgetc(f);
		if(c == EOF) { buf[n] = '\0'; return 0; }
		if(c == '\n') break;
		if(n < cap - 1) buf[n++] = (char)c;
	}
	buf[n] = '\0';
	return 1;
}

/* Splits the first two whitespace-separated words of a line. */
static void two_words(const char *line, char *w1, char *w2, int cap)
{
	int k;
	const char *p = line;
	w1[0] = w2[0] = '\0';
	while(*p && is_ws((unsigned char)*p)) p++;
	for(k = 0; *p && !is_ws((unsigned char)*p) && k < cap - 1; p++) w1[k++] = *p;
	w1[k] = '\0';
	while(*p && is_ws((unsigned char)*p)) p++;
	for(k = 0; *p && !is_ws((unsigned char)*p) && k < cap - 1; p++) w2[k++] = *p;
	w2[k] = '\0';
}

int pnm_read(struct iw_context *ctx, FILE *f)
{
	unsigned char sig[3];
	int code, w = 0, h = 0, maxval = 0, depth_pam = 0;
	char tok[100];
	struct iw_image img;
	int nch, bps, k;
	size_t bpr, total, j;

	if(fread(sig, 1, 3, f) != 3) { iw_set_error(ctx, "Error parsing header"); return 0; }
	if(sig[0] != 'P' || !((sig[1] == '7' && sig[2] == 0x0a) || (sig[1] >= '1' && sig[1] <= '6' && is_ws(sig[2])))) {
		iw_set_error(ctx, "Not a PNM/PAM file");
		iw_set_error(ctx, "Error parsing header");
		return 0;
	}
	code = sig[1] - '0';
	if(code == 7) {
		char line[100], a[100], b[100];
		for(;;) {
			if(!pam_line(f, line, sizeof(line))) { iw_set_error(ctx, "Error parsing header"); return 0; }
			if(line[0] == '#') continue;
			two_words(line, a, b, sizeof(a));
			if(!strcmp(a, "ENDHDR")) break;
			if(!a[0]) continue;
			if(!strcmp(a, "WIDTH")) w = atoi(b);
			else if(!strcmp(a, "HEIGHT")) h = atoi(b);
			else if(!strcmp(a, "DEPTH")) depth_pam = atoi(b);
			else if(!strcmp(a, "MAXVAL")) maxval = atoi(b);
		}
	}
	else {
		if(code != 4 && code != 5 && code != 6) {
			iw_set_error(ctx, "Reading this PNM format is not supported");
			iw_set_error(ctx, "Error parsing header");
			return 0;
		}
		if(!pnm_token(f, tok, sizeof(tok))) { iw_set_error(ctx, "Error parsing header"); return 0; }
		w = atoi(tok);
		if(!pnm_token(f, tok, sizeof(tok))) { iw_set_error(ctx, "Error parsing header"); return 0; }
		h = atoi(tok);
		if(code != 4) {
			if(!pnm_token(f, tok, sizeof(tok))) { iw_set_error(ctx, "Error parsing header"); return 0; }
			maxval = atoi(tok);
		}
	}
	if(code != 4 && (maxval < 1 || maxval > 65535)) {
		iw_set_errorf(ctx, "Invalid max color value (%d)\n", maxval);
		iw_set_error(ctx, "Error parsing header");
		return 0;
	}
	if(!iw_check_image_dimensions(ctx, w, h)) return 0;

	memset(&img, 0, sizeof(img));
	img.width = w;
	img.height = h;
	if(code == 4) {
		img.imgtype = IW_IMGTYPE_GRAY;
		img.native_grayscale = 1;
		img.bit_depth = 1;
		bpr = ((size_t)w + 7) / 8;
		nch = 0;
	}
	else {
		if(code == 5 || (code == 7 && depth_pam == 1)) { img.imgtype = IW_IMGTYPE_GRAY; img.native_grayscale = 1; nch = 1; }
		else if(code == 6 || (code == 7 && depth_pam == 3)) { img.imgtype = IW_IMGTYPE_RGB; nch = 3; }
		else if(code == 7 && depth_pam == 2) { img.imgtype = IW_IMGTYPE_GRAYA; nch = 2; }
		else if(code == 7 && depth_pam == 4) { img.imgtype = IW_IMGTYPE_RGBA; nch = 4; }
		else { iw_set_error(ctx, "Unsupported PNM/PAM image type"); return 0; }
		bps = maxval >= 256 ? 2 : 1;
		img.bit_depth = 8 * bps;
		bpr = (size_t)w * nch * bps;
		if(maxval != 255 && maxval != 65535)
			for(k = 0; k < nch; k++) iw_set_input_max_color_code(ctx, k, maxval);
	}
	img.bpr = (size_t)bpr;
	total = bpr * (size_t)h;
	img.pixels = (iw_byte *)iw_malloc_large(ctx, bpr, h);
	if(!img.pixels) return 0;
	if(fread(img.pixels, 1, total, f) != total) {
		iw_set_error(ctx, "Failed to read file");
		iw_free(ctx, img.pixels);
		return 0;
	}
	if(code == 4)
		for(j = 0; j < total; j++) img.pixels[j] = (iw_byte)(255 - img.pixels[j]);
	iw_set_input_image(ctx, &img);   /* the context owns the pixels now */
	return 1;
}

static int put(FILE *f, const void *p, size_t n) { return fwrite(p, 1, n, f) == n; }

/* A two-entry gray palette image (what PBM holds). */
static int bw_palette(struct iw_context *ctx, const struct iw_image *img)
{
	return img->imgtype == IW_IMGTYPE_PALETTE && iw_get_value(ctx, IW_VAL_OUTPUT_PALETTE_GRAYSCALE) &&
		iw_get_output_palette(ctx)->num_entries == 2;
}

static int header_pam(FILE *f, const struct iw_image *img, int depth, int maxval, const char *tupltype)
{
	return fprintf(f, "P7\nWIDTH %d\nHEIGHT %d\nDEPTH %d\nMAXVAL %d\nTUPLTYPE %s\nENDHDR\n", img->width, img->height,
		depth, maxval, tupltype) > 0;
}

/* The max colour code written for the given channels: the depth's, or the
 * reduced one, which must then be equal over them. */
static int written_maxval(struct iw_context *ctx, const struct iw_image *img, const int *chs, int n, const char *what)
{
	int m = img->bit_depth == 16 ? 65535 : 255, k;
	if(img->reduced_maxcolors) {
		m = (int)img->maxcolorcode[chs[0]];
		for(k = 1; k < n; k++)
			if((int)img->maxcolorcode[chs[k]] != m) { iw_set_error(ctx, what); return -1; }
	}
	if(m < 1 || m > 65535) { iw_set_error(ctx, "Unsupported PPM/PAM bit depth"); return -1; }
	return m;
}

static int write_rgb(struct iw_context *ctx, FILE *f, const struct iw_image *img, int pam)
{
	static const int rgb[3] = {IW_CHANNELTYPE_RED, IW_CHANNELTYPE_GREEN, IW_CHANNELTYPE_BLUE};
	static const int gray[1] = {IW_CHANNELTYPE_GRAY};
	int bps, m, i, j;
	size_t rowsize;
	unsigned char *row;
	if(img->bit_depth != 8 && img->bit_depth != 16) return 0;
	bps = img->bit_depth / 8;
	m = img->imgtype == IW_IMGTYPE_GRAY ? written_maxval(ctx, img, gray, 1, "") :
	    written_maxval(ctx, img, rgb, 3, "PNM/PPM/PAM format requires equal bit depths");
	if(m < 0) return 0;
	rowsize = (size_t)3 * bps * img->width;
	row = (unsigned char *)malloc(rowsize ? rowsize : 1);
	if(!row) { iw_set_error(ctx, "Out of memory"); return 0; }
	if(pam) header_pam(f, img, 3, m, "RGB");
	else fprintf(f, "P6\n%d %d\n%d\n", img->width, img->height, m);
	for(j = 0; j < img->height; j++) {
		const unsigned char *src = img->pixels + (size_t)j * img->bpr;
		if(img->imgtype == IW_IMGTYPE_RGB) memcpy(row, src, rowsize);
		else
			for(i = 0; i < img->width; i++) {
				int c;
				for(c = 0; c < 3; c++) memcpy(row + ((size_t)i * 3 + c) * bps, src + (size_t)i * bps, bps);
			}
		if(!put(f, row, rowsize)) { free(row); iw_set_error(ctx, "Failed to write file"); return 0; }
	}
	free(row);
	return 1;
}

static int write_gray(struct iw_context *ctx, FILE *f, const struct iw_image *img, int pam)
{
	static const int gray[1] = {IW_CHANNELTYPE_GRAY};
	int m, bilevel = 0, j;
	size_t rowsize;
	if(bw_palette(ctx, img)) bilevel = 1;
	else if(img->imgtype != IW_IMGTYPE_GRAY) { iw_set_error(ctx, "Cannot write non-grayscale image to PGM file"); return 0; }
	if(bilevel) m = 1;
	else if(img->bit_depth == 8) m = 255;
	else if(img->bit_depth == 16) m = 65535;
	else return 0;
	if(img->reduced_maxcolors) m = (int)img->maxcolorcode[gray[0]];
	if(m < 1 || m > 65535) { iw_set_error(ctx, "Unsupported PGM bit depth"); return 0; }
	rowsize = (size_t)(bilevel || img->bit_depth == 8 ? 1 : 2) * img->width;
	if(pam) header_pam(f, img, 1, m == 1 ? 1 : m, m == 1 ? "BLACKANDWHITE" : "GRAYSCALE");
	else fprintf(f, "P5\n%d %d\n%d\n", img->width, img->height, m);
	for(j = 0; j < img->height; j++)
		if(!put(f, img->pixels + (size_t)j * img->bpr, rowsize)) { iw_set_error(ctx, "Failed to write file"); return 0; }
	return 1;
}

static int write_alpha(struct iw_context *ctx, FILE *f, const struct iw_image *img, int nch)
{
	static const int rgba[4] = {IW_CHANNELTYPE_RED, IW_CHANNELTYPE_GREEN, IW_CHANNELTYPE_BLUE, IW_CHANNELTYPE_ALPHA};
	static const int ga[2] = {IW_CHANNELTYPE_GRAY, IW_CHANNELTYPE_ALPHA};
	int m, j;
	size_t rowsize;
	if(img->bit_depth != 8 && img->bit_depth != 16) return 0;
	m = nch == 4 ? written_maxval(ctx, img, rgba, 4, "PAM format requires equal bit depths") :
	    written_maxval(ctx, img, ga, 2, "PAM format requires equal bit depths");
	if(m < 0) return 0;
	rowsize = (size_t)nch * (img->bit_depth / 8) * img->width;
	if(nch == 4) header_pam(f, img, 4, m, "RGB_ALPHA");
	else header_pam(f, img, 2, m, m == 1 ? "BLACKANDWHITE_ALPHA" : "GRAYSCALE_ALPHA");
	for(j = 0; j < img->height; j++)
		if(!put(f, img->pixels + (size_t)j * img->bpr, rowsize)) { iw_set_error(ctx, "Failed to write file"); return 0; }
	return 1;
}

/* PBM: a two-entry gray palette image, one bit per pixel, entry 0 (black) -> 1. */
static int write_pbm(struct iw_context *ctx, FILE *f, const struct iw_image *img)
{
	size_t rowsize = ((size_t)img->width + 7) / 8;
	unsigned char *row;
	int i, j;
	if(!bw_palette(ctx, img)) { iw_set_error(ctx, "Cannot write this image type to a PBM file"); return 0; }
	row = (unsigned char *)malloc(rowsize ? rowsize : 1);
	if(!row) { iw_set_error(ctx, "Out of memory"); return 0; }
	fprintf(f, "P4\n%d %d\n", img->width, img->height);
	for(j = 0; j < img->height; j++) {
		memset(row, 0, rowsize);
		for(i = 0; i < img->width; i++)
			if(img->pixels[(size_t)j * img->bpr + i] == 0) row[i / 8] |= (unsigned char)(1 << (7 - i % 8));
		if(!put(f, row, rowsize)) { free(row); iw_set_error(ctx, "Failed to write file"); return 0; }
	}
	free(row);
	return 1;
}

int pnm_write(struct iw_context *ctx, FILE *f, int fmt)
{
	struct iw_image img;
	memset(&img, 0, sizeof(img));
	iw_get_output_image(ctx, &img);
	if(fmt == IW_FORMAT_PNM) {
		if(img.imgtype == IW_IMGTYPE_PALETTE) return write_pbm(ctx, f, &img);
		if(img.imgtype == IW_IMGTYPE_GRAY) fmt = IW_FORMAT_PGM;
		else if(img.imgtype == IW_IMGTYPE_RGB) fmt = IW_FORMAT_PPM;
		else { iw_set_error(ctx, "Internal: Bad image type for PNM"); return 0; }
		return fmt == IW_FORMAT_PGM ? write_gray(ctx, f, &img, 0) : write_rgb(ctx, f, &img, 0);
	}
	switch(fmt) {
	case IW_FORMAT_PPM: return write_rgb(ctx, f, &img, 0);
	case IW_FORMAT_PGM: return write_gray(ctx, f, &img, 0);
	case IW_FORMAT_PBM: return write_pbm(ctx, f, &img);
	case IW_FORMAT_PAM:
		if(img.imgtype == IW_IMGTYPE_RGBA) return write_alpha(ctx, f, &img, 4);
		if(img.imgtype == IW_IMGTYPE_GRAYA) return write_alpha(ctx, f, &img, 2);
		if(img.imgtype == IW_IMGTYPE_RGB) return write_rgb(ctx, f, &img, 1);
		if(img.imgtype == IW_IMGTYPE_GRAY || img.imgtype == IW_IMGTYPE_PALETTE) return write_gray(ctx, f, &img, 1);
		iw_set_error(ctx, "Unsupported image type for PAM");
		return 0;
	default:
		iw_set_error(ctx, "Internal: Bad image type for PNM");
		return 0;
	}
}
