/*
 * iw_oracle_opt.c -- CPU oracle: the output post-pass that runs after the
 * pixel pipeline (restates src/imagew-opt.c of ImageWorsener 1.3.5).
 *
 * TEST INFRASTRUCTURE ONLY (see iw_oracle.h).  The post-pass blackens fully
 * transparent pixels and then, where the output profile allows, repacks the
 * image: 16->8 bits, alpha stripping, RGB->gray, palette / low-bit gray, and
 * colour-keyed binary transparency.
 */
#include <stdlib.h>
#include <string.h>

#include "iw_oracle.h"

/* ---- scans: which properties does the image actually use (src/imagew-opt.c:18-386) ---- */

static void scan_pixels(struct orc_opt *o, int *scanned)
{
	int nch = iw_imgtype_num_channels(o->imgtype);
	int wide = o->bit_depth == 16;
	int has_a = IW_IMGTYPE_HAS_ALPHA(o->imgtype);
	int is_rgb = !IW_IMGTYPE_IS_GRAY(o->imgtype);
	int x, y, k;

	/* The reference has no scan for 8-bit gray (nothing to learn there). */
	if(o->imgtype == IW_IMGTYPE_GRAY && !wide) { *scanned = 0; return; }
	if(o->bit_depth != 8 && o->bit_depth != 16) { *scanned = 0; return; }
	*scanned = 1;

	for(y = 0; y < o->height; y++) {
		const iw_byte *row = o->pix + (size_t)y * o->bpr;
		for(x = 0; x < o->width; x++) {
			unsigned int v[4];
			const iw_byte *p = row + (size_t)x * nch * (wide ? 2 : 1);
			for(k = 0; k < nch; k++) {
				if(wide) {
					v[k] = ((unsigned int)p[2 * k] << 8) | p[2 * k + 1];
					if(p[2 * k] != p[2 * k + 1]) o->has_16bit = 1;
				}
				else v[k] = p[k];
			}
			if(has_a) {
				unsigned int a = v[nch - 1], full = wide ? 65535u : 255u;
				if(a < full) {
					o->has_trns = 1;
					if(a > 0) o->has_partial_trns = 1;
				}
			}
			if(is_rgb && (v[0] != v[1] || v[0] != v[2])) o->has_color = 1;

			/* stop once nothing more can be learned */
			if((!has_a || o->has_partial_trns) && (!is_rgb || o->has_color) && (!wide || o->has_16bit))
				return;
		}
	}
}

/* ---- repacking helpers ---- */

static void attach(struct iw_context *ctx, struct orc_opt *o, iw_byte *pix, size_t bpr)
{
	iw_free(ctx, o->tmp);
	o->tmp = pix;
	o->pix = pix;
	o->bpr = bpr;
}

static void to_8bit(struct iw_context *ctx, struct orc_opt *o, int spp)
{
	size_t bpr;
	iw_byte *np;
	int x, y, k;
	if(!ctx->opt_16to8) return;
	bpr = iw_calc_bytesperrow(o->width, 8 * spp);
	np = iw_malloc_large(ctx, bpr, o->height);
	if(!np) return;
	for(y = 0; y < o->height; y++)
		for(x = 0; x < spp * o->width; x++)
			np[(size_t)y * bpr + x] = o->pix[(size_t)y * o->bpr + 2 * (size_t)x];
	attach(ctx, o, np, bpr);
	o->bit_depth = 8;
	if(o->has_label) for(k = 0; k < 4; k++) o->label[k] >>= 8;
}

/* New image made of up to three channels (c0,c1,c2) of the current one. */
static void pick_channels(struct iw_context *ctx, struct orc_opt *o, int newtype, int c0, int c1, int c2)
{
	int on = iw_imgtype_num_channels(o->imgtype), nn = iw_imgtype_num_channels(newtype);
	int bps = o->bit_depth == 16 ? 2 : 1;
	int sel[3] = {c0, c1, c2};
	size_t bpr = iw_calc_bytesperrow(o->width, 8 * bps * nn);
	iw_byte *np = iw_malloc_large(ctx, bpr, o->height);
	int x, y, k, b;
	if(!np) return;
	for(y = 0; y < o->height; y++)
		for(x = 0; x < o->width; x++)
			for(k = 0; k < nn; k++)
				for(b = 0; b < bps; b++)
					np[(size_t)y * bpr + ((size_t)x * nn + k) * bps + b] =
						o->pix[(size_t)y * o->bpr + ((size_t)x * on + sel[k]) * bps + b];
	attach(ctx, o, np, bpr);
	o->imgtype = newtype;
}

/* Unused value nearest to 192 among count flags (src/imagew-opt.c:391-415). */
static int find_unused(const iw_byte *used, int count, iw_byte *out)
{
	int i, best = -1, bestd = 0;
	for(i = 0; i < count; i++) {
		int d = abs(i - 192);
		if(!used[i] && (best < 0 || d < bestd)) { best = i; bestd = d; }
	}
	*out = (iw_byte)(best < 0 ? 0 : best);
	return best >= 0;
}

/* Alpha channel -> colour key, for images whose alpha is only 0 or max
 * (src/imagew-opt.c:417-683).  Key colours come from a family of 256 with all
 * components 192 except the lowest byte of red (or of gray). */
static void try_binary_trns(struct iw_context *ctx, struct orc_opt *o)
{
	int gray = IW_IMGTYPE_IS_GRAY(o->imgtype), wide = o->bit_depth == 16;
	int nch = iw_imgtype_num_channels(o->imgtype), bps = wide ? 2 : 1;
	iw_byte used[256], key = 0, *mask;
	int x, y;

	if(!(ctx->profile & IW_PROFILE_BINARYTRNS) || !ctx->opt_bintrns) return;
	memset(used, 0, sizeof(used));
	mask = iw_malloc_large(ctx, o->width, o->height);
	if(!mask) return;

	for(y = 0; y < o->height; y++) {
		for(x = 0; x < o->width; x++) {
			const iw_byte *p = o->pix + (size_t)y * o->bpr + (size_t)x * nch * bps;
			const iw_byte *a = p + (nch - 1) * bps;
			int transparent = wide ? (a[0] == 0 && a[1] == 0) : (a[0] == 0);
			mask[(size_t)y * o->width + x] = transparent ? 0 : 1;
			if(transparent) continue;
			if(gray) {
				if(!wide) used[p[0]] = 1;
				else if(p[0] == 192) used[p[1]] = 1;
			}
			else if(!wide) {
				if(p[1] == 192 && p[2] == 192) used[p[0]] = 1;
			}
			else if(p[0] == 192 && p[2] == 192 && p[3] == 192 && p[4] == 192 && p[5] == 192) used[p[1]] = 1;
		}
	}
	if(!find_unused(used, 256, &key)) goto done;

	if(gray) pick_channels(ctx, o, IW_IMGTYPE_GRAY, 0, 0, 0);
	else pick_channels(ctx, o, IW_IMGTYPE_RGB, 0, 1, 2);
	if(!o->tmp) goto done;

	for(y = 0; y < o->height; y++) {
		for(x = 0; x < o->width; x++) {
			iw_byte *q;
			if(mask[(size_t)y * o->width + x]) continue;
			q = o->tmp + (size_t)y * o->bpr + (size_t)x * (gray ? 1 : 3) * bps;
			if(gray && !wide) q[0] = key;
			else if(gray) { q[0] = 192; q[1] = key; }
			else if(!wide) { q[0] = key; q[1] = 192; q[2] = 192; }
			else { q[0] = 192; q[1] = key; q[2] = q[3] = q[4] = q[5] = 192; }
		}
	}
	o->has_ckey = 1;
	if(gray) o->ckey[0] = o->ckey[1] = o->ckey[2] = wide ? 192u * 256u + key : key;
	else {
		o->ckey[0] = wide ? 192u * 256u + key : key;
		o->ckey[1] = o->ckey[2] = wide ? 192u * 256u + 192u : 192u;
	}
done:
	iw_free(ctx, mask);
}

/* ---- palette and low-bit-depth gray (src/imagew-opt.c:685-1108) ---- */

static struct iw_rgba8color pixel_color(const struct orc_opt *o, int x, int y)
{
	int spp = iw_imgtype_num_channels(o->imgtype);
	const iw_byte *p = o->pix + (size_t)y * o->bpr + (size_t)x * spp;
	struct iw_rgba8color c;
	switch(o->imgtype) {
	case IW_IMGTYPE_RGB: c.r = p[0]; c.g = p[1]; c.b = p[2]; c.a = 255; break;
	case IW_IMGTYPE_RGBA: c.r = p[0]; c.g = p[1]; c.b = p[2]; c.a = p[3]; break;
	case IW_IMGTYPE_GRAYA: c.r = c.g = c.b = p[0]; c.a = p[1]; break;
	default: c.r = c.g = c.b = p[0]; c.a = 255; break;
	}
	if(c.a == 0) c.r = c.g = c.b = 0; /* all invisible colours are one entry */
	return c;
}

static int pal_find(const struct iw_palette *pal, struct iw_rgba8color c)
{
	int i;
	for(i = 0; i < pal->num_entries; i++) {
		const struct iw_rgba8color *e = &pal->entry[i];
		if(e->r == c.r && e->g == c.g && e->b == c.b && e->a == c.a) return i;
	}
	return -1;
}

static int collect_palette(struct orc_opt *o)
{
	int x, y, i;
	for(y = 0; y < o->height; y++) {
		for(x = 0; x < o->width; x++) {
			struct iw_rgba8color c = pixel_color(o, x, y);
			if(pal_find(o->pal, c) >= 0) continue;
			if(o->pal->num_entries >= 256) return 0;
			o->pal->entry[o->pal->num_entries++] = c;
		}
	}
	if(o->pal->num_entries < 1) return 0;
	if(o->has_label) {
		/* the background label needs an entry: a transparent one, or its colour */
		struct iw_rgba8color c;
		int found = 0;
		c.r = (iw_byte)o->label[0]; c.g = (iw_byte)o->label[1]; c.b = (iw_byte)o->label[2]; c.a = 255;
		for(i = 0; i < o->pal->num_entries; i++) {
			const struct iw_rgba8color *e = &o->pal->entry[i];
			if(e->a == 0 || (e->r == c.r && e->g == c.g && e->b == c.b)) { found = 1; break; }
		}
		if(!found) {
			if(o->pal->num_entries >= 256) return 0;
			o->pal->entry[o->pal->num_entries++] = c;
		}
	}
	return 1;
}

static int pal_order(const void *pa, const void *pb)
{
	const struct iw_rgba8color *a = pa, *b = pb;
	int sa, sb;
	if(a->a == 255 && b->a < 255) return 1;
	if(a->a < 255 && b->a == 255) return -1;
	sa = a->r + a->g + a->b;
	sb = b->r + b->g + b->b;
	if(sa != sb) return sa > sb ? 1 : -1;
	if(a->g != b->g) return a->g > b->g ? 1 : -1;
	if(a->r != b->r) return a->r > b->r ? 1 : -1;
	if(a->b != b->b) return a->b > b->b ? 1 : -1;
	if(a->a != b->a) return a->a > b->a ? 1 : -1;
	return 0;
}

static int palette_ok(struct iw_context *ctx, struct orc_opt *o, int bpp)
{
	static const unsigned int prof[9] = {0, IW_PROFILE_PAL1, IW_PROFILE_PAL2, 0, IW_PROFILE_PAL4, 0, 0, 0, IW_PROFILE_PAL8};
	if(!ctx->opt_pal) return 0;
	if(o->has_trns && !(ctx->profile & IW_PROFILE_PALETTETRNS)) return 0;
	if(!(ctx->profile & prof[bpp])) return 0;
	return o->pal->num_entries <= (1 << bpp);
}

/* Can the image be written as 'bpp'-bit gray (with a colour key if needed)? */
static int gray_ok(struct iw_context *ctx, struct orc_opt *o, int bpp, int *bin, unsigned int *shade)
{
	int factor = bpp == 1 ? 255 : bpp == 2 ? 85 : bpp == 4 ? 17 : 1;
	int maxe = 1 << bpp, i;
	iw_byte used[256], key = 0;

	*bin = 0;
	*shade = 0;
	if(o->has_color || o->has_partial_trns) return 0;
	if(o->has_trns && (!ctx->opt_bintrns || !(ctx->profile & IW_PROFILE_BINARYTRNS))) return 0;
	if(o->pal->num_entries > maxe) return 0;
	if(o->has_label && bpp < 8 && o->label[0] % factor != 0) return 0;
	memset(used, 0, sizeof(used));
	for(i = 0; i < o->pal->num_entries; i++) {
		if(o->pal->entry[i].a > 0) {
			if(o->pal->entry[i].r % factor) return 0;
			used[o->pal->entry[i].r / factor] = 1;
		}
	}
	if(o->has_trns) {
		if(!find_unused(used, maxe, &key)) return 0;
		*bin = 1;
		*shade = key;
	}
	return 1;
}

static void make_gray_palette(struct orc_opt *o, int bpp)
{
	int factor = bpp == 1 ? 255 : bpp == 2 ? 85 : bpp == 4 ? 17 : 1, i;
	o->pal->num_entries = 1 << bpp;
	for(i = 0; i < o->pal->num_entries; i++) {
		o->pal->entry[i].r = o->pal->entry[i].g = o->pal->entry[i].b = (iw_byte)(factor * i);
		o->pal->entry[i].a = 255;
	}
	o->pal_is_gray = 1;
}

static void to_palette_image(struct iw_context *ctx, struct orc_opt *o)
{
	size_t bpr = o->width;
	iw_byte *np = iw_malloc_large(ctx, bpr, o->height);
	int x, y;
	if(!np) return;
	for(y = 0; y < o->height; y++) {
		for(x = 0; x < o->width; x++) {
			struct iw_rgba8color c = pixel_color(o, x, y);
			int e;
			if(o->has_ckey && c.a == 0) e = (int)o->ckey[0];
			else {
				e = pal_find(o->pal, c);
				if(e < 0) e = 0;
			}
			np[(size_t)y * bpr + x] = (iw_byte)e;
		}
	}
	attach(ctx, o, np, bpr);
	o->bit_depth = 8;
	o->imgtype = IW_IMGTYPE_PALETTE;
}

static void try_palette(struct iw_context *ctx, struct orc_opt *o)
{
	static const int bpps[4] = {1, 2, 4, 8};
	static const unsigned int grayprof[4] = {IW_PROFILE_GRAY1, IW_PROFILE_GRAY2, IW_PROFILE_GRAY4, IW_PROFILE_GRAYSCALE};
	int i, bin, chosen = 0;
	unsigned int shade;

	if(!(ctx->profile & (IW_PROFILE_PAL1 | IW_PROFILE_PAL2 | IW_PROFILE_PAL4 | IW_PROFILE_PAL8 |
		IW_PROFILE_GRAY1 | IW_PROFILE_GRAY2 | IW_PROFILE_GRAY4))) return;
	if(o->bit_depth != 8) return;
	o->pal = iw_malloc(ctx, sizeof(struct iw_palette));
	if(!o->pal) return;
	o->pal->num_entries = 0;
	if(!collect_palette(o)) goto done;

	/* Preference: gray1, pal1, gray2, pal2, gray4, pal4, (gray8: left as is), pal8. */
	for(i = 0; i < 4 && !chosen; i++) {
		if(ctx->opt_gray && (ctx->profile & grayprof[i]) && gray_ok(ctx, o, bpps[i], &bin, &shade)) {
			if(bpps[i] == 8) goto done; /* plain 8-bit gray is better; handled elsewhere */
			make_gray_palette(o, bpps[i]);
			if(bin) {
				o->has_ckey = 1;
				o->ckey[0] = o->ckey[1] = o->ckey[2] = shade;
			}
			chosen = 1;
		}
		else if(palette_ok(ctx, o, bpps[i])) chosen = 1;
	}
	if(!chosen) goto done;
	if(!o->pal_is_gray) qsort(o->pal->entry, o->pal->num_entries, sizeof(struct iw_rgba8color), pal_order);
	to_palette_image(ctx, o);
done:
	if(o->imgtype != IW_IMGTYPE_PALETTE) {
		iw_free(ctx, o->pal);
		o->pal = NULL;
	}
}

/* ---- driver (src/imagew-opt.c:1112-1314) ---- */

static void blacken_transparent(struct iw_image *img)
{
	int nch, x, y, k, wide;
	if(!IW_IMGTYPE_HAS_ALPHA(img->imgtype)) return;
	nch = iw_imgtype_num_channels(img->imgtype);
	wide = img->bit_depth > 8;
	for(y = 0; y < img->height; y++) {
		for(x = 0; x < img->width; x++) {
			iw_byte *p = img->pixels + (size_t)y * img->bpr + (size_t)x * nch * (wide ? 2 : 1);
			if(wide) {
				if(p[(nch - 1) * 2] == 0 && p[(nch - 1) * 2 + 1] == 0)
					for(k = 0; k < 2 * (nch - 1); k++) p[k] = 0;
			}
			else if(p[nch - 1] == 0)
				for(k = 0; k < nch - 1; k++) p[k] = 0;
		}
	}
}

void orc_optimize(struct iw_context *ctx)
{
	struct orc_opt *o = &ctx->opt;
	int k, scanned;

	o->width = ctx->img2.width;
	o->height = ctx->img2.height;
	o->imgtype = ctx->img2.imgtype;
	o->bit_depth = ctx->img2.bit_depth;
	o->bpr = ctx->img2.bpr;
	o->pix = ctx->img2.pixels;
	if(ctx->img2.has_bkgdlabel) {
		o->has_label = 1;
		for(k = 0; k < 4; k++)
			o->label[k] = iw_color_get_int_sample(&ctx->img2.bkgdlabel, k, ctx->img2.bit_depth == 8 ? 255 : 65535);
	}
	if(ctx->img2.sampletype != IW_SAMPLETYPE_UINT) return;
	if(ctx->reduced_out) return;

	blacken_transparent(&ctx->img2);

	if(o->has_label) {
		if(o->label[0] != o->label[1] || o->label[0] != o->label[2]) o->has_color = 1;
		if(o->bit_depth == 16 && (o->label[0] % 257 || o->label[1] % 257 || o->label[2] % 257))
			o->has_16bit = 1;
	}

	scan_pixels(o, &scanned);
	if(scanned) {
		if(o->bit_depth == 16 && !o->has_16bit) to_8bit(ctx, o, iw_imgtype_num_channels(o->imgtype));
		if(!o->has_trns && ctx->opt_strip) {
			if(o->imgtype == IW_IMGTYPE_RGBA) pick_channels(ctx, o, IW_IMGTYPE_RGB, 0, 1, 2);
			else if(o->imgtype == IW_IMGTYPE_GRAYA) pick_channels(ctx, o, IW_IMGTYPE_GRAY, 0, 0, 0);
		}
		if(!o->has_color && (ctx->profile & IW_PROFILE_GRAYSCALE) && ctx->opt_gray) {
			if(o->imgtype == IW_IMGTYPE_RGB) pick_channels(ctx, o, IW_IMGTYPE_GRAY, 0, 0, 0);
			else if(o->imgtype == IW_IMGTYPE_RGBA) pick_channels(ctx, o, IW_IMGTYPE_GRAYA, 0, 3, 0);
		}
	}

	try_palette(ctx, o);

	if((o->imgtype == IW_IMGTYPE_RGBA || o->imgtype == IW_IMGTYPE_GRAYA) && !o->has_partial_trns)
		try_binary_trns(ctx, o);
}
