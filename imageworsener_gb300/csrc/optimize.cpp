// optimize.cpp -- output post-pass (src/imagew-opt.c:1166-1314).
//
// After the pixel passes the reference optionally repacks the output image:
// 16->8 bits when no sample needs 16, alpha removal when nothing is
// transparent, RGB->gray when nothing has colour, palette / 1-2-4-bit gray
// encodings, and colour-keyed binary transparency.  The repacked image is what
// iw_get_output_image() returns, so a drop-in has to make the same choices.
// Fully transparent pixels are blackened on the GPU (fused into the
// quantisation tail), so this pass starts from that image.
#include "iwg_internal.h"

#include <cstdlib>
#include <cstring>

namespace iwg {

namespace {

int nch_of(int t) { return iw_imgtype_num_channels(t); }

// Which properties does the image use (src/imagew-opt.c:18-386)?  Stops as soon
// as every tracked property is known to be present.
bool scan_pixels(OptState &o)
{
	const bool wide = o.bit_depth == 16;
	if(o.imgtype == IW_IMGTYPE_GRAY && !wide) return false;
	if(o.bit_depth != 8 && o.bit_depth != 16) return false;
	const int n = nch_of(o.imgtype);
	const bool has_a = IW_IMGTYPE_HAS_ALPHA(o.imgtype), rgb = !IW_IMGTYPE_IS_GRAY(o.imgtype);
	const unsigned int full = wide ? 65535u : 255u;
	for(int y = 0; y < o.height; y++) {
		const iw_byte *row = o.pix + (size_t)y * o.bpr;
		for(int x = 0; x < o.width; x++) {
			unsigned int v[4];
			const iw_byte *p = row + (size_t)x * n * (wide ? 2 : 1);
			for(int k = 0; k < n; k++) {
				if(wide) {
					v[k] = ((unsigned int)p[2 * k] << 8) | p[2 * k + 1];
					if(p[2 * k] != p[2 * k + 1]) o.has_16bit = 1;
				}
				else v[k] = p[k];
			}
			if(has_a && v[n - 1] < full) {
				o.has_trns = 1;
				if(v[n - 1] > 0) o.has_partial_trns = 1;
			}
			if(rgb && (v[0] != v[1] || v[0] != v[2])) o.has_color = 1;
			if((!has_a || o.has_partial_trns) && (!rgb || o.has_color) && (!wide || o.has_16bit)) return true;
		}
	}
	return true;
}

void attach(iw_context *ctx, OptState &o, iw_byte *pix, size_t bpr)
{
	iw_free(ctx, o.tmp);
	o.tmp = pix;
	o.pix = pix;
	o.bpr = bpr;
}

void to_8bit(iw_context *ctx, OptState &o, int spp)
{
	if(!ctx->opt_16to8) return;
	size_t bpr = iw_calc_bytesperrow(o.width, 8 * spp);
	iw_byte *np = (iw_byte *)iw_malloc_large(ctx, bpr, o.height);
	if(!np) return;
	for(int y = 0; y < o.height; y++) {
		const iw_byte *s = o.pix + (size_t)y * o.bpr;
		iw_byte *d = np + (size_t)y * bpr;
		for(int i = 0; i < spp * o.width; i++) d[i] = s[2 * (size_t)i];   // high byte
	}
	attach(ctx, o, np, bpr);
	o.bit_depth = 8;
	if(o.has_label) for(int k = 0; k < 4; k++) o.label[k] >>= 8;
}

// New image made of channels (c0,c1,c2) of the current one.
void pick(iw_context *ctx, OptState &o, int newtype, int c0, int c1, int c2)
{
	const int on = nch_of(o.imgtype), nn = nch_of(newtype), bps = o.bit_depth == 16 ? 2 : 1;
	const int sel[3] = {c0, c1, c2};
	size_t bpr = iw_calc_bytesperrow(o.width, 8 * bps * nn);
	iw_byte *np = (iw_byte *)iw_malloc_large(ctx, bpr, o.height);
	if(!np) return;
	for(int y = 0; y < o.height; y++) {
		const iw_byte *s = o.pix + (size_t)y * o.bpr;
		iw_byte *d = np + (size_t)y * bpr;
		for(int x = 0; x < o.width; x++)
			for(int k = 0; k < nn; k++)
				for(int b = 0; b < bps; b++)
					d[((size_t)x * nn + k) * bps + b] = s[((size_t)x * on + sel[k]) * bps + b];
	}
	attach(ctx, o, np, bpr);
	o.imgtype = newtype;
}

// Unused flag nearest to 192 (src/imagew-opt.c:391-415).
bool find_unused(const iw_byte *used, int count, iw_byte *out)
{
	int best = -1, bestd = 0;
	for(int i = 0; i < count; i++) {
		int d = abs(i - 192);
		if(!used[i] && (best < 0 || d < bestd)) { best = i; bestd = d; }
	}
	*out = (iw_byte)(best < 0 ? 0 : best);
	return best >= 0;
}

// Alpha channel -> colour key (src/imagew-opt.c:417-683).  Candidate keys have
// every component byte 192 except the lowest byte of red (or gray).
void try_binary_trns(iw_context *ctx, OptState &o)
{
	if(!(ctx->profile & IW_PROFILE_BINARYTRNS) || !ctx->opt_bintrns) return;
	const bool gray = IW_IMGTYPE_IS_GRAY(o.imgtype), wide = o.bit_depth == 16;
	const int n = nch_of(o.imgtype), bps = wide ? 2 : 1;
	iw_byte used[256];
	memset(used, 0, sizeof(used));
	iw_byte *mask = (iw_byte *)iw_malloc_large(ctx, o.width, o.height);
	if(!mask) return;
	for(int y = 0; y < o.height; y++) {
		for(int x = 0; x < o.width; x++) {
			const iw_byte *p = o.pix + (size_t)y * o.bpr + (size_t)x * n * bps;
			const iw_byte *a = p + (n - 1) * bps;
			bool transparent = wide ? (a[0] == 0 && a[1] == 0) : (a[0] == 0);
			mask[(size_t)y * o.width + x] = transparent ? 0 : 1;
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
	iw_byte key = 0;
	if(find_unused(used, 256, &key)) {
		pick(ctx, o, gray ? IW_IMGTYPE_GRAY : IW_IMGTYPE_RGB, 0, gray ? 0 : 1, gray ? 0 : 2);
		if(o.tmp) {
			for(int y = 0; y < o.height; y++) {
				for(int x = 0; x < o.width; x++) {
					if(mask[(size_t)y * o.width + x]) continue;
					iw_byte *q = o.tmp + (size_t)y * o.bpr + (size_t)x * (gray ? 1 : 3) * bps;
					if(gray && !wide) q[0] = key;
					else if(gray) { q[0] = 192; q[1] = key; }
					else if(!wide) { q[0] = key; q[1] = 192; q[2] = 192; }
					else { q[0] = 192; q[1] = key; q[2] = q[3] = q[4] = q[5] = 192; }
				}
			}
			o.has_ckey = 1;
			if(gray) o.ckey[0] = o.ckey[1] = o.ckey[2] = wide ? 192u * 256u + key : key;
			else {
				o.ckey[0] = wide ? 192u * 256u + key : key;
				o.ckey[1] = o.ckey[2] = wide ? 192u * 256u + 192u : 192u;
			}
		}
	}
	iw_free(ctx, mask);
}

struct iw_rgba8color pixel_color(const OptState &o, int x, int y)
{
	const int spp = nch_of(o.imgtype);
	const iw_byte *p = o.pix + (size_t)y * o.bpr + (size_t)x * spp;
	struct iw_rgba8color c;
	switch(o.imgtype) {
	case IW_IMGTYPE_RGB: c.r = p[0]; c.g = p[1]; c.b = p[2]; c.a = 255; break;
	case IW_IMGTYPE_RGBA: c.r = p[0]; c.g = p[1]; c.b = p[2]; c.a = p[3]; break;
	case IW_IMGTYPE_GRAYA: c.r = c.g = c.b = p[0]; c.a = p[1]; break;
	default: c.r = c.g = c.b = p[0]; c.a = 255; break;
	}
	if(c.a == 0) c.r = c.g = c.b = 0;   // invisible colours share one entry
	return c;
}

int pal_find(const struct iw_palette *pal, struct iw_rgba8color c)
{
	for(int i = 0; i < pal->num_entries; i++) {
		const struct iw_rgba8color &e = pal->entry[i];
		if(e.r == c.r && e.g == c.g && e.b == c.b && e.a == c.a) return i;
	}
	return -1;
}

bool collect_palette(OptState &o)
{
	// Fast membership test for the 256-entry palette.
	for(int y = 0; y < o.height; y++) {
		for(int x = 0; x < o.width; x++) {
			struct iw_rgba8color c = pixel_color(o, x, y);
			if(pal_find(o.pal, c) >= 0) continue;
			if(o.pal->num_entries >= 256) return false;
			o.pal->entry[o.pal->num_entries++] = c;
		}
	}
	if(o.pal->num_entries < 1) return false;
	if(o.has_label) {
		struct iw_rgba8color c;
		c.r = (iw_byte)o.label[0]; c.g = (iw_byte)o.label[1]; c.b = (iw_byte)o.label[2]; c.a = 255;
		bool found = false;
		for(int i = 0; i < o.pal->num_entries; i++) {
			const struct iw_rgba8color &e = o.pal->entry[i];
			if(e.a == 0 || (e.r == c.r && e.g == c.g && e.b == c.b)) { found = true; break; }
		}
		if(!found) {
			if(o.pal->num_entries >= 256) return false;
			o.pal->entry[o.pal->num_entries++] = c;
		}
	}
	return true;
}

int pal_order(const void *pa, const void *pb)
{
	const struct iw_rgba8color *a = (const struct iw_rgba8color *)pa, *b = (const struct iw_rgba8color *)pb;
	if(a->a == 255 && b->a < 255) return 1;
	if(a->a < 255 && b->a == 255) return -1;
	int sa = a->r + a->g + a->b, sb = b->r + b->g + b->b;
	if(sa != sb) return sa > sb ? 1 : -1;
	if(a->g != b->g) return a->g > b->g ? 1 : -1;
	if(a->r != b->r) return a->r > b->r ? 1 : -1;
	if(a->b != b->b) return a->b > b->b ? 1 : -1;
	if(a->a != b->a) return a->a > b->a ? 1 : -1;
	return 0;
}

bool palette_ok(iw_context *ctx, OptState &o, int bpp)
{
	static const unsigned int prof[9] = {0, IW_PROFILE_PAL1, IW_PROFILE_PAL2, 0, IW_PROFILE_PAL4, 0, 0, 0, IW_PROFILE_PAL8};
	if(!ctx->opt_pal) return false;
	if(o.has_trns && !(ctx->profile & IW_PROFILE_PALETTETRNS)) return false;
	if(!(ctx->profile & prof[bpp])) return false;
	return o.pal->num_entries <= (1 << bpp);
}

bool gray_ok(iw_context *ctx, OptState &o, int bpp, bool *bin, unsigned int *shade)
{
	const int factor = bpp == 1 ? 255 : bpp == 2 ? 85 : bpp == 4 ? 17 : 1, maxe = 1 << bpp;
	*bin = false;
	*shade = 0;
	if(o.has_color || o.has_partial_trns) return false;
	if(o.has_trns && (!ctx->opt_bintrns || !(ctx->profile & IW_PROFILE_BINARYTRNS))) return false;
	if(o.pal->num_entries > maxe) return false;
	if(o.has_label && bpp < 8 && o.label[0] % factor != 0) return false;
	iw_byte used[256];
	memset(used, 0, sizeof(used));
	for(int i = 0; i < o.pal->num_entries; i++) {
		if(o.pal->entry[i].a > 0) {
			if(o.pal->entry[i].r % factor) return false;
			used[o.pal->entry[i].r / factor] = 1;
		}
	}
	if(o.has_trns) {
		iw_byte key;
		if(!find_unused(used, maxe, &key)) return false;
		*bin = true;
		*shade = key;
	}
	return true;
}

void make_gray_palette(OptState &o, int bpp)
{
	const int factor = bpp == 1 ? 255 : bpp == 2 ? 85 : bpp == 4 ? 17 : 1;
	o.pal->num_entries = 1 << bpp;
	for(int i = 0; i < o.pal->num_entries; i++) {
		o.pal->entry[i].r = o.pal->entry[i].g = o.pal->entry[i].b = (iw_byte)(factor * i);
		o.pal->entry[i].a = 255;
	}
	o.pal_is_gray = 1;
}

void to_palette_image(iw_context *ctx, OptState &o)
{
	size_t bpr = o.width;
	iw_byte *np = (iw_byte *)iw_malloc_large(ctx, bpr, o.height);
	if(!np) return;
	for(int y = 0; y < o.height; y++) {
		for(int x = 0; x < o.width; x++) {
			struct iw_rgba8color c = pixel_color(o, x, y);
			int e;
			if(o.has_ckey && c.a == 0) e = (int)o.ckey[0];
			else {
				e = pal_find(o.pal, c);
				if(e < 0) e = 0;
			}
			np[(size_t)y * bpr + x] = (iw_byte)e;
		}
	}
	attach(ctx, o, np, bpr);
	o.bit_depth = 8;
	o.imgtype = IW_IMGTYPE_PALETTE;
}

void try_palette(iw_context *ctx, OptState &o)
{
	if(!(ctx->profile & (IW_PROFILE_PAL1 | IW_PROFILE_PAL2 | IW_PROFILE_PAL4 | IW_PROFILE_PAL8 |
		IW_PROFILE_GRAY1 | IW_PROFILE_GRAY2 | IW_PROFILE_GRAY4))) return;
	if(o.bit_depth != 8) return;
	o.pal = (struct iw_palette *)iw_malloc(ctx, sizeof(struct iw_palette));
	if(!o.pal) return;
	o.pal->num_entries = 0;
	static const int bpps[4] = {1, 2, 4, 8};
	static const unsigned int grayprof[4] = {IW_PROFILE_GRAY1, IW_PROFILE_GRAY2, IW_PROFILE_GRAY4, IW_PROFILE_GRAYSCALE};
	bool chosen = false, plain_gray = false;
	if(collect_palette(o)) {
		// preference: gray1, pal1, gray2, pal2, gray4, pal4, (8-bit gray), pal8
		for(int i = 0; i < 4 && !chosen && !plain_gray; i++) {
			bool bin;
			unsigned int shade;
			if(ctx->opt_gray && (ctx->profile & grayprof[i]) && gray_ok(ctx, o, bpps[i], &bin, &shade)) {
				if(bpps[i] == 8) { plain_gray = true; break; }
				make_gray_palette(o, bpps[i]);
				if(bin) {
					o.has_ckey = 1;
					o.ckey[0] = o.ckey[1] = o.ckey[2] = shade;
				}
				chosen = true;
			}
			else if(palette_ok(ctx, o, bpps[i])) chosen = true;
		}
		if(chosen) {
			if(!o.pal_is_gray) qsort(o.pal->entry, o.pal->num_entries, sizeof(struct iw_rgba8color), pal_order);
			to_palette_image(ctx, o);
		}
	}
	if(o.imgtype != IW_IMGTYPE_PALETTE) {
		iw_free(ctx, o.pal);
		o.pal = nullptr;
	}
}

}  // namespace

void optimize(iw_context *ctx)
{
	OptState &o = ctx->opt;
	o.width = ctx->img2.width;
	o.height = ctx->img2.height;
	o.imgtype = ctx->img2.imgtype;
	o.bit_depth = ctx->img2.bit_depth;
	o.bpr = ctx->img2.bpr;
	o.pix = ctx->img2.pixels;
	if(ctx->img2.has_bkgdlabel) {
		o.has_label = 1;
		for(int k = 0; k < 4; k++)
			o.label[k] = iw_color_get_int_sample(&ctx->img2.bkgdlabel, k, ctx->img2.bit_depth == 8 ? 255 : 65535);
	}
	if(ctx->img2.sampletype != IW_SAMPLETYPE_UINT) return;
	if(ctx->reduced_out) return;
	// (transparent pixels were blackened on the device)

	if(o.has_label) {
		if(o.label[0] != o.label[1] || o.label[0] != o.label[2]) o.has_color = 1;
		if(o.bit_depth == 16 && (o.label[0] % 257 || o.label[1] % 257 || o.label[2] % 257)) o.has_16bit = 1;
	}
	bool scanned;
	if(ctx->opt_dev_props & 0x100) {   // the same scan, done on the device over the whole image
		const int f = ctx->opt_dev_props;
		if(f & 1) o.has_16bit = 1;
		if(f & 2) o.has_trns = 1;
		if(f & 4) o.has_partial_trns = 1;
		if(f & 8) o.has_color = 1;
		scanned = true;
	}
	else scanned = scan_pixels(o);
	if(scanned) {
		if(o.bit_depth == 16 && !o.has_16bit) to_8bit(ctx, o, nch_of(o.imgtype));
		if(!o.has_trns && ctx->opt_strip) {
			if(o.imgtype == IW_IMGTYPE_RGBA) pick(ctx, o, IW_IMGTYPE_RGB, 0, 1, 2);
			else if(o.imgtype == IW_IMGTYPE_GRAYA) pick(ctx, o, IW_IMGTYPE_GRAY, 0, 0, 0);
		}
		if(!o.has_color && (ctx->profile & IW_PROFILE_GRAYSCALE) && ctx->opt_gray) {
			if(o.imgtype == IW_IMGTYPE_RGB) pick(ctx, o, IW_IMGTYPE_GRAY, 0, 0, 0);
			else if(o.imgtype == IW_IMGTYPE_RGBA) pick(ctx, o, IW_IMGTYPE_GRAYA, 0, 3, 0);
		}
	}
	try_palette(ctx, o);
	if((o.imgtype == IW_IMGTYPE_RGBA || o.imgtype == IW_IMGTYPE_GRAYA) && !o.has_partial_trns) try_binary_trns(ctx, o);
}

}  // namespace iwg
