// plan.cpp -- host planning for iw_process_image().
//
// Resolves every decision of the reference's iw_prepare_processing
// (src/imagew-main.c:1463-2248): crop clamp, colour spaces, max colour codes,
// background strategy, the channel-layout strategy tables, output depth,
// dither and colour counts.  The result is a Plan: channel maps plus the
// weight sets and quantisation tables the GPU passes consume.
#include "iwg_internal.h"

#include <cmath>
#include <cstring>
#include <thread>
#include <ctime>

namespace iwg {

// ---- colour transfer functions (src/imagew-main.c:28-96, :427-446) --------

double to_linear(double v, const struct iw_csdescr &cs)
{
	switch(cs.cstype) {
	case IW_CSTYPE_LINEAR:
		return v;
	case IW_CSTYPE_GAMMA:
		return pow(v, cs.gamma);
	case IW_CSTYPE_REC709:
		if(v < 4.5 * 0.020) return v / 4.5;
		return pow((v + 0.099) / 1.099, 1.0 / 0.45);
	default:
		if(v <= 0.04045) return v / 12.92;
		return pow((v + 0.055) / (1.055), 2.4);
	}
}

double from_linear(double v, const struct iw_csdescr &cs)
{
	if(v > 0.999999999) return 1.0;
	switch(cs.cstype) {
	case IW_CSTYPE_LINEAR:
		return v;
	case IW_CSTYPE_GAMMA:
		return pow(v, 1.0 / cs.gamma);
	case IW_CSTYPE_REC709:
		if(v < 0.020) return 4.5 * v;
		return 1.099 * pow(v, 0.45) - 0.099;
	default:
		if(v <= 0.0031308) return 12.92 * v;
		return 1.055 * pow(v, 1.0 / 2.4) - 0.055;
	}
}

// src/imagew-main.c:278-305
double gray_of(const Plan &P, double r, double g, double b)
{
	if(P.gsf == IW_GSF_WEIGHTED) return P.gsw[0] * r + P.gsw[1] * g + P.gsw[2] * b;
	if(P.gsf == IW_GSF_ORDERBYVALUE) {
		double hi, mid, lo;
		if(g <= r) { hi = r; mid = g; } else { hi = g; mid = r; }
		if(b <= mid) lo = b;
		else {
			lo = mid;
			if(b <= hi) mid = b;
			else { mid = hi; hi = b; }
		}
		return P.gsw[0] * hi + P.gsw[1] * mid + P.gsw[2] * lo;
	}
	return 0.0;
}

static int ctype_of(int imgtype, int ch)
{
	switch(imgtype) {
	case IW_IMGTYPE_GRAY: return ch == 0 ? IW_CHANNELTYPE_GRAY : 0;
	case IW_IMGTYPE_GRAYA: return ch == 0 ? IW_CHANNELTYPE_GRAY : (ch == 1 ? IW_CHANNELTYPE_ALPHA : 0);
	case IW_IMGTYPE_RGB: return ch <= 2 ? ch : 0;
	case IW_IMGTYPE_RGBA: return ch <= 3 ? ch : 0;
	}
	return 0;
}

static int alpha_index(int t)
{
	return t == IW_IMGTYPE_RGBA ? 3 : (t == IW_IMGTYPE_GRAYA ? 1 : 0);
}

// src/imagew-main.c:813-828
static int bkgd_has_trns(const iw_context *ctx, const Plan &P)
{
	if(!P.apply_bk) return 0;
	if(!(ctx->profile & IW_PROFILE_TRANSPARENCY)) return 0;
	if(P.bk_strategy == BK_EARLY) return 0;
	if(P.bk_source == BKSRC_FILE) return ctx->inlabel.c[3] < 1.0;
	if(P.bk_source == BKSRC_REQ) {
		if(P.bk_checker && ctx->bkgd2.c[3] < 1.0) return 1;
		return ctx->bkgd.c[3] < 1.0;
	}
	return 0;
}

// src/imagew-main.c:1734-1823
static void decide_bkgd(iw_context *ctx, Plan &P)
{
	if(!IW_IMGTYPE_HAS_ALPHA(P.in_logtype)) {
		P.apply_bk = 0;
		return;
	}
	if(ctx->inlabel_set && (ctx->use_file_label || !ctx->bkgd_valid)) P.bk_source = BKSRC_FILE;
	else if(ctx->bkgd_valid) {
		P.bk_source = BKSRC_REQ;
		P.bk_checker = ctx->bkgd_checker;
	}
	else P.bk_source = BKSRC_NONE;

	if(P.bk_checker && ctx->check_size < 1) ctx->check_size = 1;
	if(ctx->bkgd_valid) P.apply_bk = 1;
	if(!(ctx->profile & IW_PROFILE_TRANSPARENCY)) {
		if(!ctx->bkgd_valid && !P.apply_bk)
			iw_warning(ctx, "This image may have transparency, which is incompatible with the output format. A background color will be applied.");
		P.apply_bk = 1;
	}
	if(ctx->dim[0].use_offset || ctx->dim[1].use_offset) {
		if(!ctx->bkgd_valid && !P.apply_bk)
			iw_warning(ctx, "This image may have transparency, which is incompatible with a channel offset. A background color will be applied.");
		P.apply_bk = 1;
		if(P.bk_checker && ctx->bkgd_checker) {
			iw_warning(ctx, "Checkerboard backgrounds are not supported when using a channel offset.");
			P.bk_checker = 0;
		}
		P.bk_strategy = BK_EARLY;
		return;
	}
	if(!P.apply_bk) return;
	P.bk_strategy = BK_LATE;   // checkerboards need LATE; solid colours use it too
}

// Channel-layout strategies (src/imagew-main.c:1613-1718).  A strategy is a
// pair (input layout, output layout) with layouts numbered G=1 GA=2 RGB=3 RGBA=4.
struct Strat { int in, out; bool operator==(const Strat &o) const { return in == o.in && out == o.out; } };

static void decide_strategy(iw_context *ctx, const Plan &P, Strat &s1, Strat &s2)
{
	int in = P.in_logtype == IW_IMGTYPE_RGBA ? 4 : P.in_logtype == IW_IMGTYPE_RGB ? 3 : P.in_logtype == IW_IMGTYPE_GRAYA ? 2 : 1;
	bool alpha = (in == 2 || in == 4);
	if(ctx->to_gray) { s1 = {in, alpha ? 2 : 1}; s2 = alpha ? Strat{2, 2} : Strat{1, 1}; }
	else { s1 = {in, alpha ? 4 : 3}; s2 = alpha ? Strat{4, 4} : Strat{3, 3}; }

	if(P.apply_bk && P.bk_strategy == BK_EARLY) {
		if(s1 == Strat{4, 4}) { s1 = {4, 3}; s2 = {3, 3}; }
		else if(s1 == Strat{2, 2}) { s1 = {2, 1}; s2 = {1, 1}; }
		else if(s1 == Strat{2, 4}) { s1 = {2, 3}; s2 = {3, 3}; }
		else if(s1 == Strat{4, 2}) { s1 = {4, 1}; s2 = {1, 1}; }
	}
	if(P.apply_bk && !bkgd_has_trns(ctx, P)) {
		if(s2 == Strat{2, 2}) s2 = {2, 1};
		else if(s2 == Strat{4, 4}) s2 = {4, 3};
	}
}

// src/imagew-main.c:1546-1611
static void prepare_bkgd(iw_context *ctx, Plan &P)
{
	struct iw_color b1 = {{1.0, 0.0, 1.0, 1.0}}, b2 = {{0.0, 0.0, 0.0, 1.0}};
	if(P.bk_source == BKSRC_FILE) {
		b1 = P.inlabel_lin;
		P.bk_checker = 0;
	}
	else if(P.bk_source == BKSRC_REQ) {
		b1 = ctx->bkgd;
		if(ctx->bkgd_checker) b2 = ctx->bkgd2;
	}
	if(P.bk_strategy == BK_EARLY) P.bk1_alpha = 1.0;
	else {
		P.bk1_alpha = b1.c[3];
		P.bk2_alpha = b2.c[3];
	}
	int ot = P.out_type;
	if(P.bk_strategy == BK_LATE && (ot == IW_IMGTYPE_RGB || ot == IW_IMGTYPE_RGBA)) {
		for(int i = 0; i < 3; i++) {
			P.out[i].bk1 = b1.c[i];
			if(P.bk_checker) P.out[i].bk2 = b2.c[i];
		}
	}
	else if(P.bk_strategy == BK_LATE && (ot == IW_IMGTYPE_GRAY || ot == IW_IMGTYPE_GRAYA)) {
		P.out[0].bk1 = gray_of(P, b1.c[0], b1.c[1], b1.c[2]);
		if(P.bk_checker) P.out[0].bk2 = gray_of(P, b2.c[0], b2.c[1], b2.c[2]);
	}
	else if(P.bk_strategy == BK_EARLY && ot == IW_IMGTYPE_RGB) {
		for(int i = 0; i < 3; i++) P.mid[i].bk_early = b1.c[i];
	}
	else if(P.bk_strategy == BK_EARLY && ot == IW_IMGTYPE_GRAY) {
		P.mid[0].bk_early = gray_of(P, b1.c[0], b1.c[1], b1.c[2]);
	}
}

// Whether the reference's allocators would give a buffer of n bytes
// (iw_malloc) or of n1 x n2 bytes (iw_malloc_large) under the context's
// allocation limit; sets their error when not.
static bool ref_fits(iw_context *ctx, size_t n)
{
	if(n <= ctx->max_malloc) return true;
	iw_set_error(ctx, "Out of memory");
	return false;
}

static bool ref_fits_large(iw_context *ctx, size_t n1, size_t n2)
{
	if(n2 && n1 > ctx->max_malloc / n2) {
		iw_set_error(ctx, "Image too large to process");
		return false;
	}
	return ref_fits(ctx, n1 * n2);
}

// The reference converts each float sample of a colour channel to linear
// light with libm as it reads it (x_to_linear_sample of the raw float,
// src/imagew-main.c:53-66 and :353-359; alpha samples are not converted).
// Here the host converts the stored image once, with the same formulas
// (to_linear) and glibc, on all host threads; the device passes read the
// resulting doubles (Plan::lin_in).  Samples are read as stored (4 bytes
// each, rows P.in_bpr apart); the copy keeps the stored layout, one double per
// sample.
static void linearise_float_input(iw_context *ctx, Plan &P)
{
	const iw_image &im = ctx->img1;
	const int pw = P.orient >= 4 ? P.img1_h : P.img1_w;   // stored width and rows
	const int ph = P.orient >= 4 ? P.img1_w : P.img1_h;
	const int nphys = P.in_nphys;
	const int alpha = IW_IMGTYPE_HAS_ALPHA(im.imgtype) ? nphys - 1 : -1;
	const size_t per_row = (size_t)pw * nphys;
	auto out = std::make_shared<std::vector<double>>(per_row * (size_t)(ph > 0 ? ph : 0));
	const iw_csdescr cs = ctx->cs_in;
	const unsigned char *base = (const unsigned char *)im.pixels;
	auto rows = [&](int r0, int r1) {
		for(int r = r0; r < r1; r++) {
			const unsigned char *src = base + (size_t)r * P.in_bpr;
			double *dst = out->data() + (size_t)r * per_row;
			for(size_t k = 0; k < per_row; k++) {
				float f;
				memcpy(&f, src + 4 * k, 4);
				const int ch = (int)(k % (size_t)nphys);
				dst[k] = ch == alpha ? (double)f : to_linear((double)f, cs);
			}
		}
	};
	const int nt = std::max(1, std::min((int)std::thread::hardware_concurrency(), ph / 16));
	if(nt <= 1) rows(0, ph);
	else {
		std::vector<std::thread> th;
		for(int t = 0; t < nt; t++) th.emplace_back(rows, (int)((long long)ph * t / nt), (int)((long long)ph * (t + 1) / nt));
		for(std::thread &x : th) x.join();
	}
	P.lin_in = out;
	P.lin_bpr = per_row * sizeof(double);
}

bool build_plan(iw_context *ctx, Plan &P)
{
	int w = ctx->canvas_w, h = ctx->canvas_h;

	if(!ctx->profile) {
		iw_set_error(ctx, "Output profile not set");
		return false;
	}
	if(ctx->randomize) ctx->seed = (int)time(nullptr);
	ctx->dim[0].true_size = ctx->true_valid ? ctx->true_w : (double)w;
	ctx->dim[1].true_size = ctx->true_valid ? ctx->true_h : (double)h;
	if(!iw_check_image_dimensions(ctx, ctx->img1.width, ctx->img1.height)) return false;
	if(!iw_check_image_dimensions(ctx, w, h)) return false;

	if(ctx->to_gray) {
		if(ctx->gsf == IW_GSF_STANDARD) { ctx->gsf = IW_GSF_WEIGHTED; iw_set_grayscale_weights(ctx, 0.212655, 0.715158, 0.072187); }
		else if(ctx->gsf == IW_GSF_COMPATIBLE) { ctx->gsf = IW_GSF_WEIGHTED; iw_set_grayscale_weights(ctx, 0.299, 0.587, 0.114); }
	}
	P.gsf = ctx->gsf;
	for(int i = 0; i < 3; i++) P.gsw[i] = ctx->gsw[i];

	// input layout; a transparent edge adds a virtual alpha channel
	const iw_image &im = ctx->img1;
	P.in_type = im.imgtype;
	P.in_depth = im.bit_depth;
	P.in_sampletype = im.sampletype;
	P.orient = (int)im.orient_transform;
	P.img1_w = im.width;
	P.img1_h = im.height;
	P.in_bpr = im.bpr;
	P.in_logtype = im.imgtype;
	if(ctx->dim[0].edge == IW_EDGE_POLICY_TRANSPARENT || ctx->dim[1].edge == IW_EDGE_POLICY_TRANSPARENT) {
		if(im.imgtype == IW_IMGTYPE_GRAY) P.in_logtype = IW_IMGTYPE_GRAYA;
		else if(im.imgtype == IW_IMGTYPE_RGB) P.in_logtype = IW_IMGTYPE_RGBA;
	}
	P.in_nphys = iw_imgtype_num_channels(im.imgtype);
	P.in_nlog = iw_imgtype_num_channels(P.in_logtype);
	P.in_alpha = alpha_index(P.in_logtype);
	for(int i = 0; i < P.in_nlog; i++) {
		P.mid[i].ctype = ctype_of(P.in_logtype, i);
		P.mid[i].in_ch = i;
		if(i >= P.in_nphys) P.in_slow[i] = 1;
	}
	P.out_w = w;
	P.out_h = h;
	ctx->img2.width = w;
	ctx->img2.height = h;

	// crop, clamped like the reference (including its use of the x origin
	// when the y origin lies past the bottom edge)
	P.crop_x = ctx->crop_x; P.crop_y = ctx->crop_y; P.crop_w = ctx->crop_w; P.crop_h = ctx->crop_h;
	if(P.crop_x < 0) P.crop_x = 0;
	if(P.crop_y < 0) P.crop_y = 0;
	if(P.crop_x > im.width - 1) P.crop_x = im.width - 1;
	if(P.crop_y > im.height - 1) P.crop_x = im.height - 1;
	if(P.crop_w < 0) P.crop_w = im.width - P.crop_x;
	if(P.crop_h < 0) P.crop_h = im.height - P.crop_y;
	if(P.crop_w < 1) P.crop_w = 1;
	if(P.crop_h < 1) P.crop_h = 1;
	if(P.crop_w > im.width - P.crop_x) P.crop_w = im.width - P.crop_x;
	if(P.crop_h > im.height - P.crop_y) P.crop_h = im.height - P.crop_y;
	ctx->crop_x = P.crop_x; ctx->crop_y = P.crop_y; ctx->crop_w = P.crop_w; ctx->crop_h = P.crop_h;

	// output colour space
	if(ctx->cs_out_valid) {
		ctx->cs_out = ctx->cs_out_req;
		if((ctx->profile & IW_PROFILE_ALWAYSLINEAR) && ctx->cs_out.cstype != IW_CSTYPE_LINEAR) {
			iw_warning(ctx, "Forcing output colorspace to linear; required by the output format.");
			iw_make_linear_csdescr(&ctx->cs_out);
		}
	}
	else if(ctx->profile & IW_PROFILE_ALWAYSLINEAR) iw_make_linear_csdescr(&ctx->cs_out);
	else iw_make_srgb_csdescr_2(&ctx->cs_out);

	// input max colour codes
	if(im.sampletype != IW_SAMPLETYPE_FLOATINGPOINT) {
		P.in_max = (1 << im.bit_depth) - 1;
		for(int i = 0; i < kMaxCh; i++) {
			if(ctx->in_maxcc[i] <= 0) ctx->in_maxcc[i] = P.in_max;
			P.in_maxcc_d[i] = (double)ctx->in_maxcc[i];
			if(ctx->in_maxcc[i] != P.in_max) P.reduced_in = 1;
		}
	}
	if(P.reduced_in || im.sampletype == IW_SAMPLETYPE_FLOATINGPOINT)
		for(int i = 0; i < P.in_nphys; i++) P.in_slow[i] = 1;

	for(int i = 0; i < 2; i++)
		for(int j = 0; j < 3; j++)
			if(fabs(ctx->dim[i].chan_offset[j]) > 0.00001) ctx->dim[i].use_offset = 1;
	if(ctx->to_gray && (ctx->dim[0].use_offset || ctx->dim[1].use_offset)) {
		iw_warning(ctx, "Disabling channel offset, due to grayscale output.");
		ctx->dim[0].use_offset = ctx->dim[1].use_offset = 0;
	}

	decide_bkgd(ctx, P);
	for(int i = 0; i < 2; i++)
		if(ctx->dim[i].use_offset || (P.apply_bk && P.bk_strategy == BK_EARLY && ctx->dim[i].edge == IW_EDGE_POLICY_TRANSPARENT))
			ctx->dim[i].no_cache = 1;

	Strat s1, s2;
	decide_strategy(ctx, P, s1, s2);
	if(s1 == Strat{4, 4}) P.mid_type = IW_IMGTYPE_RGBA;
	else if(s1 == Strat{2, 4}) {
		P.mid_type = IW_IMGTYPE_RGBA;
		P.mid[0].in_ch = P.mid[1].in_ch = P.mid[2].in_ch = 0;
		P.mid[3].in_ch = 1;
	}
	else if(s1 == Strat{3, 3} || s1 == Strat{4, 3}) P.mid_type = IW_IMGTYPE_RGB;
	else if(s1 == Strat{1, 3} || s1 == Strat{2, 3}) {
		P.mid_type = IW_IMGTYPE_RGB;
		P.mid[0].in_ch = P.mid[1].in_ch = P.mid[2].in_ch = 0;
	}
	else if(s1 == Strat{4, 2}) {
		P.mid_type = IW_IMGTYPE_GRAYA;
		P.mid[0].to_gray = 1;
		P.mid[0].in_ch = 0;
		P.mid[1].in_ch = 3;
	}
	else if(s1 == Strat{2, 2}) P.mid_type = IW_IMGTYPE_GRAYA;
	else if(s1 == Strat{3, 1}) { P.mid_type = IW_IMGTYPE_GRAY; P.mid[0].to_gray = 1; P.mid[0].in_ch = 0; }
	else if(s1 == Strat{1, 1}) { P.mid_type = IW_IMGTYPE_GRAY; P.mid[0].in_ch = 0; }
	else {
		// GA->G and RGBA->G: the reference has no case for these either
		iw_set_errorf(ctx, "Internal error, unknown strategy %d", 0x0 | (s1.in << 4) | s1.out);
		return false;
	}
	P.mid_n = iw_imgtype_num_channels(P.mid_type);
	P.mid_alpha = IW_IMGTYPE_HAS_ALPHA(P.mid_type) ? alpha_index(P.mid_type) : -1;
	for(int i = 0; i < P.mid_n; i++) P.mid[i].out_ch = i;

	if(s2 == Strat{4, 4}) P.out_type = IW_IMGTYPE_RGBA;
	else if(s2 == Strat{3, 3}) P.out_type = IW_IMGTYPE_RGB;
	else if(s2 == Strat{4, 3}) { P.out_type = IW_IMGTYPE_RGB; P.mid[3].out_ch = -1; }
	else if(s2 == Strat{2, 2}) P.out_type = IW_IMGTYPE_GRAYA;
	else if(s2 == Strat{1, 1}) P.out_type = IW_IMGTYPE_GRAY;
	else if(s2 == Strat{2, 1}) { P.out_type = IW_IMGTYPE_GRAY; P.mid[1].out_ch = -1; }
	else {
		iw_set_error(ctx, "Internal error");
		return false;
	}
	ctx->img2.imgtype = P.out_type;
	P.out_n = iw_imgtype_num_channels(P.out_type);
	for(int i = 0; i < P.mid_n; i++) P.mid[i].ctype = ctype_of(P.mid_type, i);
	for(int i = 0; i < P.out_n; i++) P.out[i].ctype = ctype_of(P.out_type, i);
	if(P.mid_alpha >= 0)
		for(int i = 0; i < P.mid_n; i++)
			if(P.mid[i].ctype != IW_CHANNELTYPE_ALPHA) P.mid[i].unassoc = 1;

	// output sample type and depth (src/imagew-main.c:1514-1541)
	if(ctx->profile & IW_PROFILE_HDRI) {
		P.out_sampletype = IW_SAMPLETYPE_FLOATINGPOINT;
		P.out_depth = 32;
	}
	else {
		P.out_sampletype = IW_SAMPLETYPE_UINT;
		if(ctx->req_depth > 8 && (ctx->profile & IW_PROFILE_16BPS)) P.out_depth = 16;
		else {
			if(ctx->req_depth > 8) iw_warning(ctx, "Reducing depth to 8; required by the output format.");
			P.out_depth = 8;
		}
	}
	ctx->img2.sampletype = P.out_sampletype;
	ctx->img2.bit_depth = P.out_depth;

	if(P.out_sampletype == IW_SAMPLETYPE_FLOATINGPOINT) {
		bool any = false;
		for(int i = 0; i < kNCTypes; i++) if(ctx->req_cc[i]) any = true;
		if(any) iw_warning(ctx, "Posterization is not supported with floating point output.");
	}
	else {
		int omax = (1 << P.out_depth) - 1;
		for(int i = 0; i < P.out_n; i++) P.out[i].maxcc = omax;
		if(ctx->profile & IW_PROFILE_REDUCEDBITDEPTHS) {
			for(int i = 0; i < P.out_n; i++) {
				int m = ctx->req_maxcc[P.out[i].ctype];
				if(m > 0) P.out[i].maxcc = m > omax ? omax : m;
			}
		}
		for(int i = 0; i < P.out_n; i++)
			if(P.out[i].maxcc != omax) { P.reduced_out = 1; P.no_out_tables = 1; }
	}
	ctx->reduced_out = P.reduced_out;
	for(int i = 0; i < P.out_n; i++) {
		OutChannel &o = P.out[i];
		o.cc = ctx->req_cc[o.ctype];
		if(o.cc) {
			if(o.cc < 2) o.cc = 2;
			else if(o.cc > o.maxcc) o.cc = o.maxcc;
		}
		if(o.cc == 1 + o.maxcc) o.cc = 0;
		o.dfam = ctx->dfam[o.ctype];
		o.dsub = ctx->dsub[o.ctype];
		if(o.dfam == IW_DITHERFAMILY_ERRDIFF) P.errdiff = 1;
		ctx->out_maxcc[i] = o.maxcc;
	}

	if(ctx->inlabel_set) {
		for(int i = 0; i < 3; i++) P.inlabel_lin.c[i] = to_linear(ctx->inlabel.c[i], ctx->cs_in);
		P.inlabel_lin.c[3] = ctx->inlabel.c[3];
	}
	if(P.apply_bk) prepare_bkgd(ctx, P);
	P.bk_trns = bkgd_has_trns(ctx, P);
	P.check_size = ctx->check_size;
	P.check_origin[0] = ctx->check_origin[0];
	P.check_origin[1] = ctx->check_origin[1];

	ctx->img2.rendering_intent = ctx->req_intent == IW_INTENT_UNKNOWN ? im.rendering_intent : ctx->req_intent;

	// default filters (src/imagew-main.c:1825-1840)
	for(int d = 0; d < 2; d++) {
		if(ctx->dim[d].family != IW_RESIZETYPE_AUTO) continue;
		int n_in = d == 0 ? P.crop_w : P.crop_h, n_out = d == 0 ? w : h;
		if(n_out == n_in && !ctx->dim[d].use_offset && !ctx->true_valid && ctx->dim[d].translate == 0.0)
			iw_set_resize_alg(ctx, d, IW_RESIZETYPE_NULL, 1.0, 0.0, 0.0);
		else
			iw_set_resize_alg(ctx, d, IW_RESIZETYPE_CUBIC, 1.0, 0.0, 0.5);
	}
	if(IW_IMGTYPE_HAS_ALPHA(P.out_type) && !ctx->opt_strip) {
		ctx->opt_pal = 0;
		ctx->opt_bintrns = 0;
	}

	// ---- beyond the reference's planning: resolve the work as data ----
	P.cs_in = ctx->cs_in;
	P.cs_out = ctx->cs_out;
	P.no_gamma = ctx->no_gamma;
	P.intclamp = ctx->intclamp;
	P.negate = ctx->negate;
	P.out_bpr = iw_calc_bytesperrow(w, P.out_depth * P.out_n);
	P.blacken = P.out_sampletype == IW_SAMPLETYPE_UINT && !P.reduced_out && IW_IMGTYPE_HAS_ALPHA(P.out_type);

	if(im.sampletype == IW_SAMPLETYPE_FLOATINGPOINT && im.bit_depth == 32 && !ctx->no_gamma &&
		ctx->cs_in.cstype != IW_CSTYPE_LINEAR)
		linearise_float_input(ctx, P);

	// The reference's buffers and their size limits, checked without
	// allocating, in its order, before any device work
	// (src/imagew-main.c:1385-1417, :851-858, :979-985).  This library keeps
	// its images on the device, but a job the reference refuses is refused
	// here with the same message: an image whose output or intermediate
	// exceeds the allocation limit ("Image too large to process"), and a crop
	// that the reference's clamp leaves with a negative size (a negative
	// width fails at the intermediate image, a negative height at the
	// vertical pass's column buffer, "Out of memory").
	{
		const size_t mid_px = (size_t)(long long)((long long)P.crop_w * h);   // an int product there
		if(!ref_fits_large(ctx, P.out_bpr, (size_t)h)) return false;
		if(!ref_fits_large(ctx, mid_px, sizeof(float))) return false;
		if(P.errdiff)
			for(int k = 0; k < 3; k++)
				if(!ref_fits(ctx, (size_t)w * sizeof(double))) return false;
		if(IW_IMGTYPE_HAS_ALPHA(P.mid_type)) {
			if(!ref_fits_large(ctx, mid_px, sizeof(float))) return false;
			if(!ref_fits_large(ctx, (size_t)(long long)((long long)w * h), sizeof(float))) return false;
		}
	}

	// A crop that the reference's clamp leaves without rows or columns (its y
	// origin at the image's height): the reference carries on and resamples
	// from empty column buffers, reading past their end.  It is refused here,
	// before any weight list is built on an empty source, whenever both
	// passes' column buffers fit the allocation limit (when one does not, the
	// loop below reports the reference's own error first).
	{
		auto fits = [&](size_t n) { return n <= ctx->max_malloc; };
		bool cols_fit = true;
		for(int d = 1; d >= 0; d--) {
			int n_in = d == 0 ? P.crop_w : P.crop_h, n_out = d == 0 ? w : h;
			cols_fit = cols_fit && fits((size_t)(long long)n_in * sizeof(double)) && fits((size_t)n_out * sizeof(double));
		}
		if(cols_fit && (P.crop_w < 1 || P.crop_h < 1)) {
			iw_set_error(ctx, "Input crop is empty");
			return false;
		}
	}

	// Weight sets.  One per dimension unless a channel offset or an early
	// background on a transparent edge makes them differ per channel
	// (src/imagew-main.c:2031-2045).  Vertical first, each after its pass's
	// column buffers, as the reference builds them.
	for(int d = 1; d >= 0; d--) {
		int n_in = d == 0 ? P.crop_w : P.crop_h, n_out = d == 0 ? w : h;
		if(!ref_fits(ctx, (size_t)(long long)n_in * sizeof(double))) return false;
		if(!ref_fits(ctx, (size_t)n_out * sizeof(double))) return false;
		P.wsets[d].clear();
		for(int m = 0; m < P.mid_n; m++) {
			const MidChannel &mc = P.mid[m];
			double edge_bk = (P.apply_bk && P.bk_strategy == BK_EARLY)
				? P.mid[mc.ctype < kMaxCh ? mc.ctype : 0].bk_early : 0.0;
			auto wt = build_weights(ctx, ctx->dim[d], mc.ctype, n_in, n_out, edge_bk);
			if(!wt) return false;
			int found = -1;
			for(size_t k = 0; k < P.wsets[d].size(); k++)
				if(P.wsets[d][k]->same_as(*wt)) { found = (int)k; break; }
			if(found < 0) {
				found = (int)P.wsets[d].size();
				P.wsets[d].push_back(wt);
			}
			if(d == 0) P.mid[m].wset_h = found;
			else P.mid[m].wset_v = found;
		}
	}
	if(P.crop_w < 1 || P.crop_h < 1) {
		// (the check before the weight lists refuses these first; this one
		// stays so that no device pass can ever see an empty source)
		iw_set_error(ctx, "Input crop is empty");
		return false;
	}

	// decode transfer per intermediate channel: alpha and no-gamma use linear
	for(int m = 0; m < P.mid_n; m++)
		P.mid[m].lin_cs = (P.mid[m].ctype == IW_CHANNELTYPE_ALPHA) || P.no_gamma;

	// quantisation tables per output channel
	if(P.out_sampletype == IW_SAMPLETYPE_UINT) {
		bool nc_ok = !P.no_out_tables && !P.no_gamma && P.cs_out.cstype != IW_CSTYPE_LINEAR &&
			P.out_depth <= 8 && ((size_t)w) * h > 512;
		for(int i = 0; i < P.out_n; i++) {
			OutChannel &o = P.out[i];
			bool is_alpha = o.ctype == IW_CHANNELTYPE_ALPHA;
			Quant &q = o.q;
			q.maxcc = o.maxcc;
			q.cc = o.cc;
			q.dfam = o.dfam;
			q.dsub = o.dsub;
			bool lin = is_alpha || P.no_gamma;
			q.cstype = lin ? IW_CSTYPE_LINEAR : P.cs_out.cstype;
			q.gamma = lin ? 0.0 : P.cs_out.gamma;
			q.use_nc = nc_ok && !is_alpha && o.dfam == IW_DITHERFAMILY_NONE && o.cc == 0;
			build_quant(q);
		}
	}
	else {
		for(int i = 0; i < P.out_n; i++) P.out[i].q.float_out = 1;
	}
	return true;
}

// Nearest representable code for a background-label colour component
// (calc_sample_convert_from_linear, src/imagew-main.c:769-799).
static unsigned int label_code(double v, const struct iw_csdescr &cs, double maxc)
{
	if(v < 0.0) v = 0.0;
	if(v > 1.0) v = 1.0;
	double e = from_linear(v, cs) * maxc;
	if(e > maxc) e = maxc;
	if(e < 0.0) e = 0.0;
	double lo = floor(e), hi = ceil(e), s;
	if((unsigned int)lo == (unsigned int)hi) s = lo;
	else {
		double llo, lhi;
		if(cs.cstype == IW_CSTYPE_LINEAR) { llo = lo / maxc; lhi = hi / maxc; }
		else { llo = to_linear(((double)(unsigned int)lo) / maxc, cs); lhi = to_linear(((double)(unsigned int)hi) / maxc, cs); }
		s = (lhi - v <= v - llo) ? hi : lo;
	}
	return (unsigned int)(0.5 + s);
}

// Quantised background label of the output image (src/imagew-main.c:1238-1322).
void bkgd_label(iw_context *ctx, const Plan &P)
{
	if(!(ctx->profile & (IW_PROFILE_PNG_BKGD | IW_PROFILE_RGB8_BKGD | IW_PROFILE_RGB16_BKGD))) return;
	if(ctx->no_outlabel) return;
	struct iw_color c = {{1.0, 0.0, 1.0, 1.0}};
	if(ctx->outlabel_valid) c = ctx->outlabel;
	else if(ctx->inlabel_set) c = P.inlabel_lin;
	else return;
	if(ctx->to_gray) {
		double g = gray_of(P, c.c[0], c.c[1], c.c[2]);
		c.c[0] = c.c[1] = c.c[2] = g;
	}
	double maxc;
	if(ctx->profile & IW_PROFILE_RGB8_BKGD) maxc = 255.0;
	else if(ctx->profile & IW_PROFILE_RGB16_BKGD) maxc = 65535.0;
	else if(ctx->img2.bit_depth == 8) maxc = 255.0;
	else if(ctx->img2.bit_depth == 16) maxc = 65535.0;
	else return;
	for(int k = 0; k < 3; k++) ctx->img2.bkgdlabel.c[k] = ((double)label_code(c.c[k], ctx->cs_out, maxc)) / maxc;
	unsigned int u;
	if(c.c[3] <= 0.0) u = 0;
	else if(c.c[3] >= 1.0) u = (unsigned int)maxc;
	else u = (unsigned int)(0.5 + c.c[3] * (unsigned int)maxc);
	ctx->img2.bkgdlabel.c[3] = ((double)u) / maxc;
	ctx->img2.has_bkgdlabel = 1;
}

}  // namespace iwg
