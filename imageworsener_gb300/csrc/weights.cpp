// weights.cpp -- resampling weight lists (host).
//
// Each output pixel of a resampling pass is a weighted sum of input pixels.
// The weights come from one of 13 filter kernels, scaled for downsampling,
// optionally blurred, shifted by translation / channel offsets, and
// normalised to sum to 1 (src/imagew-resize.c:62-556).  They are computed here
// in double precision with the host libm, exactly as the reference computes
// them, and stored as CSR lists in the reference's accumulation order.  The
// GPU passes then only multiply and add.
#include "iwg_internal.h"

#include <cmath>
#include <cstring>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

namespace iwg {

bool Weights::same_as(const Weights &o) const
{
	return kind == o.kind && n_in == o.n_in && n_out == o.n_out && edge_value == o.edge_value &&
		off == o.off && src == o.src && w == o.w && pos == o.pos;
}

namespace {

struct Kernel {
	int family = 0;
	double radius = 0, b = 0, c = 0, mix = 0;
};

double sinc(double x)
{
	if(x <= 0.000000005) return 1.0;
	return sin(M_PI * x) / (M_PI * x);
}

// Kernel value at distance x >= 0 (src/imagew-resize.c:62-185).
double kernel_at(const Kernel &k, double x)
{
	const double r = k.radius;
	switch(k.family) {
	case IW_RESIZETYPE_LANCZOS: return x < r ? sinc(x) * sinc(x / r) : 0.0;
	case IW_RESIZETYPE_HANNING: return x < r ? sinc(x) * (0.5 * cos(M_PI * x / r) + 0.5) : 0.0;
	case IW_RESIZETYPE_BLACKMAN:
		if(x >= r) return 0.0;
		return sinc(x) * (0.5 * cos(M_PI * x / r) + 0.08 * cos(2.0 * M_PI * x / r) + 0.42);
	case IW_RESIZETYPE_SINC: return x < r ? sinc(x) : 0.0;
	case IW_RESIZETYPE_GAUSSIAN: {
		if(x >= 2.0) return 0.0;
		double g = exp(-2.0 * x * x) * 0.79788456080286535587989;   // 1/sqrt(pi/2)
		if(x <= 1.999) return g;
		return 1000.0 * (2.0 - x) * g;   // taper to 0 at 2.0
	}
	case IW_RESIZETYPE_TRIANGLE: return x < 1.0 ? 1.0 - x : 0.0;
	case IW_RESIZETYPE_QUADRATIC:
		if(x < 0.5) return 0.75 - x * x;
		if(x < 1.5) return 0.50 * (x - 1.5) * (x - 1.5);
		return 0.0;
	case IW_RESIZETYPE_CUBIC: {   // Mitchell-Netravali family
		double b = k.b, c = k.c;
		if(x < 1.0)
			return ((12.0 - 9.0 * b - 6.0 * c) * x * x * x + (-18.0 + 12.0 * b + 6.0 * c) * x * x + (6.0 - 2.0 * b)) / 6.0;
		if(x < 2.0)
			return ((-b - 6.0 * c) * x * x * x + (6.0 * b + 30.0 * c) * x * x + (-12.0 * b - 48.0 * c) * x + (8.0 * b + 24.0 * c)) / 6.0;
		return 0.0;
	}
	case IW_RESIZETYPE_HERMITE: return x < 1.0 ? 2.0 * x * x * x - 3.0 * x * x + 1.0 : 0.0;
	case IW_RESIZETYPE_BOX: return x <= 0.5 ? 1.0 : 0.0;
	case IW_RESIZETYPE_BOXAVG:
		if(x < 0.4999999) return 1.0;
		return x <= 0.5000001 ? 0.5 : 0.0;
	case IW_RESIZETYPE_MIX:
		if(x < (0.5 - k.mix / 2.0)) return 1.0;
		if(x < (0.5 + k.mix / 2.0)) return 0.5 - (x - 0.5) / k.mix;
		return 0.0;
	}
	return 0.0;
}

}  // namespace

std::shared_ptr<const Weights> build_weights(iw_context *ctx, const DimRequest &d, int ctype,
	int n_in, int n_out, double edge_bkgd_value)
{
	auto wt = std::make_shared<Weights>();
	Kernel k;
	k.family = d.family;
	bool standard = true, boxhack = false, sincfam = false;
	wt->n_in = n_in;
	wt->n_out = n_out;

	switch(d.family) {
	case IW_RESIZETYPE_NULL: standard = false; break;
	case IW_RESIZETYPE_NEAREST: standard = false; boxhack = true; break;
	case IW_RESIZETYPE_MIX:
		k.mix = ((double)n_out) / n_in;
		if(k.mix > 1.0) k.mix = 1.0 / k.mix;
		k.radius = 0.5 + k.mix;
		break;
	case IW_RESIZETYPE_BOX: k.radius = 0.501; boxhack = true; break;
	case IW_RESIZETYPE_BOXAVG: k.radius = 0.501; break;
	case IW_RESIZETYPE_TRIANGLE: k.radius = 1.0; break;
	case IW_RESIZETYPE_QUADRATIC: k.radius = 1.5; break;
	case IW_RESIZETYPE_GAUSSIAN: k.radius = 2.0; break;
	case IW_RESIZETYPE_HERMITE: k.radius = 1.0; break;
	case IW_RESIZETYPE_CUBIC:
		k.radius = 2.0;
		k.b = d.p1 < -100.0 ? -100.0 : (d.p1 > 100.0 ? 100.0 : d.p1);
		k.c = d.p2 < -100.0 ? -100.0 : (d.p2 > 100.0 ? 100.0 : d.p2);
		break;
	case IW_RESIZETYPE_LANCZOS: case IW_RESIZETYPE_HANNING:
	case IW_RESIZETYPE_BLACKMAN: case IW_RESIZETYPE_SINC:
		sincfam = true;
		break;
	default:
		iw_set_error(ctx, "Internal: Unknown resize algorithm");
		return nullptr;
	}
	if(sincfam) {   // "lobes", clamped to [2,100]
		k.radius = floor(d.p1 + 0.5);
		if(k.radius < 2.0) k.radius = 2.0;
		if(k.radius > 100.0) k.radius = 100.0;
	}
	wt->edge_value = d.edge == IW_EDGE_POLICY_TRANSPARENT ? edge_bkgd_value : 0.0;

	double offset = d.translate;
	if(boxhack) offset -= 0.00000000001;   // keep pixel centres off box borders
	if(d.use_offset && ctype >= 0 && ctype <= 2) offset += d.chan_offset[ctype];

	wt->off.assign(1, 0);
	if(!standard) {
		// NULL: copy, padding with 0 (src/imagew-resize.c:399-410);
		// NEAREST: nearest source pixel (src/imagew-resize.c:377-393).
		wt->kind = RowKind::Copy;
		for(int o = 0; o < n_out; o++) {
			int s;
			if(d.family == IW_RESIZETYPE_NULL) s = o < n_in ? o : -1;
			else {
				double c = (0.5 + (double)o - offset) / (double)n_out;
				s = (int)floor(c * (double)n_in);
				if(s < 0) s = 0;
				if(s > n_in - 1) s = n_in - 1;
			}
			wt->src.push_back(s);
			wt->pos.push_back(s);
			wt->w.push_back(1.0);
			wt->off.push_back((int)wt->src.size());
		}
		wt->max_taps = 1;
		wt->wsum_abs_max = 1.0;
		return wt;
	}

	double blur = d.blur;
	if(blur < 0.0001) blur = 0.0001;
	if(blur > 10000.0) blur = 10000.0;
	double rf = (d.true_size < (double)n_in) ? ((double)n_in) / d.true_size : 1.0;
	rf *= blur;

	// The reference sizes its first allocation from this estimate; an
	// estimate above the allocation limit is an out-of-memory error there.
	double est = 2.0 * k.radius * rf * n_out;
	if(((size_t)(int)est + 32) * 16 > ctx->max_malloc) {
		iw_set_error(ctx, "Out of memory");
		return nullptr;
	}
	wt->src.reserve((size_t)est + 32);

	for(int o = 0; o < n_out; o++) {
		double center = (0.5 + (double)o - offset) / d.true_size;
		double p = center * (double)n_in - 0.5;
		int first = (int)ceil(p - k.radius * rf - 0.0001);
		int last = (int)floor(p + k.radius * rf + 0.0001);
		size_t start = wt->w.size();
		int count = 0;
		double sum = 0.0;
		for(int ip = first; ip <= last; ip++) {
			if(d.edge == IW_EDGE_POLICY_STANDARD && (ip < 0 || ip >= n_in)) continue;
			double x = (((double)ip) - p) / rf;
			double v = kernel_at(k, x < 0 ? -x : x);
			if(v == 0.0) continue;
			sum += v;
			count++;
			int s = ip;
			if(ip < 0 || ip > n_in - 1) {
				if(d.edge == IW_EDGE_POLICY_TRANSPARENT) s = -1;
				else s = ip < 0 ? 0 : n_in - 1;
			}
			wt->src.push_back(s);
			wt->pos.push_back(ip);
			wt->w.push_back(v);
		}
		if(count > 0)
			for(size_t i = start; i < wt->w.size(); i++) wt->w[i] = (sum != 0.0) ? wt->w[i] / sum : 0.0;
		wt->off.push_back((int)wt->w.size());
		int nt = (int)(wt->w.size() - start);
		if(nt > wt->max_taps) wt->max_taps = nt;
		double sa = 0, sn = 0;
		for(size_t i = start; i < wt->w.size(); i++) {
			sa += fabs(wt->w[i]);
			if(wt->w[i] < 0) sn -= wt->w[i];
		}
		if(sa > wt->wsum_abs_max) wt->wsum_abs_max = sa;
		if(sn > wt->wsum_neg_max) wt->wsum_neg_max = sn;
	}
	return wt;
}

}  // namespace iwg
