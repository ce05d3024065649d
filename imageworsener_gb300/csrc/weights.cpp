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
#include <map>
#include <mutex>
#include <tuple>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

namespace iwg {

bool Weights::same_as(const Weights &o) const
{
	if(this == &o) return true;   // the same memoized list
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

namespace {

// Filter parameters of one dimension (src/imagew-resize.c:412-556).
struct DimSetup {
	Kernel k;
	bool standard = true;
	double offset = 0.0;
	double rf = 1.0;
	double edge_value = 0.0;
	int max_window = 1;   // upper bound on the taps of one output
};

// Returns false for an unknown filter family.
bool setup_dim(const DimRequest &d, int ctype, int n_in, int n_out, double edge_bkgd_value, DimSetup &S)
{
	Kernel &k = S.k;
	k.family = d.family;
	bool boxhack = false, sincfam = false;
	switch(d.family) {
	case IW_RESIZETYPE_NULL: S.standard = false; break;
	case IW_RESIZETYPE_NEAREST: S.standard = false; boxhack = true; break;
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
		return false;
	}
	if(sincfam) {   // "lobes", clamped to [2,100]
		k.radius = floor(d.p1 + 0.5);
		if(k.radius < 2.0) k.radius = 2.0;
		if(k.radius > 100.0) k.radius = 100.0;
	}
	S.edge_value = d.edge == IW_EDGE_POLICY_TRANSPARENT ? edge_bkgd_value : 0.0;
	S.offset = d.translate;
	if(boxhack) S.offset -= 0.00000000001;   // keep pixel centres off box borders
	if(d.use_offset && ctype >= 0 && ctype <= 2) S.offset += d.chan_offset[ctype];
	if(S.standard) {
		double blur = d.blur;
		if(blur < 0.0001) blur = 0.0001;
		if(blur > 10000.0) blur = 10000.0;
		S.rf = (d.true_size < (double)n_in) ? ((double)n_in) / d.true_size : 1.0;
		S.rf *= blur;
		S.max_window = (int)floor(2.0 * k.radius * S.rf + 0.0002) + 2;
	}
	return true;
}

}  // namespace

int weights_into(const DimRequest &d, int ctype, int n_in, int n_out, double edge_bkgd_value,
	int *off, int *src, double *w, int *pos, int cap, int *kind, double *edge_value)
{
	DimSetup S;
	if(!setup_dim(d, ctype, n_in, n_out, edge_bkgd_value, S)) return -2;
	*edge_value = S.edge_value;
	off[0] = 0;
	int n = 0;
	if(!S.standard) {
		// NULL: copy, padding with 0 (src/imagew-resize.c:399-410);
		// NEAREST: nearest source pixel (src/imagew-resize.c:377-393).
		*kind = (int)RowKind::Copy;
		if(cap < n_out) return -1;
		for(int o = 0; o < n_out; o++) {
			int s;
			if(d.family == IW_RESIZETYPE_NULL) s = o < n_in ? o : -1;
			else {
				double c = (0.5 + (double)o - S.offset) / (double)n_out;
				s = (int)floor(c * (double)n_in);
				if(s < 0) s = 0;
				if(s > n_in - 1) s = n_in - 1;
			}
			src[n] = s;
			if(pos) pos[n] = s;
			w[n] = 1.0;
			n++;
			off[o + 1] = n;
		}
		return n;
	}
	*kind = (int)RowKind::Sum;
	const Kernel &k = S.k;
	for(int o = 0; o < n_out; o++) {
		double center = (0.5 + (double)o - S.offset) / d.true_size;
		double p = center * (double)n_in - 0.5;
		int first = (int)ceil(p - k.radius * S.rf - 0.0001);
		int last = (int)floor(p + k.radius * S.rf + 0.0001);
		int start = n, count = 0;
		double sum = 0.0;
		for(int ip = first; ip <= last; ip++) {
			if(d.edge == IW_EDGE_POLICY_STANDARD && (ip < 0 || ip >= n_in)) continue;
			double x = (((double)ip) - p) / S.rf;
			double v = kernel_at(k, x < 0 ? -x : x);
			if(v == 0.0) continue;
			sum += v;
			count++;
			int s = ip;
			if(ip < 0 || ip > n_in - 1) {
				if(d.edge == IW_EDGE_POLICY_TRANSPARENT) s = -1;
				else s = ip < 0 ? 0 : n_in - 1;
			}
			if(n >= cap) return -1;
			src[n] = s;
			if(pos) pos[n] = ip;
			w[n] = v;
			n++;
		}
		if(count > 0)
			for(int i = start; i < n; i++) w[i] = (sum != 0.0) ? w[i] / sum : 0.0;
		off[o + 1] = n;
	}
	return n;
}

int weights_max_taps(const DimRequest &d, int n_in, int n_out)
{
	DimSetup S;
	if(!setup_dim(d, 0, n_in, n_out, 0.0, S)) return -1;
	return S.standard ? S.max_window : 1;
}

std::shared_ptr<const Weights> build_weights(iw_context *ctx, const DimRequest &d, int ctype,
	int n_in, int n_out, double edge_bkgd_value)
{
	DimSetup S;
	if(!setup_dim(d, ctype, n_in, n_out, edge_bkgd_value, S)) {
		iw_set_error(ctx, "Internal: Unknown resize algorithm");
		return nullptr;
	}
	if(S.standard) {
		// The reference sizes its first allocation from this estimate; an
		// estimate above the allocation limit is an out-of-memory error there.
		double est = 2.0 * S.k.radius * S.rf * n_out;
		if(((size_t)(int)est + 32) * 16 > ctx->max_malloc) {
			iw_set_error(ctx, "Out of memory");
			return nullptr;
		}
	}
	// Weight lists depend only on the settings setup_dim reads and the sizes:
	// built once per process for each distinct set (a plan asks for one per
	// intermediate channel and dimension, and a server or a batch sees the
	// same geometries again and again).  Bounded: cleared past kMemoMax.
	auto bits = [](double v) { uint64_t b; memcpy(&b, &v, sizeof b); return b; };
	const double eff_offset = S.offset;
	const double eff_edge = S.edge_value;
	using Key = std::tuple<int, int, uint64_t, uint64_t, uint64_t, uint64_t, uint64_t, uint64_t, int, int>;
	const Key key{d.family, d.edge, bits(d.blur), bits(d.p1), bits(d.p2), bits(d.true_size), bits(eff_offset),
		bits(eff_edge), n_in, n_out};
	static std::mutex memo_mu;
	static std::map<Key, std::shared_ptr<const Weights>> *memo = new std::map<Key, std::shared_ptr<const Weights>>();
	constexpr size_t kMemoMax = 1024;
	{
		std::lock_guard<std::mutex> lk(memo_mu);
		auto it = memo->find(key);
		if(it != memo->end()) return it->second;
	}
	auto wt = std::make_shared<Weights>();
	wt->n_in = n_in;
	wt->n_out = n_out;
	size_t cap = (size_t)n_out * (size_t)S.max_window;
	wt->off.resize(n_out + 1);
	wt->src.resize(cap);
	wt->w.resize(cap);
	wt->pos.resize(cap);
	int kind = 0;
	int n = weights_into(d, ctype, n_in, n_out, edge_bkgd_value, wt->off.data(), wt->src.data(), wt->w.data(),
		wt->pos.data(), (int)cap, &kind, &wt->edge_value);
	if(n < 0) {
		iw_set_error(ctx, "Internal: weight list overflow");
		return nullptr;
	}
	wt->kind = (RowKind)kind;
	wt->src.resize(n);
	wt->w.resize(n);
	wt->pos.resize(n);
	for(int o = 0; o < n_out; o++) {
		int nt = wt->off[o + 1] - wt->off[o];
		if(nt > wt->max_taps) wt->max_taps = nt;
		double sa = 0, sn = 0;
		for(int t = wt->off[o]; t < wt->off[o + 1]; t++) {
			sa += fabs(wt->w[t]);
			if(wt->w[t] < 0) sn -= wt->w[t];
		}
		if(sa > wt->wsum_abs_max) wt->wsum_abs_max = sa;
		if(sn > wt->wsum_neg_max) wt->wsum_neg_max = sn;
	}
	{
		std::lock_guard<std::mutex> lk(memo_mu);
		if(memo->size() >= kMemoMax) memo->clear();
		(*memo)[key] = wt;
	}
	return wt;
}

}  // namespace iwg
