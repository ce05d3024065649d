// tables.cpp -- host-built tables that stand in for every transcendental
// function evaluation of the reference's pixel path.
//
// The reference calls pow() per sample when it converts a sample to linear
// light (src/imagew-main.c:28-66) and when it quantises a linear sample
// (get_nearest_valid_colors, src/imagew-main.c:570-629).  A GPU pow() is not
// glibc's, so the library never evaluates these on the device.  Instead:
//
//  * input tables map every integer code of an input channel to its exact
//    double linear value (the reference's own values, computed with host pow);
//  * quantisation tables give, for one output channel, the exact double
//    thresholds at which floor(from_linear(v) * P) steps (U) and at which the
//    product stops being an integer (X), the output code of each bracket, and
//    the linear value of each output code (rev).  With them the device decides
//    every output code with comparisons and IEEE add/sub/div only, which the
//    GPU performs exactly like the host.
//
// Tables depend only on (transfer function, max code, colour count), so they
// are cached process-wide.
#include "iwg_internal.h"

#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>
#include <tuple>

namespace iwg {

namespace {

std::mutex g_cache_mu;

uint64_t dbits(double v)
{
	uint64_t u;
	memcpy(&u, &v, 8);
	return u;
}

double bitsd(uint64_t u)
{
	double v;
	memcpy(&v, &u, 8);
	return v;
}

struct CsKey {
	int cstype;
	uint64_t gamma;
	bool operator<(const CsKey &o) const { return std::tie(cstype, gamma) < std::tie(o.cstype, o.gamma); }
};

}  // namespace

// Linear value of every code 0..ncodes-1 of an input channel with max code
// 'maxcc' (src/imagew-main.c:257-327: v/maxcc, then the transfer function).
std::shared_ptr<const std::vector<double>> input_table(int cstype, double gamma, int maxcc, int ncodes, bool linear)
{
	static std::map<std::tuple<int, uint64_t, int, int>, std::shared_ptr<const std::vector<double>>> cache;
	if(linear) { cstype = IW_CSTYPE_LINEAR; gamma = 0.0; }
	auto key = std::make_tuple(cstype, dbits(gamma), maxcc, ncodes);
	std::lock_guard<std::mutex> lk(g_cache_mu);
	auto it = cache.find(key);
	if(it != cache.end()) return it->second;
	struct iw_csdescr cs{};
	cs.cstype = cstype;
	cs.gamma = gamma;
	auto t = std::make_shared<std::vector<double>>(ncodes);
	double m = (double)maxcc;
	for(int v = 0; v < ncodes; v++) (*t)[v] = to_linear(((double)v) / m, cs);
	cache[key] = t;
	return t;
}

namespace {

// g(v): the reference's floor argument, clamped (src/imagew-main.c:577-611).
struct GFun {
	struct iw_csdescr cs{};
	double P = 255.0;
	double operator()(double v) const
	{
		double e = from_linear(v, cs) * P;
		if(e > P) e = P;
		if(e < 0.0) e = 0.0;
		return e;
	}
};

// Smallest double v in [0, 1] with pred(v) true, for a predicate that is
// false below some point and true from it on.  'guess' seeds the search.
template<class Pred>
double lowest_true(const Pred &pred, double guess)
{
	const uint64_t lo_lim = 0, hi_lim = dbits(1.0);
	if(!(guess >= 0.0)) guess = 0.0;
	if(guess > 1.0) guess = 1.0;
	uint64_t g = dbits(guess), lo, hi;   // invariant: pred(lo)==false, pred(hi)==true
	if(pred(bitsd(g))) {
		hi = g;
		uint64_t step = 1;
		for(;;) {
			if(hi - lo_lim <= step) { lo = lo_lim; if(pred(bitsd(lo))) return bitsd(lo); break; }
			uint64_t c = hi - step;
			if(!pred(bitsd(c))) { lo = c; break; }
			hi = c;
			step *= 2;
		}
	}
	else {
		lo = g;
		uint64_t step = 1;
		for(;;) {
			if(hi_lim - lo <= step) { hi = hi_lim; if(!pred(bitsd(hi))) return std::numeric_limits<double>::infinity(); break; }
			uint64_t c = lo + step;
			if(pred(bitsd(c))) { hi = c; break; }
			lo = c;
			step *= 2;
		}
	}
	while(hi - lo > 1) {
		uint64_t mid = lo + (hi - lo) / 2;
		if(pred(bitsd(mid))) hi = mid; else lo = mid;
	}
	return bitsd(hi);
}

struct QuantTables {
	std::shared_ptr<const std::vector<double>> U, X, rev, nc;
	std::shared_ptr<const std::vector<int>> code;
};

}  // namespace

void quant_fill(int cstype, double gamma, int maxcc, int cc, double *U, double *X, int *code, double *rev)
{
	struct iw_csdescr cs{};
	cs.cstype = cstype;
	cs.gamma = gamma;
	const int P = cc ? cc - 1 : maxcc, M = maxcc;
	GFun g;
	g.cs = cs;
	g.P = (double)P;
	const double inf = std::numeric_limits<double>::infinity();
	U[0] = -inf;
	U[P + 1] = inf;
	for(int k = 1; k <= P; k++) {
		double guess = to_linear((double)k / P, cs);
		U[k] = lowest_true([&](double v) { return g(v) >= (double)k; }, guess);
	}
	for(int k = 0; k < P; k++) {
		double guess = U[k + 1];
		if(k > 0 && guess < U[k]) guess = U[k];
		X[k] = lowest_true([&](double v) { return g(v) > (double)k; }, guess);
	}
	X[P] = inf;
	// bracket -> code: posterised codes are floor(0.5000000001 + k*(M/P))
	for(int k = 0; k <= P; k++) {
		if(cc) code[k] = (int)(unsigned int)floor(0.5000000001 + (double)k * ((double)M / (double)P));
		else code[k] = k;
	}
	code[P + 1] = code[P];
	for(int c = 0; c <= M; c++) rev[c] = to_linear(((double)c) / (double)M, cs);
}

// midpoints between adjacent 8-bit codes in linear light (src/imagew-main.c:1197-1236)
void nc_fill(int cstype, double gamma, double *nc)
{
	struct iw_csdescr cs{};
	cs.cstype = cstype;
	cs.gamma = gamma;
	double prev = 0.0;
	for(int i = 0; i < 255; i++) {
		double cur = to_linear(((double)(i + 1)) / 255, cs);
		nc[i] = (prev + cur) / 2.0;
		prev = cur;
	}
}

// Decision records of a bracket (src/imagew-main.c:727-748; error diffusion
// and the exact re-evaluation of the fast form read them): in
// bracket k a sample v below X[k] is exact (no error sent); above it the
// reference compares d_ceil = rev_hi - v with d_floor = v - rev_lo, each
// rounded.  The first is non-increasing in v and the second non-decreasing,
// so "d_ceil <= d_floor" holds from a least v on: C[k], found by bisection on
// the bit patterns.  The sent error is then v - rev[code] either way
// (-(rev_hi - v) rounds to the same value as v - rev_hi).
void rec_fill(int P, const double *U, const double *X, const int *code, const double *rev, long long *rec)
{
	for(int k = 0; k <= P; k++) {
		const double rl = rev[code[k]], rh = rev[code[k + 1]];
		double c = std::numeric_limits<double>::infinity();
		if(k < P) c = lowest_true([&](double v) { return rh - v <= v - rl; }, 0.5 * (rl + rh));
		long long *r = rec + 8 * (size_t)k;
		r[0] = (long long)dbits(U[k]);
		r[1] = (long long)dbits(U[k + 1]);
		r[2] = (long long)dbits(X[k]);
		r[3] = (long long)dbits(c);
		r[4] = (long long)dbits(rl);
		r[5] = (long long)dbits(rh);
		r[6] = (long long)(((unsigned long long)(unsigned int)code[k + 1] << 32) | (unsigned int)code[k]);
		r[7] = 0;
	}
}

void build_quant(Quant &q)
{
	static std::map<std::tuple<int, uint64_t, int, int>, std::shared_ptr<const std::vector<long long>>> rec_cache;
	static std::map<std::tuple<int, uint64_t, int, int>, QuantTables> cache;
	static std::map<std::tuple<int, uint64_t>, std::shared_ptr<const std::vector<double>>> nc_cache;

	q.P = q.cc ? q.cc - 1 : q.maxcc;
	auto key = std::make_tuple(q.cstype, dbits(q.gamma), q.maxcc, q.cc);
	std::lock_guard<std::mutex> lk(g_cache_mu);
	auto it = cache.find(key);
	if(it == cache.end()) {
		auto U = std::make_shared<std::vector<double>>(q.P + 2);
		auto X = std::make_shared<std::vector<double>>(q.P + 1);
		auto code = std::make_shared<std::vector<int>>(q.P + 2);
		auto rev = std::make_shared<std::vector<double>>(q.maxcc + 1);
		quant_fill(q.cstype, q.gamma, q.maxcc, q.cc, U->data(), X->data(), code->data(), rev->data());
		QuantTables t;
		t.U = U; t.X = X; t.code = code; t.rev = rev;
		it = cache.emplace(key, t).first;
	}
	q.U = it->second.U;
	q.X = it->second.X;
	q.code = it->second.code;
	q.rev = it->second.rev;
	// records for error diffusion, and for the outputs the fast form takes
	// (at most 4096 levels), whose re-evaluation reads one record per decision
	if(q.dfam == IW_DITHERFAMILY_ERRDIFF || (!q.float_out && q.maxcc <= 4095)) {
		auto rit = rec_cache.find(key);
		if(rit == rec_cache.end()) {
			auto rec = std::make_shared<std::vector<long long>>(8 * (size_t)(q.P + 1));
			rec_fill(q.P, q.U->data(), q.X->data(), q.code->data(), q.rev->data(), rec->data());
			rit = rec_cache.emplace(key, rec).first;
		}
		q.rec = rit->second;
	}
	if(q.use_nc) {
		auto nkey = std::make_tuple(q.cstype, dbits(q.gamma));
		auto nit = nc_cache.find(nkey);
		if(nit == nc_cache.end()) {
			auto nc = std::make_shared<std::vector<double>>(255);
			nc_fill(q.cstype, q.gamma, nc->data());
			nit = nc_cache.emplace(nkey, nc).first;
		}
		q.nc = nit->second;
	}
}

}  // namespace iwg
