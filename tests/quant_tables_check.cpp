// Invariants of the quantisation tables the device decisions rely on, built
// by the library's own build_quant (linked from libimagew_gb300.so):
//   * the bracket edges U[1..P] are non-decreasing, so a search started
//     anywhere and stepped up while U[k+1] <= v, then down while U[k] > v,
//     ends in the bracket a binary search finds (the re-evaluation of the
//     fast form starts from a coarse start table);
//   * each bracket record holds exactly the table entries it restates
//     (edges, exactness threshold, the two codes and their reverse values),
//     and records exist for error diffusion and for every integer output of
//     at most 4096 levels.
// Prints "OK" and exits 0, else prints the first failure and exits 1.
#include "iwg_internal.h"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>

using iwg::Quant;

static long long bits(double d)
{
	long long b;
	std::memcpy(&b, &d, 8);
	return b;
}

// The count of U[1..P] <= v (the bracket of v), by binary search.
static int bracket_bisect(const Quant &q, double v)
{
	const double *U = q.U->data() + 1;
	int lo = 0, hi = q.P;
	while(lo < hi) {
		const int mid = (lo + hi) >> 1;
		if(U[mid] <= v) lo = mid + 1; else hi = mid;
	}
	return lo;
}

// The same by stepping from a start k (any value in [0, P]).
static int bracket_step(const Quant &q, double v, int k)
{
	const double *U = q.U->data();
	while(k < q.P && U[k + 1] <= v) k++;
	while(k > 0 && U[k] > v) k--;
	return k;
}

static int fail(const char *what, const Quant &q, int k)
{
	std::printf("FAIL %s: cstype %d gamma %g maxcc %d cc %d dfam %d, bracket %d\n", what, q.cstype, q.gamma, q.maxcc,
		q.cc, q.dfam, k);
	return 1;
}

static int check(int cstype, double gamma, int maxcc, int cc, int dfam, std::mt19937_64 &rng)
{
	Quant q;
	q.cstype = cstype;
	q.gamma = gamma;
	q.maxcc = maxcc;
	q.cc = cc;
	q.dfam = dfam;
	iwg::build_quant(q);
	const int P = q.P;
	if(!q.U || (int)q.U->size() != P + 2 || !q.X || (int)q.X->size() != P + 1 || !q.code || !q.rev) return fail("table sizes", q, -1);
	const std::vector<double> &U = *q.U;
	for(int k = 1; k < P; k++)
		if(!(U[k] <= U[k + 1])) return fail("edges decrease", q, k);
	for(int k = 1; k <= P; k++)
		if(!(U[k] >= 0.0) || std::signbit(U[k])) return fail("negative edge", q, k);
	const bool want_rec = dfam == IW_DITHERFAMILY_ERRDIFF || maxcc <= 4095;
	if(want_rec != (bool)q.rec) return fail("records present", q, -1);
	if(q.rec) {
		if((int)q.rec->size() != 8 * (P + 1)) return fail("record count", q, -1);
		for(int k = 0; k <= P; k++) {
			const long long *r = q.rec->data() + 8 * (size_t)k;
			const int clo = (*q.code)[k], chi = (*q.code)[k + 1];
			if(r[0] != bits(U[k]) || r[1] != bits(U[k + 1]) || r[2] != bits((*q.X)[k])) return fail("record edges", q, k);
			if(r[4] != bits((*q.rev)[clo]) || r[5] != bits((*q.rev)[chi])) return fail("record reverse values", q, k);
			const unsigned long long c = (unsigned long long)r[6];
			if((int)(unsigned int)(c & 0xffffffffu) != clo || (int)(unsigned int)(c >> 32) != chi) return fail("record codes", q, k);
		}
	}
	// stepping from any start finds the binary search's bracket: random
	// values, every edge and its neighbours
	std::uniform_real_distribution<double> uni(0.0, 1.0);
	std::uniform_int_distribution<int> start(0, P);
	auto probe = [&](double v) -> int {
		if(!(v >= 0.0 && v <= 1.0)) return 0;
		const int want = bracket_bisect(q, v);
		for(int k0 : {0, P, start(rng), want})
			if(bracket_step(q, v, k0) != want) return fail("stepped search", q, k0);
		return 0;
	};
	for(int t = 0; t < 2000; t++)
		if(probe(uni(rng))) return 1;
	const int step = P > 4096 ? 17 : 1;   // every edge, or a spread of 16-bit edges
	for(int k = 1; k <= P; k += step)
		for(double v : {U[k], std::nextafter(U[k], -1.0), std::nextafter(U[k], 2.0)})
			if(probe(v)) return 1;
	return 0;
}

int main()
{
	std::mt19937_64 rng(12345);
	const int maxccs[] = {1, 3, 15, 255, 1023, 4095, 65535};
	const int dfams[] = {IW_DITHERFAMILY_NONE, IW_DITHERFAMILY_ORDERED, IW_DITHERFAMILY_ERRDIFF};
	struct Cs { int type; double gamma; };
	const Cs css[] = {{IW_CSTYPE_SRGB, 0.0}, {IW_CSTYPE_LINEAR, 0.0}, {IW_CSTYPE_GAMMA, 2.2}, {IW_CSTYPE_GAMMA, 0.45},
		{IW_CSTYPE_REC709, 0.0}};
	int n = 0;
	for(const Cs &cs : css)
		for(int maxcc : maxccs)
			for(int dfam : dfams)
				for(int cc : {0, 2, 17}) {
					if(cc > maxcc + 1 || (cc && maxcc > 255)) continue;
					// 16-bit error-diffusion records take seconds to build (a
					// bisection per bracket); the 16-bit edges are checked
					// without them
					if(maxcc > 4095 && dfam == IW_DITHERFAMILY_ERRDIFF) continue;
					if(check(cs.type, cs.gamma, maxcc, cc, dfam, rng)) return 1;
					n++;
				}
	std::printf("OK %d table sets\n", n);
	return 0;
}
