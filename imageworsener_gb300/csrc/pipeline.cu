// pipeline.cu -- the GPU pixel pipeline of iw_process_image().
//
// Two forms compute the same bytes:
//   * plain  (FP64): the reference's arithmetic sample for sample -- a
//     vertical pass into a float intermediate (src/imagew-main.c:831-927), a
//     horizontal pass fused with the quantisation tail
//     (src/imagew-main.c:929-1155), and a serial scan for error-diffusion and
//     random dither, whose order the reference fixes;
//   * fast  (FP32 + guard band, fastpath.cu): FP32 resampling with a
//     rigorous per-sample error bound; samples whose error interval touches a
//     quantisation decision are recomputed here in FP64.  Integer output is
//     identical to the plain form's.
// Host code here packs the plan into a device Job, manages device memory and
// launches the kernels on the library's stream.
#include "iwg_internal.h"
#include "device.cuh"
#include "fastpath.cuh"
#include "imagew_gb300.h"

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <functional>
#include <thread>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

namespace iwg {

using namespace dev;

// ===========================================================================
// Plain-form kernels
// ===========================================================================

// Vertical pass: one thread per (column x, intermediate row j), all channels.
__device__ __forceinline__ void vpass_exact_at(const Job &J, int x, int j)
{
	if(x >= J.mid_w || j >= J.mid_h) return;
	for(int m = 0; m < J.mid_n; m++) {
		const DMid &mc = J.mid[m];
		const DWeights &W = J.wv[mc.wv];
		double s = 0.0;
		if(W.kind == 1) {
			int src = W.src[j];
			s = src < 0 ? 0.0 : decode_exact(J, mc, x, src);
		}
		else {
			for(int t = W.off[j]; t < W.off[j + 1]; t++) {
				int src = W.src[t];
				double v = src >= 0 ? decode_exact(J, mc, x, src) : W.edge_value;
				s = dadd(s, dmul(v, W.w[t]));
			}
		}
		if(J.intclamp) s = s < 0.0 ? 0.0 : (s > 1.0 ? 1.0 : s);
		J.interm[(unsigned long long)m * J.interm_plane + (unsigned long long)j * J.mid_w + x] = __double2float_rn(s);
	}
}

__global__ void k_vpass_exact(Job J)
{
	vpass_exact_at(J, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y);
}

// Exact intermediate value of channel m at (column x, row j): read from the
// plain form's vertical pass, or recomputed (the fast form keeps FP32 values
// in its intermediate buffer).
template<bool RECOMPUTE>
__device__ __forceinline__ double interm_exact(const Job &J, int m, int x, int j)
{
	if(!RECOMPUTE) return (double)J.interm[(unsigned long long)m * J.interm_plane + (unsigned long long)j * J.mid_w + x];
	const DMid &mc = J.mid[m];
	const DWeights &W = J.wv[mc.wv];
	double s = 0.0;
	if(W.kind == 1) {
		int src = W.src[j];
		s = src < 0 ? 0.0 : decode_exact(J, mc, x, src);
	}
	else {
		for(int t = W.off[j]; t < W.off[j + 1]; t++) {
			int src = W.src[t];
			double v = src >= 0 ? decode_exact(J, mc, x, src) : W.edge_value;
			s = dadd(s, dmul(v, W.w[t]));
		}
	}
	if(J.intclamp) s = s < 0.0 ? 0.0 : (s > 1.0 ? 1.0 : s);
	return (double)__double2float_rn(s);
}

// interm_exact<true> with its loads issued ahead: eight taps' samples (and
// alphas), then their decode-table values, in flight together; the FP64
// operations are interm_exact's, in its order, so the value is the same.
// For the re-evaluation of the fast form, whose plans have no grayscale
// conversion, early background, float input or orientation change (others
// take interm_exact itself).
__device__ double interm_exact_ahead(const Job &J, int m, int x, int j)
{
	const DMid &mc = J.mid[m];
	const DWeights &W = J.wv[mc.wv];
	if(mc.to_gray || J.bk_early || J.in_float || J.orient != 0 || W.kind == 1) return interm_exact<true>(J, m, x, j);
	const int tb = W.off[j], te = W.off[j + 1];
	const int px = J.crop_x + x;
	const bool has_ch = mc.in_ch < J.in_nphys, has_a = J.in_alpha < J.in_nphys;
	double s = 0.0;
	for(int t0 = tb; t0 < te; t0 += 8) {
		int src[8];
#pragma unroll
		for(int u = 0; u < 8; u++) src[u] = t0 + u < te ? W.src[t0 + u] : -1;
		unsigned int cv[8], ca[8];
#pragma unroll
		for(int u = 0; u < 8; u++) {
			cv[u] = ca[u] = 0u;
			if(src[u] < 0) continue;
			const int py = J.crop_y + src[u];
			if(has_ch) cv[u] = raw_code(J, px, py, mc.in_ch);
			if(mc.unassoc && has_a) ca[u] = raw_code(J, px, py, J.in_alpha);
		}
		double v[8], a[8], w[8];
#pragma unroll
		for(int u = 0; u < 8; u++) {
			v[u] = has_ch ? mc.tab[0][cv[u]] : 1.0;               // in_value (virtual channel: 1)
			a[u] = (mc.unassoc && has_a) ? J.alpha_tab[ca[u]] : 1.0;
			w[u] = t0 + u < te ? W.w[t0 + u] : 0.0;
		}
#pragma unroll
		for(int u = 0; u < 8; u++) {
			if(t0 + u >= te) break;
			double d = W.edge_value;
			if(src[u] >= 0) {
				d = v[u];
				if(mc.unassoc) d = dmul(d, a[u]);   // decode_exact
			}
			s = dadd(s, dmul(d, w[u]));
		}
	}
	if(J.intclamp) s = s < 0.0 ? 0.0 : (s > 1.0 ? 1.0 : s);
	return (double)__double2float_rn(s);
}

// Horizontal pass of one channel for output pixel (i, j).  interm(m, k, x)
// returns the exact intermediate value of channel m at column x, the k-th tap.
template<class Interm>
__device__ __forceinline__ double hsum_exact(const Job &J, int m, int i, int j, Interm interm)
{
	const DWeights &W = J.wh[J.mid[m].wh];
	double s = 0.0;
	const int t0 = W.off[i];
	if(W.kind == 1) {
		int src = W.src[i];
		s = src < 0 ? 0.0 : interm(m, 0, src);
	}
	else {
		for(int t = t0; t < W.off[i + 1]; t++) {
			int src = W.src[t];
			double v = src >= 0 ? interm(m, t - t0, src) : W.edge_value;
			s = dadd(s, dmul(v, W.w[t]));
		}
	}
	if(J.intclamp) s = s < 0.0 ? 0.0 : (s > 1.0 ? 1.0 : s);
	return s;
}

// Unassociate alpha and composite a late background
// (src/imagew-main.c:1079-1115).  'a' is the float-rounded resampled alpha.
__device__ __forceinline__ double unassoc_and_bkgd(const Job &J, const DMid &mc, const DOut &oc, double v,
	double a, int alt, bool is_alpha)
{
	double bka = J.bk_trns ? (alt ? J.bk2_alpha : J.bk1_alpha) : 0.0;
	if(mc.unassoc) {
		if(a != 0.0) v = ddiv(v, a);
		if(J.bk_late) {
			double bc = alt ? oc.bk2 : oc.bk1;
			if(J.bk_trns) v = dadd(dmul(v, a), dmul(dmul(bc, bka), dsub(1.0, a)));
			else v = dadd(dmul(v, a), dmul(bc, dsub(1.0, a)));
		}
	}
	else if(is_alpha && J.bk_trns) {
		v = dadd(v, dmul(bka, dsub(1.0, v)));
	}
	return v;
}

// Quantise / store every channel of output pixel (i, j) exactly.  Used by the
// plain form for all pixels and by the fast form for flagged pixels.
// 'mask' selects the intermediate channels to evaluate (bit m); the alpha
// channel must be included whenever a colour channel is.
// Output codes of one pixel, kept in registers (an array indexed by a run-time
// channel would live in local memory, and a kernel that needs local memory
// can make the driver wait for the whole device when it launches).
struct Codes4 {
	int c0 = -1, c1 = -1, c2 = -1, c3 = -1;
	__device__ __forceinline__ void set(int k, int v)
	{
		if(k == 0) c0 = v;
		else if(k == 1) c1 = v;
		else if(k == 2) c2 = v;
		else c3 = v;
	}
	__device__ __forceinline__ int operator[](int k) const { return k == 0 ? c0 : (k == 1 ? c1 : (k == 2 ? c2 : c3)); }
};
static_assert(dev::kMaxCh == 4, "Codes4 holds four channels");

template<class Interm>
__device__ void pixel_exact(const Job &J, int i, int j, bool apply_post, Interm interm, unsigned int mask = 0xfu)
{
	double a = 0.0;
	int alpha_code = -1;
	Codes4 codes;
	int alt = checker_alt(J, i, j);
	for(int k = 0; k < J.mid_n; k++) {
		int m = J.order[k];
		if(!((mask >> m) & 1u)) continue;
		const DMid &mc = J.mid[m];
		bool is_alpha = mc.ctype == IW_CHANNELTYPE_ALPHA;
		double s = hsum_exact(J, m, i, j, interm);
		if(is_alpha) a = (double)__double2float_rn(s);
		int oc = mc.out_ch;
		if(oc < 0) continue;
		const DOut &o = J.outc[oc];
		double v = unassoc_and_bkgd(J, mc, o, s, a, alt, is_alpha);
		if(J.dbg) J.dbg[((unsigned long long)oc * J.out_h + j) * J.out_w + i] = v;
		if(J.out_float) {
			float f = __double2float_rn(v);
			if(J.negate && !is_alpha) f = __fsub_rn(1.0f, f);
			store_float(J, oc, i, j, f);
			continue;
		}
		if(o.scan) {
			J.scanbuf[((unsigned long long)oc * J.out_h + j) * J.out_w + i] = v;
			codes.set(oc, -1);
			continue;
		}
		int c = quantize_exact(o.q, v, i, j);
		if(is_alpha) alpha_code = c;
		codes.set(oc, c);
	}
	if(J.out_float) return;
	for(int oc = 0; oc < J.out_n; oc++) {
		int c = codes[oc];
		if(c < 0) continue;
		if(apply_post) {
			bool is_alpha = J.outc[oc].ctype == IW_CHANNELTYPE_ALPHA;
			if(!is_alpha) {
				if(J.negate) c = J.outc[oc].maxcc - c;
				if(J.blacken && alpha_code == 0) c = 0;
			}
		}
		store_code(J, oc, i, j, (unsigned int)c);
	}
}

__device__ __forceinline__ void hpass_exact_at(const Job &J, int i, int j)
{
	if(i >= J.out_w || j >= J.out_h) return;
	pixel_exact(J, i, j, !J.any_scan, [&](int m, int, int x) { return interm_exact<false>(J, m, x, j); });
}

__global__ void k_hpass_exact(Job J)
{
	hpass_exact_at(J, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y);
}

// Serial scans for error-diffusion and random dither of one output channel
// (src/imagew-main.c:487-567, :1072-1136).  The reference visits samples in a
// fixed order and each decision depends on the previous ones.  Error
// diffusion runs serpentine: a right-to-left row starts where the row above
// ended, so it needs that whole row's errors and rows cannot overlap in a
// wavefront.  Channels are independent and run in separate warps.

// Bracket of v in [0, 1] with integer comparisons: for non-negative doubles
// the order of the bit patterns is the order of the values (the tables' -inf
// and +inf ends compare correctly as signed integers), which keeps the FP64
// pipe free for the arithmetic.
__device__ __forceinline__ Bracket bracket_bits(const DQuant &q, double v)
{
	const long long vb = __double_as_longlong(v);
	const long long *U = reinterpret_cast<const long long *>(q.U) + 1;
	int lo = 0, hi = q.P;
	while(lo < hi) {
		const int mid = (lo + hi) >> 1;
		if(__ldg(U + mid) <= vb) lo = mid + 1; else hi = mid;
	}
	Bracket b;
	const int k = lo;
	b.exact = (k == q.P) || (vb < __ldg(reinterpret_cast<const long long *>(q.X) + k));
	b.lo = q.code[k];
	b.hi = q.code[k + 1];
	b.d_lo = b.d_hi = 0.0;
	if(!b.exact) {
		b.d_lo = dsub(v, q.rev[b.lo]);
		b.d_hi = dsub(q.rev[b.hi], v);
	}
	return b;
}

// The twelve error-diffusion weights of subtype 'dsub': numerators over a
// denominator (positions x+1 x+2 / x-2 x-1 x x+1 x+2 / the same on the row
// after next), as separately rounded quotients like the reference's.
__constant__ signed char c_ed_num[8][12] = {
	{7,0, 0,3,5,1,0, 0,0,0,0,0}, {7,5, 3,5,7,5,3, 1,3,5,3,1}, {8,4, 2,4,8,4,2, 1,2,4,2,1},
	{8,4, 2,4,8,4,2, 0,0,0,0,0}, {5,3, 2,4,5,4,2, 0,2,3,2,0}, {4,3, 1,2,3,2,1, 0,0,0,0,0},
	{2,0, 0,1,1,0,0, 0,0,0,0,0}, {1,1, 0,1,1,1,0, 0,0,1,0,0}};
__constant__ double c_ed_den[8] = {16.0, 48.0, 42.0, 32.0, 32.0, 16.0, 4.0, 8.0};

__device__ __forceinline__ void errdiff_weights(int dsub, double *c)
{
	const int sub = (dsub >= 0 && dsub <= 7) ? dsub : 0;
#pragma unroll
	for(int k = 0; k < 12; k++) c[k] = ddiv((double)c_ed_num[sub][k], c_ed_den[sub]);
}

constexpr int kScanChunk = 256;   // samples staged per warp for the serial walk

// The reference's clamp to [0, 1] ("if(v<0) v=0; if(v>1) v=1"), by integer
// tests of the bit pattern (NaN passes through, as there); -0 becomes +0,
// which compares and adds like -0 everywhere downstream.
// a <= b for non-NaN doubles by integer comparison of order-preserving keys
// (negative values' magnitude bits are flipped).  -0 and +0 differ in key,
// but a difference of equal finite values is +0, so -0 does not occur where
// this is used.
__device__ __forceinline__ bool dle_bits(double a, double b)
{
	long long ka = __double_as_longlong(a), kb = __double_as_longlong(b);
	ka ^= (ka >> 63) & 0x7fffffffffffffffLL;
	kb ^= (kb >> 63) & 0x7fffffffffffffffLL;
	return ka <= kb;
}

__device__ __forceinline__ double clamp01_bits(double v)
{
	const long long b = __double_as_longlong(v);
	if((b & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL) return v;   // NaN
	if(b < 0) return 0.0;
	if(b > 0x3ff0000000000000LL) return 1.0;
	return v;
}

// Bracket index k (U[k] <= v < U[k+1]) of v in [+0, 1]: the count of
// U[1..P] <= v, from a start point in q.lut (stepped to the exact count in
// double; any start gives the same count), else by binary search.
__device__ __forceinline__ int bracket_index(const DQuant &q, long long vb)
{
	const long long *U = reinterpret_cast<const long long *>(q.U) + 1;
	if(q.lut) {
		const float vf = __double2float_rd(__longlong_as_double(vb));
		const int cell = min(max((int)__fmul_rn(vf, (float)kBracketLutCells), 0), kBracketLutCells - 1);
		int k = (int)__ldg(q.lut + cell);
		while(k < q.P && __ldg(U + k) <= vb) k++;
		while(k > 0 && __ldg(U + k - 1) > vb) k--;
		return k;
	}
	int lo = 0, hi = q.P;
	while(lo < hi) {
		const int mid = (lo + hi) >> 1;
		if(__ldg(U + mid) <= vb) lo = mid + 1; else hi = mid;
	}
	return lo;
}

// One bracket's decision record (the 8 words of DQuant::rec).
struct EdRec {
	long long lo, hi, x, c;   // bit patterns: U[k], U[k+1], X[k], C[k]
	double rev_lo, rev_hi;
	int code_lo, code_hi;
};

__device__ __forceinline__ EdRec ed_rec(const long long *rec, int k)
{
	const longlong2 *r = reinterpret_cast<const longlong2 *>(rec + 8 * (long long)k);
	const longlong2 a = __ldg(r), b = __ldg(r + 1), c = __ldg(r + 2), d = __ldg(r + 3);
	EdRec e;
	e.lo = a.x; e.hi = a.y; e.x = b.x; e.c = b.y;
	e.rev_lo = __longlong_as_double(c.x);
	e.rev_hi = __longlong_as_double(c.y);
	e.code_lo = (int)(unsigned int)(unsigned long long)d.x;
	e.code_hi = (int)(unsigned int)((unsigned long long)d.x >> 32);
	return e;
}

__device__ __forceinline__ bool is_nan_bits(double v)
{
	return (__double_as_longlong(v) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
}

// Error diffusion of one channel by one warp.  Per row:
//   1. all lanes clamp the row's values and find their brackets and the
//      brackets' bounds (the value before its error is added; the error moves
//      it by about one code);
//   2. lane 0 walks the samples in the reference's order doing only what
//      the next sample depends on -- the value plus its accumulated error
//      (the error carried from the previous rows plus the two in-row
//      contributions, kept in registers and added in the reference's order),
//      the decision, and the sample's error;
//   3. all lanes send the row's errors to the next two rows (e1, e2), each
//      lane owning target positions and adding the contributions in the order
//      the reference adds them (sample x-2f, x-f, x, x+f, x+2f); rows rotate.
// On GB300 every FP64 instruction holds the SM sub-partition's FP64 unit for
// tens of cycles whether one lane or 32 are active, and the walk is one
// dependent chain, so step 2 is kept short: four FP64 operations per sample
// for Floyd-Steinberg (the in-row product and sum, the value plus error, the
// sample's error) and a few integer ones -- the bracket from the staged
// bounds, one record load, two compares for the decision.  Products with a
// zero weight are skipped: they add a signed zero to an accumulator that
// starts at +0 and can never become -0 (a sum of nonzero values that cancels
// is +0), which leaves it unchanged.  For the same reason a sample that sends
// no error (an exact one) is given the error +0: its contributions change
// nothing, so the walk and the spreading need no test for it.
// Error buffer of a channel: three rotating error rows and the row's errors,
// out_w doubles each; the staged chunk lives in shared memory (kScanChunk).
template<bool C1>   // C1: the weight of sample x+2f in the same row is nonzero
__device__ __forceinline__ void errdiff_warp(const Job &J, int oc)
{
	__shared__ double s_v[dev::kMaxCh][kScanChunk], s_e[dev::kMaxCh][kScanChunk];
	__shared__ long long s_lo[dev::kMaxCh][kScanChunk], s_hi[dev::kMaxCh][kScanChunk];
	__shared__ int s_k[dev::kMaxCh][kScanChunk];
	double *const sv = s_v[oc], *const se = s_e[oc];
	long long *const slo = s_lo[oc], *const shi = s_hi[oc];
	int *const sk = s_k[oc];
	const int lane = threadIdx.x & 31;
	const DOut &o = J.outc[oc];
	const DQuant &q = o.q;
	const int W = J.out_w, H = J.out_h, P = q.P;
	const long long *const U = reinterpret_cast<const long long *>(q.U);
	const long long *const rec = q.rec;
	uint8_t *const out = J.out;
	const unsigned long long out_bpr = J.out_bpr;
	const int out_n = J.out_n, wide = J.out_depth == 8 ? 0 : 1;
	const double *const scan = J.scanbuf + (unsigned long long)oc * H * W;
	double *e0 = J.errbuf + (unsigned long long)oc * 5 * W, *e1 = e0 + W, *e2 = e1 + W;
	double *const er = e2 + W;
	double c[12];
	errdiff_weights(q.dsub, c);
	bool nz1[5], nz2[5];   // nonzero weights toward the next row / the row after, source offset k = -2..2
	bool any2 = false;
#pragma unroll
	for(int k = 0; k < 5; k++) {
		nz1[k] = c[6 - k] != 0.0;
		nz2[k] = c[11 - k] != 0.0;
		any2 = any2 || nz2[k];
	}
	const double c0 = c[0], c1 = c[1];
	for(int x = lane; x < 3 * W; x += 32) e0[x] = 0.0;
	__syncwarp();
	for(int y = 0; y < H; y++) {
		const int f = (y % 2) ? -1 : 1;
		const double *row = scan + (unsigned long long)y * W;
		uint8_t *const orow = out + (unsigned long long)y * out_bpr + ((size_t)oc << wide);
		double err1 = 0.0, err2 = 0.0;     // errors of the previous two samples of the row
		for(int z0 = 0; z0 < W; z0 += kScanChunk) {
			const int cn = min(kScanChunk, W - z0);
			const int xb = (y % 2) ? W - 1 - z0 : z0;   // x of the chunk's first sample
			// stage the chunk (in processing order): clamped value, carried
			// error, bracket (-1 for NaN) and the bracket's bounds
			{
				constexpr int kPer = kScanChunk / 32;
				double rv[kPer], re[kPer];
#pragma unroll
				for(int i = 0; i < kPer; i++) {   // all loads first: they overlap
					const int zz = lane + 32 * i;
					const int x = xb + zz * f;
					rv[i] = zz < cn ? row[x] : 0.0;
					re[i] = zz < cn ? e0[x] : 0.0;
				}
#pragma unroll
				for(int i = 0; i < kPer; i++) {
					const int zz = lane + 32 * i;
					if(zz >= cn) break;
					const double v = clamp01_bits(rv[i]);   // +0 for any negative value, NaN kept
					sv[zz] = v;
					se[zz] = re[i];
					const int k = is_nan_bits(v) ? -1 : bracket_index(q, __double_as_longlong(v));
					sk[zz] = k;
					slo[zz] = k < 0 ? 0 : __ldg(U + k);
					shi[zz] = k < 0 ? 0 : __ldg(U + k + 1);
				}
			}
			__syncwarp();
			if(lane == 0) {
				double s_n = sv[0], e_n = se[0];
				long long lo_n = slo[0], hi_n = shi[0];
				int k_n = sk[0];
				for(int zz = 0; zz < cn; zz++) {
					const int x = xb + zz * f;
					const double sval = s_n;
					double e = e_n;
					const long long lo0 = lo_n, hi0 = hi_n;
					const int k0 = k_n;
					if(zz + 1 < cn) {   // the next sample's staged values, ahead of the chain
						s_n = sv[zz + 1];
						e_n = se[zz + 1];
						lo_n = slo[zz + 1];
						hi_n = shi[zz + 1];
						k_n = sk[zz + 1];
					}
					// the records of the staged bracket and its neighbours, loaded
					// while the FP64 chain runs
					const int kc = k0 < 0 ? 0 : k0;
					const EdRec rm = ed_rec(rec, kc > 0 ? kc - 1 : 0), r0 = ed_rec(rec, kc),
						rp = ed_rec(rec, kc < P ? kc + 1 : P);
					// e0[x] as the reference has it when it reaches x: the carried
					// error, then x-2f's contribution, then x-f's
					if(C1) e = dadd(e, dmul(err2, c1));
					e = dadd(e, dmul(err1, c0));
					int code = 0;
					double err = 0.0;
					if(k0 >= 0) {
						// the reference's clamp; the value is not NaN here
						const double w = dadd(sval, e);
						const long long wb = __double_as_longlong(w);
						const double v = wb < 0 ? 0.0 : (wb > 0x3ff0000000000000LL ? 1.0 : w);
						const long long vb = __double_as_longlong(v);
						const bool below = vb < lo0, above = vb >= hi0;
						EdRec r = below ? rm : (above ? rp : r0);
						if((below && vb < rm.lo) || (above && vb >= rp.hi)) {   // moved more than one bracket
							int k = k0;
							while(k < P && __ldg(U + k + 1) <= vb) k++;
							while(k > 0 && __ldg(U + k) > vb) k--;
							r = ed_rec(rec, k);
						}
						code = r.code_lo;
						if(vb >= r.x) {   // not exact (X[P] is +inf)
							const bool up = vb >= r.c;
							code = up ? r.code_hi : r.code_lo;
							err = dsub(v, up ? r.rev_hi : r.rev_lo);
						}
					}
					er[x] = err;
					err2 = err1;
					err1 = err;
					uint8_t *const p = orow + ((size_t)x * out_n << wide);
					if(wide) {
						p[0] = (uint8_t)(code >> 8);
						p[1] = (uint8_t)(code & 0xff);
					}
					else p[0] = (uint8_t)code;
				}
			}
			__syncwarp();
		}
		for(int t = lane; t < W; t += 32) {
			double a1 = e1[t], a2 = e2[t];
#pragma unroll
			for(int k = -2; k <= 2; k++) {          // source sample t + k*f, in processing order
				if(!nz1[k + 2] && !nz2[k + 2]) continue;
				const int qx = t + k * f;
				if(qx < 0 || qx >= W) continue;
				const double err = er[qx];
				if(nz1[k + 2]) a1 = dadd(a1, dmul(err, c[4 - k]));
				if(nz2[k + 2]) a2 = dadd(a2, dmul(err, c[9 - k]));
			}
			e1[t] = a1;
			if(any2) e2[t] = a2;
			e0[t] = 0.0;   // becomes the row after next
		}
		__syncwarp();
		double *t0 = e0;
		e0 = e1;
		e1 = e2;
		e2 = t0;
	}
}

// Multiply-with-carry generator of the reference (src/imagew-util.c:202-233).
__device__ unsigned int prng_next(unsigned int &mult, unsigned int &carry)
{
	unsigned long long x = 0xfff0bf23ULL * mult + carry;
	carry = (unsigned int)(x >> 32);
	mult = 0xffffffffU - (unsigned int)(x & 0xffffffffULL);
	return mult;
}

// ---- random dither: the generator jumped ahead per row ----
//
// The generator's state (mult m, carry c) packs into w = a*m + c (a =
// 0xfff0bf23, c < a, m < 2^32), and one draw maps w to -a*w + a*(2^32-1)
// modulo the prime q = a*2^32 + 1 (a complementary multiply-with-carry is
// an affine map on w).  The state after n draws is that map composed n
// times, found by squaring, so each row of samples starts from its own state
// and rows run in parallel while every sample still gets the draw the
// reference gives it (one draw per sample in row-major order).
constexpr unsigned long long kMwcA = 0xfff0bf23ULL;
constexpr unsigned long long kMwcQ = 0xfff0bf2300000001ULL;   // a * 2^32 + 1
constexpr unsigned long long kMwcD = 0x000f40dcffffffffULL;   // 2^64 - q = 2^64 mod q

__device__ __forceinline__ unsigned long long mwc_mod(unsigned long long hi, unsigned long long lo)
{
	while(hi) {   // hi * 2^64 + lo == hi * D + lo (mod q); D < 2^52, so hi shrinks each round
		const unsigned long long ph = __umul64hi(hi, kMwcD), pl = hi * kMwcD;
		const unsigned long long nl = pl + lo;
		hi = ph + (nl < pl ? 1ULL : 0ULL);
		lo = nl;
	}
	return lo >= kMwcQ ? lo - kMwcQ : lo;
}

__device__ __forceinline__ unsigned long long mwc_mul(unsigned long long x, unsigned long long y)
{
	return mwc_mod(__umul64hi(x, y), x * y);
}

__device__ __forceinline__ unsigned long long mwc_add(unsigned long long x, unsigned long long y)
{
	const unsigned long long s = x + y;
	return mwc_mod(s < x ? 1ULL : 0ULL, s);
}

// Generator state after n draws from (mult, carry).
__device__ void mwc_jump(unsigned int &mult, unsigned int &carry, unsigned long long n)
{
	unsigned long long A = 1, B = 0;                                  // identity map
	unsigned long long pa = kMwcQ - kMwcA, pb = kMwcQ - 1 - kMwcA;    // one draw: w -> -a*w + a*(2^32-1)
	while(n) {
		if(n & 1) {
			B = mwc_add(mwc_mul(pa, B), pb);
			A = mwc_mul(pa, A);
		}
		pb = mwc_add(mwc_mul(pa, pb), pb);
		pa = mwc_mul(pa, pa);
		n >>= 1;
	}
	const unsigned long long w = mwc_add(mwc_mul(A, kMwcA * mult + carry), B);
	mult = (unsigned int)(w / kMwcA);
	carry = (unsigned int)(w % kMwcA);
}

// Random dither of one channel by one warp: lane l takes rows l, l+32, ...
__device__ void random_warp(const Job &J, int oc)
{
	const int lane = threadIdx.x & 31;
	const DOut &o = J.outc[oc];
	const DQuant &q = o.q;
	const int W = J.out_w;
	const int s = (q.dsub == IW_DITHERSUBTYPE_SAMEPATTERN && o.ctype != IW_CHANNELTYPE_ALPHA) ? J.seed : J.seed + o.ctype;
	for(int y = lane; y < J.out_h; y += 32) {
		unsigned int mult = 0x03333333U + (unsigned int)s, carry = 0x05555555U + (unsigned int)s;
		mwc_jump(mult, carry, (unsigned long long)y * W);
		const double *row = J.scanbuf + ((unsigned long long)oc * J.out_h + y) * W;
		for(int x = 0; x < W; x++) {
			double v = row[x];
			if(v < 0.0) v = 0.0;
			if(v > 1.0) v = 1.0;
			int code;
			if(v != v) {
				code = 0;
				(void)prng_next(mult, carry);
			}
			else {
				Bracket b = bracket_bits(q, dadd(v, 0.0));
				if(b.exact) {
					code = b.lo;
					(void)prng_next(mult, carry);   // one draw per sample
				}
				else {
					double fr = ddiv(b.d_lo, dadd(b.d_lo, b.d_hi));
					double thr = ddiv((double)prng_next(mult, carry), (double)0xffffffffU);
					code = fr >= thr ? b.hi : b.lo;
				}
			}
			store_code(J, oc, x, y, (unsigned int)code);
		}
	}
}

// One warp per output channel of the image (at most four warps per block).
__device__ __forceinline__ void scan_warp(const Job &J, int oc)
{
	if(oc >= J.out_n || oc >= dev::kMaxCh || !J.outc[oc].scan) return;
	if(J.outc[oc].q.dfam == IW_DITHERFAMILY_ERRDIFF) {
		const int sub = J.outc[oc].q.dsub;
		if(sub <= 0 || sub == 6 || sub > 7) errdiff_warp<false>(J, oc);   // Floyd-Steinberg, Sierra "4A": no x+2f weight
		else errdiff_warp<true>(J, oc);
	}
	else random_warp(J, oc);
}

__global__ void k_scan(Job J)
{
	scan_warp(J, threadIdx.x >> 5);
}

// Negation and blackening of fully transparent pixels, for outputs whose
// channels were (partly) quantised by the serial scan.
__device__ __forceinline__ void finalize_at(const Job &J, int i, int j)
{
	if(i >= J.out_w || j >= J.out_h) return;
	int alpha_oc = -1;
	for(int oc = 0; oc < J.out_n; oc++) if(J.outc[oc].ctype == IW_CHANNELTYPE_ALPHA) alpha_oc = oc;
	bool clear = J.blacken && alpha_oc >= 0 && load_code(J, alpha_oc, i, j) == 0;
	for(int oc = 0; oc < J.out_n; oc++) {
		if(oc == alpha_oc) continue;
		unsigned int c = load_code(J, oc, i, j);
		if(J.negate) c = (unsigned int)J.outc[oc].maxcc - c;
		if(clear) c = 0;
		store_code(J, oc, i, j, c);
	}
}

__global__ void k_finalize(Job J)
{
	finalize_at(J, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y);
}

// ---- the plain form for a batch: jobs in device memory, block -> image by a
// prefix table of per-image block counts ----

__device__ __forceinline__ int find_job(const int *start, int n, int b)
{
	int lo = 0, hi = n - 1;
	while(lo < hi) {
		const int mid = (lo + hi + 1) >> 1;
		if(__ldg(start + mid) <= b) lo = mid; else hi = mid - 1;
	}
	return lo;
}

// The batched plain passes walk their logical blocks with a block stride, so
// that a lane of long background work can run them on a capped grid and leave
// room on the SMs for other lanes.
__global__ void kb_vpass_exact(const Job *jobs, const int *start, int n, int total)
{
	for(int b = blockIdx.x; b < total; b += gridDim.x) {
		const int g = find_job(start, n, b);
		const Job &J = jobs[g];
		const int local = b - start[g], gx = (J.mid_w + blockDim.x - 1) / blockDim.x;
		vpass_exact_at(J, (local % gx) * blockDim.x + threadIdx.x, local / gx);
	}
}

__global__ void kb_hpass_exact(const Job *jobs, const int *start, int n, int total)
{
	for(int b = blockIdx.x; b < total; b += gridDim.x) {
		const int g = find_job(start, n, b);
		const Job &J = jobs[g];
		const int local = b - start[g], gx = (J.out_w + blockDim.x - 1) / blockDim.x;
		hpass_exact_at(J, (local % gx) * blockDim.x + threadIdx.x, local / gx);
	}
}

// One warp per output channel; a block takes images blockIdx.x,
// blockIdx.x + gridDim.x, ...  The grid is at most one block per SM: two scan
// warps on one SM sub-partition share its FP64 unit and each runs at about
// half speed, so a second image on the same SM would finish no sooner than if
// it waited its turn, and would delay the first.  With a completion flag the
// block also does the image's negation / blackening and then reports the
// image done, so the host can take its output before the rest of the batch
// ends (without one, kb_finalize follows for the whole batch).
__global__ void kb_scan(const Job *jobs, int n)
{
	for(int g = blockIdx.x; g < n; g += gridDim.x) {
		const Job &J = jobs[g];
		if(J.any_scan) scan_warp(J, threadIdx.x >> 5);
		__syncthreads();   // the shared staging buffers are reused by the next image
		if(J.done_flag) {
			if(J.any_scan && (J.negate || J.blacken)) {
				const long long npx = (long long)J.out_w * J.out_h;
				for(long long p = threadIdx.x; p < npx; p += blockDim.x) finalize_at(J, (int)(p % J.out_w), (int)(p / J.out_w));
			}
			__threadfence();   // every thread's output stores, device-wide, before the flag
			__syncthreads();
			if(threadIdx.x == 0) {
				__threadfence_system();
				*J.done_flag = 1;
			}
		}
	}
}

__global__ void kb_finalize(const Job *jobs, const int *start, int n, int total)
{
	for(int b = blockIdx.x; b < total; b += gridDim.x) {
		const int g = find_job(start, n, b);
		const Job &J = jobs[g];
		if(!J.any_scan || !(J.negate || J.blacken)) continue;
		const int local = b - start[g], gx = (J.out_w + blockDim.x - 1) / blockDim.x;
		finalize_at(J, (local % gx) * blockDim.x + threadIdx.x, local / gx);
	}
}

// Position of the r-th set bit of 'mask' (r counts from 0).
__device__ __forceinline__ int nth_bit(unsigned int mask, int r)
{
	for(int k = 0; k < r; k++) mask &= mask - 1u;
	return __ffs(mask) - 1;
}

// ---- double-float tier of the re-evaluation ----
//
// A flagged pixel is first re-evaluated in double-float arithmetic (48-bit,
// on the FP32 pipe) with a rigorous bound against the reference's FP64
// computation.  Every float32 intermediate the pixel reads is certified:
// the reference's sum S_ref lies within delta of the double-float sum, and
// if no float rounding boundary lies in that interval, fl32(S_ref) is the
// float nearest the double-float value, exactly.  The horizontal sum,
// the float alpha and the division get the same treatment, and the output
// code is taken only if it is the same over the whole remaining interval
// (with a margin for the rounding of the ordered-dither fraction).  Anything
// uncertain leaves the pixel to the FP64 path.  Bounds (u = 2^-24, n taps,
// A = sum of |term|): decode / weight conversion 2u^2 each, products 5u^2,
// additions 3u^2 relative to the partial sum, all within 24*n*u^2*A for a
// vertical sum; the reference's own rounding adds (2n+2)*2^-53*A.

// True if every real within 'delta' of hi + lo rounds to the float hi.
__device__ __forceinline__ bool rounds_to_hi(dfl x, float delta)
{
	const float up = __fsub_rn(nextafterf(x.hi, INFINITY), x.hi);
	const float down = __fsub_rn(x.hi, nextafterf(x.hi, -INFINITY));
	return isfinite(up) && isfinite(down) && __fsub_rn(x.lo, delta) > -0.5f * down && __fadd_rn(x.lo, delta) < 0.5f * up;
}

// The reference's float intermediates of every channel in 'mask' at (column
// x, row j), if all are certain.  The channels share the vertical weights
// (the fast form has one weight set per dimension), so each tap's pixel is
// read and its alpha decoded once for all of them.  UNROLL: taps whose loads
// are in flight together (register budget of the caller).
template<int UNROLL = 4>
__device__ __forceinline__ bool interm_df_all(const Job &J, unsigned int mask, int x, int j, float *out, int stride)
{
	const DWeights &W = J.wv[J.mid[0].wv];
	dfl acc[dev::kMaxCh];
	float A[dev::kMaxCh];
#pragma unroll
	for(int m = 0; m < dev::kMaxCh; m++) { acc[m] = {0.0f, 0.0f}; A[m] = 0.0f; }
	const int px = J.crop_x + x;
	int n = 1;
	// the alpha sample is read only for premultiplied channels, and only when
	// it is stored (a virtual alpha is 1; images without alpha have no table)
	bool need_alpha = false;
#pragma unroll
	for(int m = 0; m < dev::kMaxCh; m++)
		if(m < J.mid_n && ((mask >> m) & 1u) && J.mid[m].unassoc) need_alpha = true;
	need_alpha = need_alpha && J.in_alpha < J.in_nphys && J.df_atab != nullptr;
	auto add_tap = [&](int src, dfl w, bool copy) {
		const int py = J.crop_y + src;
		dfl a = {1.0f, 0.0f};
		if(need_alpha) a = df_of(J.df_atab[raw_code(J, px, py, J.in_alpha)]);
#pragma unroll
		for(int m = 0; m < dev::kMaxCh; m++) {
			if(m >= J.mid_n || !((mask >> m) & 1u)) continue;
			const DMid &mc = J.mid[m];
			dfl v = {1.0f, 0.0f};
			if(mc.in_ch < J.in_nphys) v = df_of(J.df_tab[m][raw_code(J, px, py, mc.in_ch)]);
			if(mc.unassoc && need_alpha) v = df_mul(v, a);
			if(copy) {
				acc[m] = v;
				A[m] = fabsf(v.hi);
			}
			else {
				acc[m] = df_add(acc[m], df_mul(v, w));
				A[m] = __fmaf_rn(fabsf(v.hi), fabsf(w.hi), A[m]);
			}
		}
	};
	if(W.kind == 1) {
		const int src = W.src[j];
		if(src >= 0) add_tap(src, {1.0f, 0.0f}, true);
	}
	else {
		const int tb = W.off[j], te = W.off[j + 1];
		n = te - tb;
#pragma unroll UNROLL
		for(int t = tb; t < te; t++) {   // unrolled so that the taps' loads are in flight together
			const int src = W.src[t];
			if(src >= 0) add_tap(src, df_of(J.df_wv[t]), false);   // edge taps add 0
		}
	}
	bool ok = true;
	const float kd = (float)(24 * n) * 3.5527137e-15f + (float)(2 * n + 2) * 1.1102231e-16f;
#pragma unroll
	for(int m = 0; m < dev::kMaxCh; m++) {
		if(m >= J.mid_n || !((mask >> m) & 1u)) continue;
		const float delta = __fmaf_rn(A[m] * 1.01f, kd, 1e-30f);
		out[m * stride] = acc[m].hi;
		// A == 0: every term is exactly zero (the smallest nonzero term, a
		// premultiplied code-1 sample times a weight, is far above the float
		// underflow), so the reference's sum is a zero too; its sign never
		// changes a later result or decision
		ok = ok && (A[m] == 0.0f || rounds_to_hi(acc[m], delta));
	}
	return ok;
}

// Ordered-dither thresholds (rank + 0.5) / 64: exact in float and double,
// equal to the reference's (double)(rank + 0.5) / 64.0.
__device__ __forceinline__ float dither_threshold(int rank) { return __fmul_rn((float)rank + 0.5f, 0.015625f); }

// Double-float copy of a double: hi + lo within u^2 |d| of d (d - hi is
// exact in double: hi carries d's leading 24 bits).
__device__ __forceinline__ dfl df_from_double(double d)
{
	const float hi = __double2float_rn(d);
	return {hi, __double2float_rn(dsub(d, (double)hi))};
}

// x / y in double-float for 0 <= x <= y: a float quotient and one
// correction from the double-float remainder; error below about 20 u^2
// (7e-14) absolute.
__device__ __forceinline__ dfl df_div_le1(dfl x, dfl y)
{
	const float q1 = __fdiv_rn(x.hi, y.hi);
	const dfl r = df_add(x, df_mul(y, {-q1, 0.0f}));
	return df_fast_two_sum(q1, __fdiv_rn(r.hi, y.hi));
}

// quantize_exact's code for one end of an interval (quantize_end), with FP64
// only for the two distances: the clamp, bracket and exactness tests compare
// bit patterns (order-preserving for non-negative doubles), and the
// ordered-dither fraction d_lo / (d_lo + d_hi) is taken in double-float:
// within 7e-14 of the exact ratio, and the reference's double fraction is
// within 2.3e-16 of it, so a decision 1e-12 or more away from the threshold
// is the reference's; nearer, 'ok' is cleared and the caller falls back to
// the exact path.
//
// The bits quantize_end decides on: v clamped to [+0, 1]; false for NaN
// (both candidate codes of a NaN convert to 0).
__device__ __forceinline__ bool quant_bits(double v, long long &vb)
{
	vb = __double_as_longlong(v);
	if((vb & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL) return false;
	if(vb < 0) vb = 0;                                                  // v < 0 (or -0): +0
	else if(vb > 0x3ff0000000000000LL) vb = 0x3ff0000000000000LL;       // v > 1: 1
	return true;
}

// quantize_end's decision for clamped bits vb in bracket k (no nearest-colour
// table).
__device__ __forceinline__ int quantize_in(const DQuant &q, long long vb, int k, int x, int y, bool &ok)
{
	const int clo = q.code[k], chi = q.code[k + 1];
	if(k == q.P || vb < __ldg(reinterpret_cast<const long long *>(q.X) + k)) return clo;   // exact
	const double vc = __longlong_as_double(vb);
	const double d_lo = dsub(vc, q.rev[clo]), d_hi = dsub(q.rev[chi], vc);
	if(q.dfam == IW_DITHERFAMILY_ORDERED) {
		const dfl l = df_from_double(d_lo), h = df_from_double(d_hi);
		const dfl f = df_div_le1(l, df_add(l, h));
		const float thr = dither_threshold(dither_rank(q.dsub, x, y));
		// f.hi - thr is exact near the threshold (Sterbenz)
		const float diff = __fadd_rn(__fsub_rn(f.hi, thr), f.lo);
		if(fabsf(diff) <= 1e-12f) ok = false;
		return diff >= 0.0f ? chi : clo;
	}
	return dle_bits(d_hi, d_lo) ? chi : clo;
}

// Bracket k of clamped bits vb with its decision record r (q.rec, 8 words
// per bracket): from q.lut's start point (else a binary search), stepped
// until r.lo <= vb < r.hi -- the bracket bracket_index finds.
__device__ __forceinline__ int bracket_rec(const DQuant &q, long long vb, EdRec &r)
{
	int k;
	if(q.lut) {
		const float vf = __double2float_rd(__longlong_as_double(vb));
		const int cell = min(max((int)__fmul_rn(vf, (float)kBracketLutCells), 0), kBracketLutCells - 1);
		k = min((int)__ldg(q.lut + cell), q.P);
	}
	else k = bracket_index(q, vb);
	r = ed_rec(q.rec, k);
	while(k < q.P && r.hi <= vb) r = ed_rec(q.rec, ++k);
	while(k > 0 && r.lo > vb) r = ed_rec(q.rec, --k);
	return k;
}

// quantize_in from bracket k's record.
__device__ __forceinline__ int quantize_in_rec(const DQuant &q, long long vb, int k, const EdRec &r, int x, int y, bool &ok)
{
	if(k == q.P || vb < r.x) return r.code_lo;   // exact
	const double vc = __longlong_as_double(vb);
	const double d_lo = dsub(vc, r.rev_lo), d_hi = dsub(r.rev_hi, vc);
	if(q.dfam == IW_DITHERFAMILY_ORDERED) {
		const dfl l = df_from_double(d_lo), h = df_from_double(d_hi);
		const dfl f = df_div_le1(l, df_add(l, h));
		const float thr = dither_threshold(dither_rank(q.dsub, x, y));
		const float diff = __fadd_rn(__fsub_rn(f.hi, thr), f.lo);
		if(fabsf(diff) <= 1e-12f) ok = false;
		return diff >= 0.0f ? r.code_hi : r.code_lo;
	}
	return dle_bits(d_hi, d_lo) ? r.code_hi : r.code_lo;
}

__device__ __forceinline__ int quantize_end(const DQuant &q, double v, int x, int y, bool &ok)
{
	long long vb;
	if(!quant_bits(v, vb)) return 0;
	if(q.use_nc) {
		const long long *nc = reinterpret_cast<const long long *>(q.nc);
		int lo = 0, hi = 255;
		while(lo < hi) {
			const int mid = (lo + hi) >> 1;
			if(__ldg(nc + mid) <= vb) lo = mid + 1; else hi = mid;
		}
		return lo;
	}
	return quantize_in(q, vb, bracket_index(q, vb), x, y, ok);
}

// Output code of every v in [vlo, vhi] as quantize_exact computes it;
// 'ok' false if it is not the same code over the interval (the decision is
// monotone in v within a bracket, and each end is checked above).
__device__ __forceinline__ int quantize_interval(const DQuant &q, double vlo, double vhi, int x, int y, bool &ok)
{
	long long blo, bhi;
	if(q.use_nc || !quant_bits(vlo, blo) || !quant_bits(vhi, bhi)) {
		const int clo = quantize_end(q, vlo, x, y, ok), chi = quantize_end(q, vhi, x, y, ok);
		if(clo != chi) ok = false;
		return clo;
	}
	// vlo <= vhi, so their brackets are in order: one search, and vhi's
	// bracket is vlo's unless vhi reaches that bracket's upper edge U[k+1]
	if(q.rec) {
		EdRec r, rh;
		const int k = bracket_rec(q, blo, r);
		int khi = k;
		rh = r;
		if(k < q.P && r.hi <= bhi) khi = bracket_rec(q, bhi, rh);
		const int clo = quantize_in_rec(q, blo, k, r, x, y, ok), chi = quantize_in_rec(q, bhi, khi, rh, x, y, ok);
		if(clo != chi) ok = false;
		return clo;
	}
	const int k = bracket_index(q, blo);
	const int khi = (k < q.P && __ldg(reinterpret_cast<const long long *>(q.U) + 1 + k) <= bhi) ? bracket_index(q, bhi) : k;
	const int clo = quantize_in(q, blo, k, x, y, ok), chi = quantize_in(q, bhi, khi, x, y, ok);
	if(clo != chi) ok = false;
	return clo;
}

// Horizontal taps of output column i (the fast form's one horizontal
// weight set): source columns, double-float weights (null: one tap of
// weight 1) and their count.
__device__ __forceinline__ void h_taps(const Job &J, int i, const int *&src, const float2 *&w, int &n)
{
	const DWeights &W = J.wh[J.mid[0].wh];
	if(W.kind == 1) {
		src = W.src + i;
		w = nullptr;
		n = 1;
	}
	else {
		src = W.src + W.off[i];
		w = J.df_wh + W.off[i];
		n = W.off[i + 1] - W.off[i];
	}
}

// Second half of the double-float re-evaluation of pixel (i, j), by a group
// of GW lanes (GW = 4: several pixels per warp, GW = 32: one): lane m of
// the group sums channel m's horizontal taps (hsrc, hw, nh as h_taps gives
// them) from the certified intermediate values in 'my' (maxt per channel),
// unassociates and quantises; true (group-uniform) with the codes stored if
// every decision was certain.  Every lane of the warp calls it; a lane whose
// group has no pixel passes live = false and never touches J.
template<int GW>
__device__ __forceinline__ bool fix_df_finish_g(const Job &J, int i, int j, unsigned int mask, const float *my, int maxt,
	int lane, bool live, const int *hsrc, const float2 *hw, int nh)
{
	static_assert(GW == 4 || GW == 32, "lane groups of 4 or 32");
	const int ch = lane & (GW - 1);
	const unsigned int gmask = GW == 32 ? 0xffffffffu : (((1u << GW) - 1u) << (lane & ~(GW - 1)));
	const bool mine = live && ch < J.mid_n && ((mask >> ch) & 1u);
	dfl s = {0.0f, 0.0f};
	float A = 0.0f;
	if(!mine) nh = 1;
	else {
		for(int tb = 0; tb < nh; tb += 8) {   // eight taps' loads in flight together
			int src[8];
			float I[8];
			float2 w[8];
#pragma unroll
			for(int u = 0; u < 8; u++) {
				const int t = tb + u;
				src[u] = t < nh ? hsrc[t] : -1;
				I[u] = t < nh ? my[ch * maxt + t] : 0.0f;
				w[u] = t >= nh ? make_float2(0.0f, 0.0f) : (hw ? hw[t] : make_float2(1.0f, 0.0f));
			}
#pragma unroll
			for(int u = 0; u < 8; u++) {
				if(src[u] < 0) continue;   // edge taps add nothing
				s = df_add_sloppy(s, df_mul_f(I[u], df_of(w[u])));   // per term below 3u^2 (table) + 2u^2 + 2.01u^2 of A
				A = __fmaf_rn(fabsf(I[u]), fabsf(w[u].x), A);
			}
		}
	}
	const float ds = __fmaf_rn(A * 1.01f, (float)(20 * nh) * 3.5527137e-15f + (float)(2 * nh + 2) * 1.1102231e-16f, 1e-30f);
	// the float alpha the reference divides by
	const int al = (live && J.mid_alpha >= 0) ? J.mid_alpha : 0;
	bool a_ok = true;
	if(mine && ch == al && J.mid_alpha >= 0) a_ok = A == 0.0f || rounds_to_hi(s, ds);   // A == 0: exact zero
	const float a32 = __shfl_sync(0xffffffffu, s.hi, al, GW);
	bool ok = __shfl_sync(0xffffffffu, a_ok ? 1 : 0, al, GW) != 0;
	int code = -1, oc = -1;
	bool is_alpha = false;
	if(mine && ok) {
		const DMid &mc = J.mid[ch];
		is_alpha = mc.ctype == IW_CHANNELTYPE_ALPHA;
		oc = mc.out_ch;
		dfl v = s;
		float dv = ds;
		if(mc.unassoc && a32 != 0.0f) {
			v = df_div_f(s, a32);
			dv = __fmaf_rn(fabsf(v.hi), 2.9e-14f + 1.2e-16f, __fdiv_rn(ds, fabsf(a32)) * 1.0001f);
		}
		if(oc >= 0) {
			const double vd = dadd((double)v.hi, (double)v.lo);
			const double d = (double)dv * 1.01 + fabs(vd) * 4.5e-16 + 1e-300;
			code = quantize_interval(J.outc[oc].q, dsub(vd, d), dadd(vd, d), i, j, ok);
		}
	}
	const bool gbad = (__ballot_sync(0xffffffffu, !ok) & gmask) != 0u;
	const int ac = __shfl_sync(0xffffffffu, code, al, GW);
	if(gbad || !live) return false;
	const int alpha_code = (J.mid_alpha >= 0 && J.mid[al].out_ch >= 0) ? ac : -1;
	if(code >= 0) {
		if(!is_alpha) {
			if(J.negate) code = J.outc[oc].maxcc - code;
			if(J.blacken && alpha_code == 0) code = 0;
		}
		store_code(J, oc, i, j, (unsigned int)code);
	}
	return true;
}

__device__ __forceinline__ bool fix_df_finish(const Job &J, int i, int j, unsigned int mask, const float *my, int maxt, int lane)
{
	const int *hsrc;
	const float2 *hw;
	int nh;
	h_taps(J, i, hsrc, hw, nh);
	return fix_df_finish_g<32>(J, i, j, mask, my, maxt, lane, true, hsrc, hw, nh);
}

// The codes of every channel of stored pixel (px, py): one aligned 8- or
// 4-byte load for 16-bit RGBA and 8-bit RGBA rows (where 'wide' says the
// image's rows and base allow it), else byte loads.
__device__ __forceinline__ void pixel_codes(const Job &J, int px, int py, bool wide, unsigned int (&c)[dev::kMaxCh])
{
	const uint8_t *row = J.in + (unsigned long long)py * J.in_bpr;
	if(wide && J.in_depth == 16) {
		const uint2 v = __ldg(reinterpret_cast<const uint2 *>(row) + px);
		c[0] = __byte_perm(v.x, 0u, 0x4401u);
		c[1] = __byte_perm(v.x, 0u, 0x4423u);
		c[2] = __byte_perm(v.y, 0u, 0x4401u);
		c[3] = __byte_perm(v.y, 0u, 0x4423u);
		return;
	}
	if(wide) {
		const unsigned int v = __ldg(reinterpret_cast<const unsigned int *>(row) + px);
#pragma unroll
		for(int k = 0; k < dev::kMaxCh; k++) c[k] = (v >> (8 * k)) & 0xffu;
		return;
	}
#pragma unroll
	for(int k = 0; k < dev::kMaxCh; k++) c[k] = k < J.in_nphys ? raw_code(J, px, py, k) : 0u;
}

// c[k] for a run-time k, by selects (an indexed register array would live in
// local memory)
__device__ __forceinline__ unsigned int pick4(const unsigned int (&c)[dev::kMaxCh], int k)
{
	return k == 0 ? c[0] : (k == 1 ? c[1] : (k == 2 ? c[2] : c[3]));
}

// The FP64 path of one flagged pixel, by a whole block: the block's threads
// recompute the intermediate values of every (channel, horizontal tap) at
// once, then warp 0 finishes each channel (lane m: channel m).  Every thread of the block calls it with the same entry.
__device__ void fix_pixel_fp64_block(const Job &J, int4 e, float *my, int maxt)
{
	const int lane = threadIdx.x & 31;
	const int p = e.x;
	const unsigned int mask = (unsigned int)e.y & ((1u << J.mid_n) - 1u);
	const int i = p % J.out_w, j = p / J.out_w;
	const int ntask = __popc(mask) * maxt;
	for(int k = threadIdx.x; k < ntask; k += blockDim.x) {
		const int r = k / maxt, t = k - r * maxt;
		const int m = nth_bit(mask, r);
		const DWeights &W = J.wh[J.mid[m].wh];
		const int t0 = W.kind == 1 ? i : W.off[i];
		const int nt = W.kind == 1 ? 1 : W.off[i + 1] - t0;
		if(t < nt) {
			const int src = W.src[t0 + t];
			if(src >= 0) my[m * maxt + t] = (float)interm_exact_ahead(J, m, src, j);
		}
	}
	__syncthreads();
	if(threadIdx.x < 32) {
		const bool mine = lane < J.mid_n && ((mask >> lane) & 1u);
		double s = 0.0;
		if(mine) s = hsum_exact(J, lane, i, j, [&](int m, int k, int) { return (double)my[m * maxt + k]; });
		const int al = J.mid_alpha >= 0 ? J.mid_alpha : 0;
		const double a = (double)__double2float_rn(__shfl_sync(0xffffffffu, s, al));
		int code = -1, oc = -1;
		bool is_alpha = false;
		if(mine) {
			const DMid &mc = J.mid[lane];
			is_alpha = mc.ctype == IW_CHANNELTYPE_ALPHA;
			oc = mc.out_ch;
			if(oc >= 0) {
				const DOut &o = J.outc[oc];
				const double v = unassoc_and_bkgd(J, mc, o, s, a, checker_alt(J, i, j), is_alpha);
				if(J.out_float) {
					float fv = __double2float_rn(v);
					if(J.negate && !is_alpha) fv = __fsub_rn(1.0f, fv);
					store_float(J, oc, i, j, fv);
				}
				else if(o.scan) J.scanbuf[((unsigned long long)oc * J.out_h + j) * J.out_w + i] = v;
				else code = quantize_exact(o.q, v, i, j);
			}
		}
		const int ac = __shfl_sync(0xffffffffu, code, al);
		const int alpha_code = (J.mid_alpha >= 0 && J.mid[al].out_ch >= 0) ? ac : -1;
		if(code >= 0) {
			if(!is_alpha) {
				if(J.negate) code = J.outc[oc].maxcc - code;
				if(J.blacken && alpha_code == 0) code = 0;
			}
			store_code(J, oc, i, j, (unsigned int)code);
		}
	}
	__syncthreads();   // 'my' is reused by the next pixel
}

// Re-evaluation of flagged pixels with small windows (up to 1280 input
// pixels per flagged pixel), a few pixels per block, each step one link of
// dependent loads long:
// step 0: the block's flag entries, then its pixels' vertical and horizontal
//   taps (source rows / columns and double-float weights) into shared memory;
// step 1: every (pixel, vertical tap, horizontal tap) input pixel is loaded
//   once -- up to kFixStageTasks per thread, all loads in flight together --
//   and decoded for every masked channel, leaving the double-float term
//   v * (a * w_v) in shared memory (an edge row leaves +0);
// step 2: thread (pixel, horizontal tap, channel) sums its column's terms
//   with df_add_sloppy and certifies the float intermediate as
//   interm_df_all does (bound (13 + 2.01 nv) u^2 A <= 24 nv u^2 A, which
//   holds for the exact real products in any order);
// step 3: four lanes of warp 0 per pixel finish it (fix_df_finish_g): the
//   decision reads one bracket record (q.rec) found from q.lut's start;
// step 4: a pixel steps 2-3 could not certify takes the FP64 path in place,
//   the whole block on it (fix_pixel_fp64_block).
// Shared memory (fix_stage_bytes): terms [pb][kMaxCh][maxv][maxt] float2,
// values [pb][kMaxCh][maxt] float, vertical and horizontal weights and
// sources.  Launch: pb * kMaxCh * maxt <= blockDim.x and
// pb * maxv * maxt <= kFixStageTasks * blockDim.x, pb <= 8.
constexpr int kFixStageThreads = 320;
constexpr int kFixStageTasks = 4;

__host__ __device__ __forceinline__ size_t fix_stage_bytes(int pb, int maxv, int maxt)
{
	const size_t terms = (size_t)pb * dev::kMaxCh * maxv * maxt * sizeof(float2);
	const size_t vals = (((size_t)pb * dev::kMaxCh * maxt + 1) & ~(size_t)1) * sizeof(float);
	return terms + vals + (size_t)pb * (maxv + maxt) * (sizeof(float2) + sizeof(int));
}

template<bool BATCH>
__global__ void __launch_bounds__(kFixStageThreads, 2) k_fix_stage(Job J1, const Job *jobs, int *count, const int *list,
	int maxv, int maxt, int pb, int listcap)
{
	extern __shared__ float4 fixs_smem[];
	const int TV = maxv * maxt;
	float2 *const s_term = reinterpret_cast<float2 *>(fixs_smem);
	float *const s_val = reinterpret_cast<float *>(s_term + (size_t)pb * dev::kMaxCh * TV);
	float2 *const s_vw = reinterpret_cast<float2 *>(s_val + ((pb * dev::kMaxCh * maxt + 1) & ~1));
	float2 *const s_hw = s_vw + pb * maxv;
	int *const s_vsrc = reinterpret_cast<int *>(s_hw + pb * maxt);
	int *const s_hsrc = s_vsrc + pb * maxv;
	__shared__ int4 s_e[8];
	__shared__ int s_nv[8], s_nh[8], s_bad[8];
	const int n = min(*count, listcap);
	for(int f0 = blockIdx.x * pb; f0 < n; f0 += gridDim.x * pb) {
		// ---- step 0: entries, then taps ----
		if(threadIdx.x < 8) {
			const int g = threadIdx.x;
			int4 e = make_int4(0, 0, 0, 0);
			int nv = 0, nh = 0, bad = 0;
			if(g < pb && f0 + g < n) {
				e = reinterpret_cast<const int4 *>(list)[f0 + g];
				const Job &J = BATCH ? jobs[e.z] : J1;
				const int i = e.x % J.out_w, j = e.x / J.out_w;
				const DWeights &WH = J.wh[J.mid[0].wh], &WV = J.wv[J.mid[0].wv];
				nh = WH.kind == 1 ? 1 : WH.off[i + 1] - WH.off[i];
				nv = WV.kind == 1 ? 1 : WV.off[j + 1] - WV.off[j];
				// windows never exceed the launch's maxv x maxt; a pixel
				// without double-float tables goes to the FP64 path
				if(J.df_wv == nullptr || nv > maxv || nh > maxt) {
					bad = 1;
					nv = nh = 0;
				}
			}
			s_e[g] = e;
			s_nv[g] = nv;
			s_nh[g] = nh;
			s_bad[g] = bad;
		}
		__syncthreads();
		for(int idx = threadIdx.x; idx < pb * (maxv + maxt); idx += blockDim.x) {
			const bool vert = idx < pb * maxv;
			const int q = vert ? idx : idx - pb * maxv;
			const int g = vert ? q / maxv : q / maxt, r = vert ? q - g * maxv : q - g * maxt;
			if(r >= (vert ? s_nv[g] : s_nh[g])) continue;
			const int4 e = s_e[g];
			const Job &J = BATCH ? jobs[e.z] : J1;
			const int i = e.x % J.out_w, j = e.x / J.out_w;
			if(vert) {
				const DWeights &WV = J.wv[J.mid[0].wv];
				const int t0 = WV.kind == 1 ? j : WV.off[j];
				s_vsrc[g * maxv + r] = WV.src[t0 + r];
				s_vw[g * maxv + r] = WV.kind == 1 ? make_float2(1.0f, 0.0f) : J.df_wv[t0 + r];
			}
			else {
				const DWeights &WH = J.wh[J.mid[0].wh];
				const int t0 = WH.kind == 1 ? i : WH.off[i];
				s_hsrc[g * maxt + r] = WH.src[t0 + r];
				s_hw[g * maxt + r] = WH.kind == 1 ? make_float2(1.0f, 0.0f) : J.df_wh[t0 + r];
			}
		}
		__syncthreads();
		// ---- step 1: the terms ----
		{
			const int total = pb * TV;
			int gg[kFixStageTasks], rr[kFixStageTasks], tt[kFixStageTasks];
			bool in[kFixStageTasks], live[kFixStageTasks];
			unsigned int cc[kFixStageTasks][dev::kMaxCh];
#pragma unroll
			for(int u = 0; u < kFixStageTasks; u++) {
				const int q = threadIdx.x + u * blockDim.x;
				gg[u] = rr[u] = tt[u] = 0;
				in[u] = live[u] = false;
				if(q < total) {
					const int g = q / TV, rem = q - g * TV, r = rem / maxt, t = rem - r * maxt;
					gg[u] = g;
					rr[u] = r;
					tt[u] = t;
					in[u] = r < s_nv[g] && t < s_nh[g];
					live[u] = in[u] && s_vsrc[g * maxv + r] >= 0 && s_hsrc[g * maxt + t] >= 0;
				}
#pragma unroll
				for(int m = 0; m < dev::kMaxCh; m++) cc[u][m] = 0u;
			}
#pragma unroll
			for(int u = 0; u < kFixStageTasks; u++) {
				if(!live[u]) continue;
				const Job &J = BATCH ? jobs[s_e[gg[u]].z] : J1;
				const bool wide = J.in_nphys == 4 && (J.in_depth == 16 || J.in_depth == 8) &&
					(((uintptr_t)J.in | (uintptr_t)J.in_bpr) & (J.in_depth == 16 ? 7u : 3u)) == 0;
				pixel_codes(J, J.crop_x + s_hsrc[gg[u] * maxt + tt[u]], J.crop_y + s_vsrc[gg[u] * maxv + rr[u]], wide, cc[u]);
			}
			float2 av[kFixStageTasks], vv[kFixStageTasks][dev::kMaxCh];
#pragma unroll
			for(int u = 0; u < kFixStageTasks; u++) {
				av[u] = make_float2(1.0f, 0.0f);
#pragma unroll
				for(int m = 0; m < dev::kMaxCh; m++) vv[u][m] = make_float2(0.0f, 0.0f);
				if(!live[u]) continue;
				const Job &J = BATCH ? jobs[s_e[gg[u]].z] : J1;
				const unsigned int mask = (unsigned int)s_e[gg[u]].y & ((1u << J.mid_n) - 1u);
				const bool have_a = J.in_alpha < J.in_nphys && J.df_atab != nullptr;
				bool need_a = false;
#pragma unroll
				for(int m = 0; m < dev::kMaxCh; m++) {
					if(m >= J.mid_n || !((mask >> m) & 1u)) continue;
					need_a = need_a || J.mid[m].unassoc;
					vv[u][m] = J.mid[m].in_ch < J.in_nphys ? __ldg(J.df_tab[m] + pick4(cc[u], J.mid[m].in_ch)) : make_float2(1.0f, 0.0f);
				}
				if(need_a && have_a) av[u] = __ldg(J.df_atab + pick4(cc[u], J.in_alpha));
			}
#pragma unroll
			for(int u = 0; u < kFixStageTasks; u++) {
				if(!in[u]) continue;
				const int g = gg[u];
				const Job &J = BATCH ? jobs[s_e[g].z] : J1;
				const unsigned int mask = (unsigned int)s_e[g].y & ((1u << J.mid_n) - 1u);
				const bool have_a = J.in_alpha < J.in_nphys && J.df_atab != nullptr;
				const dfl w = df_of(s_vw[g * maxv + rr[u]]);
				const dfl aw = df_mul(df_of(av[u]), w);
#pragma unroll
				for(int m = 0; m < dev::kMaxCh; m++) {
					if(m >= J.mid_n || !((mask >> m) & 1u)) continue;
					dfl tm = {0.0f, 0.0f};   // an edge row adds +0
					if(live[u]) tm = df_mul(df_of(vv[u][m]), (J.mid[m].unassoc && have_a) ? aw : w);
					s_term[((size_t)(g * dev::kMaxCh + m) * maxv + rr[u]) * maxt + tt[u]] = make_float2(tm.hi, tm.lo);
				}
			}
		}
		__syncthreads();
		// ---- step 2: certified column sums ----
		{
			const int g = threadIdx.x / (dev::kMaxCh * maxt), k = threadIdx.x - g * dev::kMaxCh * maxt;
			const int t = k / dev::kMaxCh, m = k - t * dev::kMaxCh;
			if(g < pb && f0 + g < n && !s_bad[g] && t < s_nh[g] && s_hsrc[g * maxt + t] >= 0) {
				const Job &J = BATCH ? jobs[s_e[g].z] : J1;
				const unsigned int mask = (unsigned int)s_e[g].y & ((1u << J.mid_n) - 1u);
				if(m < J.mid_n && ((mask >> m) & 1u)) {
					const int nv = s_nv[g];
					const float2 *col = s_term + (size_t)(g * dev::kMaxCh + m) * TV + t;
					dfl acc = {0.0f, 0.0f};
					float A = 0.0f;
					for(int r = 0; r < nv; r++) {
						const float2 v = col[r * maxt];
						acc = df_add_sloppy(acc, df_of(v));
						A = __fadd_rn(A, fabsf(v.x));
					}
					s_val[(g * dev::kMaxCh + m) * maxt + t] = acc.hi;
					const float kd = (float)(24 * nv) * 3.5527137e-15f + (float)(2 * nv + 2) * 1.1102231e-16f;
					const float delta = __fmaf_rn(A * 1.01f, kd, 1e-30f);
					// A == 0: every term is exactly zero (see interm_df_all)
					if(!(A == 0.0f || rounds_to_hi(acc, delta))) s_bad[g] = 1;
				}
			}
		}
		__syncthreads();
		// ---- step 3: finish ----
		if(threadIdx.x < 32) {
			const int g = threadIdx.x >> 2;
			const bool live = g < pb && f0 + g < n && !s_bad[g];
			const int4 e = s_e[g];
			const Job &J = BATCH ? jobs[e.z] : J1;   // read only when live
			unsigned int mask = 0u;
			int i = 0, j = 0;
			if(live) {
				mask = (unsigned int)e.y & ((1u << J.mid_n) - 1u);
				i = e.x % J.out_w;
				j = e.x / J.out_w;
			}
			const bool ok = fix_df_finish_g<dev::kMaxCh>(J, i, j, mask, s_val + g * dev::kMaxCh * maxt, maxt, threadIdx.x,
				live, s_hsrc + g * maxt, s_hw + g * maxt, live ? s_nh[g] : 1);
			if((threadIdx.x & 3) == 0 && live && !ok) s_bad[g] = 1;
		}
		__syncthreads();
		// ---- step 4: FP64 path ----
		for(int g = 0; g < pb && f0 + g < n; g++) {
			if(!s_bad[g]) continue;   // block-uniform
			const int4 e = s_e[g];
			if(threadIdx.x == 0) atomicAdd(count + 1, 1);   // pixels that needed the FP64 path
			fix_pixel_fp64_block(BATCH ? jobs[e.z] : J1, e, s_val, maxt);
		}
		__syncthreads();   // the shared arrays are reused by the next pixels
	}
}

// The FP64 path for the pixels listed at the tail of the flag list (count[3]
// entries from its end), one block per pixel.
template<bool BATCH>
__global__ void __launch_bounds__(256) k_fix_leftover(Job J1, const Job *jobs, const int *count, const int *list, int maxt,
	int cap)
{
	extern __shared__ float fix_cache[];
	const int n = min(*count, cap), left = min(count[3], cap - n);
	for(int L = blockIdx.x; L < left; L += gridDim.x) {
		const int4 e = reinterpret_cast<const int4 *>(list)[cap - 1 - L];
		fix_pixel_fp64_block(BATCH ? jobs[e.z] : J1, e, fix_cache, maxt);
	}
}

// Re-evaluation of flagged pixels with wide horizontal windows (48 taps or
// more), one block per pixel: the block's threads (one per horizontal tap)
// compute the certified double-float intermediate values the pixel reads --
// each a vertical sum over the pixel's rows, its loads in flight together
// with those of the other taps -- then warp 0 finishes (fix_df_finish).
// A pixel the double-float tier cannot decide is listed at the tail of the
// flag list for k_fix_leftover while there is room, else its FP64 path runs
// here.  Scratch: kMaxCh * maxt floats of shared memory.
template<bool BATCH>
__global__ void __launch_bounds__(256, 1) k_fix_wide_df(Job J1, const Job *jobs, int *count, int *list, int maxt, int cap)
{
	extern __shared__ float fix_cache[];
	float *my = fix_cache;
	__shared__ int s_ok, s_slot;
	const int n = min(*count, cap);
	const int lane = threadIdx.x & 31;
	for(int f = blockIdx.x; f < n; f += gridDim.x) {
		const int4 e = reinterpret_cast<const int4 *>(list)[f];
		const Job &J = BATCH ? jobs[e.z] : J1;
		const int p = e.x;
		const unsigned int mask = (unsigned int)e.y & ((1u << J.mid_n) - 1u);
		const int i = p % J.out_w, j = p / J.out_w;
		bool bad = J.df_wv == nullptr;
		if(!bad) {
			const DWeights &W = J.wh[J.mid[0].wh];
			const int t0 = W.kind == 1 ? i : W.off[i];
			const int nt = W.kind == 1 ? 1 : W.off[i + 1] - t0;
			// start the pixel's input window towards L2 (the walk below is a
			// chain of dependent loads: sample -> decode table): each thread
			// its column of every vertical tap's row (identity orientation,
			// byte samples; a hint only)
			if(J.orient == 0 && J.in_depth >= 8) {
				const DWeights &V = J.wv[J.mid[0].wv];
				const int vb = V.kind == 1 ? j : V.off[j], vn = V.kind == 1 ? 1 : V.off[j + 1] - vb;
				const unsigned long long bpp = (unsigned long long)J.in_nphys * (J.in_depth / 8);
				for(int t = threadIdx.x; t < nt; t += blockDim.x) {
					const int src = W.src[t0 + t];
					if(src < 0) continue;
					const uint8_t *colp = J.in + (unsigned long long)(J.crop_x + src) * bpp;
					for(int r = 0; r < vn; r++) {
						const int sv = V.src[vb + r];
						if(sv >= 0) asm volatile("prefetch.global.L2 [%0];" ::"l"(colp + (unsigned long long)(J.crop_y + sv) * J.in_bpr));
					}
				}
			}
			for(int t = threadIdx.x; t < nt; t += blockDim.x) {
				const int src = W.src[t0 + t];
				if(src >= 0 && !interm_df_all<8>(J, mask, src, j, my + t, maxt)) bad = true;
			}
		}
		bad = __syncthreads_or(bad) != 0;
		if(threadIdx.x < 32) {
			const bool ok = !bad && fix_df_finish(J, i, j, mask, my, maxt, lane);
			if(lane == 0) s_ok = ok ? 1 : 0;
		}
		__syncthreads();
		if(!s_ok) {
			if(threadIdx.x == 0) {
				atomicAdd(count + 1, 1);                  // pixels that needed the FP64 path
				s_slot = cap - 1 - atomicAdd(count + 3, 1);   // their entries at the list's tail
			}
			__syncthreads();
			const int slot = s_slot;
			if(slot >= n) {
				if(threadIdx.x == 0) reinterpret_cast<int4 *>(list)[slot] = e;
			}
			else fix_pixel_fp64_block(J, e, my, maxt);
		}
		__syncthreads();   // s_ok, s_slot and 'my' are reused by the next pixel
	}
}

// Fallback for very wide horizontal windows: one thread per flagged pixel.
template<bool BATCH>
__global__ void k_fix_flagged_thread(Job J1, const Job *jobs, int *count, const int *list, int cap)
{
	const int n = min(*count, cap);
	for(int f = blockIdx.x * blockDim.x + threadIdx.x; f < n; f += gridDim.x * blockDim.x) {
		const int4 e = reinterpret_cast<const int4 *>(list)[f];
		const Job &J = BATCH ? jobs[e.z] : J1;
		const int p = e.x;
		const int j = p / J.out_w;
		pixel_exact(J, p % J.out_w, j, true, [&](int m, int, int x) { return interm_exact<true>(J, m, x, j); },
			(unsigned int)e.y);
	}
}

// Launches the exact re-evaluation of flagged pixels on 'st' (flag list of
// capacity 'cap' entries).  Returns the launches.
template<bool BATCH>
static int launch_fix(cudaStream_t st, const Job &J, const Job *jobs, int maxv, int maxt, int *count, int *list, int cap)
{
	int sms = 152;
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
	const int T = dev::kMaxCh * maxt;
	{
		// small windows: every input pixel decoded once, in shared memory
		// (k_fix_stage); the most pixels per block that fit
		constexpr size_t kSmem = 96 * 1024;
		int pb = 8;
		while(pb > 0 && (pb * T > kFixStageThreads || pb * maxv * maxt > kFixStageTasks * kFixStageThreads ||
			fix_stage_bytes(pb, maxv, maxt) > kSmem))
			pb--;
		// one pixel per block leaves two pixels in flight per SM (registers):
		// the block-per-pixel kernel below keeps several times more
		if(pb >= 2) {
			static bool attr_done[2] = {false, false};
			if(!attr_done[BATCH]) {
				cudaFuncSetAttribute(k_fix_stage<BATCH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
				attr_done[BATCH] = true;
			}
			const int need = std::max(pb * T, (pb * maxv * maxt + kFixStageTasks - 1) / kFixStageTasks);
			const int threads = (need + 31) / 32 * 32;
			k_fix_stage<BATCH><<<8 * sms, threads, fix_stage_bytes(pb, maxv, maxt), st>>>(J, jobs, count, list, maxv, maxt, pb,
				cap);
			return 1;
		}
	}
	const size_t per_block = (size_t)T * sizeof(float);
	if(per_block <= 48 * 1024) {
		// larger windows: a block per pixel, one thread per horizontal tap
		// (small blocks, many pixels in flight per SM); the pixels left to
		// FP64 are listed at the tail of the flag list
		const int tpb = std::min(256, (maxt + 31) / 32 * 32);
		k_fix_wide_df<BATCH><<<8 * sms, tpb, per_block, st>>>(J, jobs, count, list, maxt, cap);
		k_fix_leftover<BATCH><<<4 * sms, 256, per_block, st>>>(J, jobs, count, list, maxt, cap);
		return 2;
	}
	k_fix_flagged_thread<BATCH><<<24 * sms, 64, 0, st>>>(J, jobs, count, list, cap);
	return 1;
}

void launch_fix_flagged(cudaStream_t st, const Job &J, int *count, int *list, int cap)
{
	int maxt = 1, maxv = 1;
	for(int m = 0; m < J.mid_n; m++) {
		maxt = std::max(maxt, J.wh[J.mid[m].wh].max_taps);
		maxv = std::max(maxv, J.wv[J.mid[m].wv].max_taps);
	}
	launch_fix<false>(st, J, nullptr, maxv, maxt, count, list, cap);
}

// The same for a batch: flag entries name their image in 'jobs' (device
// memory); maxt is the widest horizontal window of any image.
int launch_fix_flagged_batch(cudaStream_t st, const Job *jobs, int maxv, int maxt, int *count, int *list, int cap)
{
	Job none;
	memset(&none, 0, sizeof(none));
	return launch_fix<true>(st, none, jobs, maxv, maxt, count, list, cap);
}

// Device form of the output post-pass's property scan (optimize.cpp
// scan_pixels; src/imagew-opt.c:18-386) over the output image while it is in
// device memory: bit 0 a 16-bit sample whose two bytes differ (16 bits
// needed), bit 1 an alpha below full (transparency), bit 2 an alpha strictly
// between 0 and full (partial transparency), bit 3 a pixel whose R, G and B
// differ (colour).  Warp-level OR, one atomic per warp with a bit set.
__global__ void k_out_props(const uint8_t *out, int w, int h, unsigned long long bpr, int nch, int wide, int has_a,
	int rgb, unsigned int *flags)
{
	unsigned int f = 0;
	const unsigned int full = wide ? 65535u : 255u;
	const long long total = (long long)w * h;
	const long long step = (long long)gridDim.x * blockDim.x;
	for(long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < total; p += step) {
		const int y = (int)(p / w), x = (int)(p - (long long)y * w);
		const uint8_t *q = out + (unsigned long long)y * bpr + (unsigned long long)x * nch * (wide ? 2 : 1);
		unsigned int v[4] = {0, 0, 0, 0};
		for(int k = 0; k < nch && k < 4; k++) {
			if(wide) {
				v[k] = ((unsigned int)q[2 * k] << 8) | q[2 * k + 1];
				if(q[2 * k] != q[2 * k + 1]) f |= 1u;
			}
			else v[k] = q[k];
		}
		if(has_a && v[nch - 1] < full) {
			f |= 2u;
			if(v[nch - 1] > 0) f |= 4u;
		}
		if(rgb && (v[0] != v[1] || v[0] != v[2])) f |= 8u;
	}
	f = __reduce_or_sync(0xffffffffu, f);
	if((threadIdx.x & 31) == 0 && f) atomicOr(flags, f);
}

// ===========================================================================
// Host side: device memory, tables, launches
// ===========================================================================

namespace {

// Grow-only device buffer, allocated and freed in stream order on its lane's
// stream, so growing it never waits for work on other streams (a plain
// cudaFree would wait for the whole device).
struct DevBuf {
	void *p = nullptr;
	size_t cap = 0;
	cudaStream_t st = nullptr;
	bool ensure(size_t n)
	{
		if(n <= cap) return true;
		if(p) cudaFreeAsync(p, st);
		p = nullptr;
		cap = 0;
		size_t want = n + n / 4 + 4096;
		if(cudaMallocAsync(&p, want, st) != cudaSuccess) {
			cudaGetLastError();
			p = nullptr;
			return false;
		}
		cap = want;
		return true;
	}
};

// ---- host <-> device transfers through pinned staging ----
//
// A kernel reading the caller's pageable buffer directly (zero copy) is fast
// once the device has touched those pages, but the first touch of fresh pages
// costs a translation per page.  Staging copies instead: host threads copy the
// caller's bytes into one half of a pinned buffer while the copy engine moves
// the other half, so neither waits for page pinning or page faults.

// A fixed set of host threads for parallel memcpy.
struct HostPool {
	std::mutex run_mu;   // one run at a time (callers on different lanes take turns)
	std::mutex mu;
	std::condition_variable cv, cv_done;
	std::vector<std::thread> th;
	std::function<void(int)> task;
	int ntask = 0, next = 0, pending = 0;
	unsigned gen = 0;
	bool stop = false;
	HostPool()
	{
		int n = (int)std::thread::hardware_concurrency();
		n = std::max(1, std::min(n, 32)) - 1;
		for(int k = 0; k < n; k++) th.emplace_back([this] { loop(); });
	}
	void loop()
	{
		unsigned seen = 0;
		for(;;) {
			std::unique_lock<std::mutex> lk(mu);
			cv.wait(lk, [&] { return stop || gen != seen; });
			if(stop) return;
			seen = gen;
			while(next < ntask) {
				const int t = next++;
				lk.unlock();
				task(t);
				lk.lock();
				if(--pending == 0) cv_done.notify_all();
			}
		}
	}
	// Runs fn(0..n-1) on the pool and the calling thread; returns when all are done.
	void run(int n, const std::function<void(int)> &fn)
	{
		if(n <= 0) return;
		std::lock_guard<std::mutex> one(run_mu);
		std::unique_lock<std::mutex> lk(mu);
		task = fn;
		ntask = n;
		next = 0;
		pending = n;
		gen++;
		cv.notify_all();
		while(next < ntask) {
			const int t = next++;
			lk.unlock();
			fn(t);
			lk.lock();
			if(--pending == 0) cv_done.notify_all();
		}
		cv_done.wait(lk, [&] { return pending == 0; });
	}
};

HostPool &host_pool()
{
	static HostPool *p = new HostPool();   // never destroyed
	return *p;
}

// Device copy of a host buffer the GPU can read (pageable memory on a system
// with pageable memory access): 16-byte loads, four in flight per thread,
// then the tail.  Both pointers 16-byte aligned.
__global__ void __launch_bounds__(256) k_pull(uint8_t *dst, const uint8_t *src, size_t n)
{
	const size_t n16 = n / 16;
	const uint4 *s16 = reinterpret_cast<const uint4 *>(src);
	uint4 *d16 = reinterpret_cast<uint4 *>(dst);
	const size_t stride = (size_t)gridDim.x * blockDim.x;
	size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	for(; i + 3 * stride < n16; i += 4 * stride) {
		const uint4 a = s16[i], b = s16[i + stride], c = s16[i + 2 * stride], d = s16[i + 3 * stride];
		d16[i] = a;
		d16[i + stride] = b;
		d16[i + 2 * stride] = c;
		d16[i + 3 * stride] = d;
	}
	for(; i < n16; i += stride) d16[i] = s16[i];
	const size_t t = n16 * 16 + (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if(t < n) dst[t] = src[t];
}

// The same for a batch: block b copies images b, b + grid, ... (16-byte
// words where both ends are aligned, bytes otherwise).
struct PullItem { uint8_t *dst; const uint8_t *src; unsigned long long n; };

__global__ void __launch_bounds__(256) k_pull_many(const PullItem *items, int count)
{
	for(int it = blockIdx.x; it < count; it += gridDim.x) {
		const PullItem p = items[it];
		if(((uintptr_t)p.src | (uintptr_t)p.dst) & 15) {
			for(unsigned long long b = threadIdx.x; b < p.n; b += blockDim.x) p.dst[b] = p.src[b];
			continue;
		}
		const unsigned long long n16 = p.n / 16;
		const uint4 *s16 = reinterpret_cast<const uint4 *>(p.src);
		uint4 *d16 = reinterpret_cast<uint4 *>(p.dst);
		unsigned long long i = threadIdx.x;
		for(; i + 3 * blockDim.x < n16; i += 4 * blockDim.x) {
			const uint4 a = s16[i], b = s16[i + blockDim.x], c = s16[i + 2 * blockDim.x], d = s16[i + 3 * blockDim.x];
			d16[i] = a;
			d16[i + blockDim.x] = b;
			d16[i + 2 * blockDim.x] = c;
			d16[i + 3 * blockDim.x] = d;
		}
		for(; i < n16; i += blockDim.x) d16[i] = s16[i];
		const unsigned long long t = n16 * 16 + threadIdx.x;
		if(t < p.n) p.dst[t] = p.src[t];
	}
}

struct Piece { uint8_t *dst; const uint8_t *src; size_t n; };

// memcpy of many pieces, split in 1 MiB parts over the host pool.
void copy_pieces(const std::vector<Piece> &pieces)
{
	constexpr size_t kPart = (size_t)1 << 20;
	std::vector<Piece> parts;
	size_t total = 0;
	for(const Piece &p : pieces)
		for(size_t o = 0; o < p.n; o += kPart) {
			parts.push_back({p.dst + o, p.src + o, std::min(kPart, p.n - o)});
			total += std::min(kPart, p.n - o);
		}
	if(total < ((size_t)2 << 20)) {
		for(const Piece &p : parts) memcpy(p.dst, p.src, p.n);
		return;
	}
	host_pool().run((int)parts.size(), [&](int k) { memcpy(parts[k].dst, parts[k].src, parts[k].n); });
}

struct Xfer { uint8_t *dev; uint8_t *host; size_t n; };

// Waits for an event or a stream.  A patient wait sleeps between queries
// instead of spinning: lanes that wait seconds for a serial scan must not take
// host cores from the planning and copying threads.
cudaError_t wait_event(cudaEvent_t e, bool patient)
{
	if(!patient) return cudaEventSynchronize(e);
	cudaError_t r;
	while((r = cudaEventQuery(e)) == cudaErrorNotReady) std::this_thread::sleep_for(std::chrono::microseconds(200));
	return r;
}

cudaError_t wait_stream(cudaStream_t st, bool patient)
{
	if(!patient) return cudaStreamSynchronize(st);
	cudaError_t r;
	while((r = cudaStreamQuery(st)) == cudaErrorNotReady) std::this_thread::sleep_for(std::chrono::microseconds(200));
	return r;
}

struct Stager {
	uint8_t *pin[2] = {nullptr, nullptr};
	size_t half = 0;
	bool patient = false;
	cudaEvent_t ev[2] = {nullptr, nullptr};
	bool ensure()
	{
		if(pin[0]) return true;
		const size_t want = (size_t)64 << 20;
		if(cudaMallocHost((void **)&pin[0], 2 * want) != cudaSuccess) { pin[0] = nullptr; return false; }
		pin[1] = pin[0] + want;
		half = want;
		cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming);
		cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming);
		return true;
	}
};

// Host -> device for every item, on 'st'.  Returns once the host side is
// done; the last copies may still be in flight on the stream.
bool stage_h2d(Stager &G, cudaStream_t st, const std::vector<Xfer> &items)
{
	if(!G.ensure()) return false;
	int slot = 0;
	size_t fill = 0;
	std::vector<Piece> host_side;
	std::vector<Xfer> dma;
	auto flush = [&]() {
		if(!fill) return;
		copy_pieces(host_side);
		for(const Xfer &x : dma) cudaMemcpyAsync(x.dev, x.host, x.n, cudaMemcpyHostToDevice, st);
		cudaEventRecord(G.ev[slot], st);
		host_side.clear();
		dma.clear();
		fill = 0;
		slot ^= 1;
		wait_event(G.ev[slot], G.patient);   // the other half is free again
	};
	wait_event(G.ev[0], G.patient);
	for(const Xfer &x : items) {
		size_t off = 0;
		while(off < x.n) {
			const size_t take = std::min(G.half - fill, x.n - off);
			host_side.push_back({G.pin[slot] + fill, x.host + off, take});
			dma.push_back({x.dev + off, G.pin[slot] + fill, take});
			fill += take;
			off += take;
			if(fill == G.half) flush();
		}
	}
	flush();
	return true;
}

// Device -> host for every item after the work queued on 'st'; returns when
// the bytes are in the callers' buffers.
bool stage_d2h(Stager &G, cudaStream_t st, const std::vector<Xfer> &items)
{
	if(!G.ensure()) return false;
	struct Group { std::vector<Piece> out; std::vector<Xfer> dma; };
	std::vector<Group> groups(1);
	size_t fill = 0;
	for(const Xfer &x : items) {
		size_t off = 0;
		while(off < x.n) {
			if(fill == G.half) { groups.emplace_back(); fill = 0; }
			const size_t take = std::min(G.half - fill, x.n - off);
			// pin offsets are relative; the half is chosen when the group is issued
			groups.back().dma.push_back({x.dev + off, (uint8_t *)(uintptr_t)fill, take});
			groups.back().out.push_back({x.host + off, (const uint8_t *)(uintptr_t)fill, take});
			fill += take;
			off += take;
		}
	}
	auto issue = [&](size_t g) {
		uint8_t *pin = G.pin[g & 1];
		for(const Xfer &x : groups[g].dma)
			cudaMemcpyAsync(pin + (uintptr_t)x.host, x.dev, x.n, cudaMemcpyDeviceToHost, st);
		cudaEventRecord(G.ev[g & 1], st);
	};
	for(size_t g = 0; g < groups.size() && g < 2; g++) issue(g);
	using Clk = std::chrono::steady_clock;
	double t_wait = 0, t_copy = 0;
	for(size_t g = 0; g < groups.size(); g++) {
		const Clk::time_point t0 = Clk::now();
		if(wait_event(G.ev[g & 1], G.patient) != cudaSuccess) return false;
		const Clk::time_point t1 = Clk::now();
		std::vector<Piece> out = groups[g].out;
		for(Piece &p : out) p.src = G.pin[g & 1] + (uintptr_t)p.src;
		copy_pieces(out);
		t_wait += std::chrono::duration<double, std::milli>(t1 - t0).count();
		t_copy += std::chrono::duration<double, std::milli>(Clk::now() - t1).count();
		if(g + 2 < groups.size()) issue(g + 2);
	}
	if(!G.patient) {   // lane 0: account the device wait and the host copies apart
		batch_phase_add(8, t_wait);
		batch_phase_add(9, t_copy);
	}
	return true;
}

// Per-process device state: one stream, grow-only buffers and a cache of
// device copies of the shared host tables.  Calls are serialised on it.
struct DeviceState {
	std::mutex mu;
	int lane = 0;
	bool init = false;
	std::string init_error;
	int device = 0;
	int pageable = 0;          // kernels may access pageable host memory (Grace: NVLink-C2C + ATS)
	cudaStream_t stream = nullptr;
	DevBuf in, interm, out, scan, err, params, flags, dbg;
	DevBuf batch_io, batch_tab;   // batches: buffers + tables of all images
	cudaStream_t dl_stream = nullptr;   // scan lanes: per-image downloads while the batch's scans run
	int *done_h = nullptr;              // scan lanes: per-image completion flags (mapped host memory)
	int *done_d = nullptr;
	int done_cap = 0;
	std::map<const void *, std::pair<std::shared_ptr<const void>, void *>> table_cache;
	std::mutex table_mu;   // table_cache: batches build jobs on several host threads
	std::vector<uint8_t> staging;
	Stager stager;
};

// Hardware work queues: CUDA maps streams onto CUDA_DEVICE_MAX_CONNECTIONS
// queues (8 unless set), and work queued behind a long kernel of another
// stream on the same queue waits for it.  The lanes' streams each get a
// queue of their own with 32; the variable is read when the process creates
// its CUDA context, and a value the process set itself is kept.
__attribute__((constructor)) static void iwg_hardware_queues()
{
	setenv("CUDA_DEVICE_MAX_CONNECTIONS", "32", 0);
}

// Lanes: independent device states (stream, buffers, table cache), so that a
// request server can keep long serial work (dither scans) on lanes of its own,
// apart from its batches and from each other.  Lane 0 serves the public entry
// points.  A lane's stream and buffers are created on its first use.
DeviceState &state(int lane = 0)
{
	static DeviceState *s[kLanes] = {};   // never destroyed: outlive other statics
	static std::once_flag once;
	std::call_once(once, [] {
		for(int k = 0; k < kLanes; k++) {
			s[k] = new DeviceState();
			s[k]->lane = k;
		}
	});
	return *s[(unsigned)lane % (unsigned)kLanes];
}

// A kernel that needs 256 bytes of local memory per thread, launched once
// at initialisation: the driver sizes its local-memory allocation at the
// first launch that needs more than it has, and that resize waits for the
// whole device; done here, before any lane runs work, no later launch of the
// library's kernels (at most a few dozen bytes of spill) has to resize.
__global__ void k_size_local_memory(int *sink)
{
	volatile int buf[64];
	for(int k = 0; k < 64; k++) buf[k] = k + (int)threadIdx.x;
	if(sink) sink[threadIdx.x] = buf[(threadIdx.x * 7) & 63];
}

// Every kernel of the library, loaded once per process before any lane runs
// work: under lazy module loading a kernel's first launch loads its module,
// and that can wait for long scans running on other lanes.
void preload_kernels()
{
	static std::once_flag once;
	std::call_once(once, [] {
		k_size_local_memory<<<1, 32>>>(nullptr);
		cudaDeviceSynchronize();
		cudaFuncAttributes a;
		for(const void *k : {(const void *)k_vpass_exact, (const void *)k_hpass_exact, (const void *)k_scan,
			(const void *)k_finalize, (const void *)kb_vpass_exact, (const void *)kb_hpass_exact, (const void *)kb_scan,
			(const void *)kb_finalize,
			(const void *)k_fix_stage<true>, (const void *)k_fix_stage<false>,
			(const void *)k_fix_wide_df<true>, (const void *)k_fix_wide_df<false>, (const void *)k_out_props,
			(const void *)k_fix_leftover<true>, (const void *)k_fix_leftover<false>,
			(const void *)k_fix_flagged_thread<true>, (const void *)k_fix_flagged_thread<false>,
			(const void *)k_pull,
			(const void *)k_pull_many})
			cudaFuncGetAttributes(&a, k);
		preload_fast_kernels();
		preload_batch_kernels();
		preload_noalloc_kernels();
		cudaGetLastError();
	});
}

bool ensure_init(DeviceState &S, std::string &err)
{
	if(S.init) return true;
	int n = 0;
	cudaError_t e = cudaGetDeviceCount(&n);
	if(e != cudaSuccess || n < 1) {
		err = std::string("No CUDA device available: ") + cudaGetErrorString(e);
		return false;
	}
	cudaGetDevice(&S.device);
	cudaDeviceGetAttribute(&S.pageable, cudaDevAttrPageableMemoryAccess, S.device);
	// lane 0 (the public entry points, a server's batches) on the highest
	// priority: the block scheduler then serves it first while long scans of
	// other lanes hold part of the GPU
	int least = 0, greatest = 0;
	cudaDeviceGetStreamPriorityRange(&least, &greatest);
	if(cudaStreamCreateWithPriority(&S.stream, cudaStreamNonBlocking, S.lane == 0 ? greatest : least) != cudaSuccess) {
		err = "cudaStreamCreate failed";
		return false;
	}
	for(DevBuf *b : {&S.in, &S.interm, &S.out, &S.scan, &S.err, &S.params, &S.flags, &S.dbg, &S.batch_io, &S.batch_tab})
		b->st = S.stream;
	S.stager.patient = S.lane != 0;
	if(S.lane != 0 && cudaStreamCreateWithPriority(&S.dl_stream, cudaStreamNonBlocking, least) != cudaSuccess) {
		err = "cudaStreamCreate failed";
		return false;
	}
	preload_kernels();
	{   // keep freed stream-ordered memory in the pool rather than returning it at
		// every synchronise; and never let an allocation on one lane reuse memory
		// whose free on another lane's stream is still pending (the pool would
		// make the first stream wait for the second, e.g. behind a long scan)
		cudaMemPool_t pool;
		if(cudaDeviceGetDefaultMemPool(&pool, S.device) == cudaSuccess) {
			unsigned long long keep = ~0ULL;
			cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
			int no = 0;
			cudaMemPoolSetAttribute(pool, cudaMemPoolReuseAllowInternalDependencies, &no);
		}
		cudaGetLastError();
	}
	S.init = true;
	return true;
}

template<class T>
const T *cached_table(DeviceState &S, const std::shared_ptr<const std::vector<T>> &v)
{
	if(!v) return nullptr;
	std::lock_guard<std::mutex> lk(S.table_mu);
	auto it = S.table_cache.find(v.get());
	if(it != S.table_cache.end()) return (const T *)it->second.second;
	void *d = nullptr;
	size_t n = v->size() * sizeof(T);
	if(cudaMalloc(&d, n ? n : 16) != cudaSuccess) return nullptr;
	cudaMemcpyAsync(d, v->data(), n, cudaMemcpyHostToDevice, S.stream);   // the lane's stream, not the legacy one
	cudaStreamSynchronize(S.stream);
	S.table_cache[v.get()] = {std::static_pointer_cast<const void>(v), d};
	return (const T *)d;
}

// Packs per-call arrays into one staging block uploaded with a single copy.
struct Packer {
	std::vector<uint8_t> &buf;
	explicit Packer(std::vector<uint8_t> &b) : buf(b) { buf.clear(); }
	template<class T>
	size_t add(const T *p, size_t n)
	{
		size_t off = (buf.size() + 255) & ~(size_t)255;
		buf.resize(off + n * sizeof(T));
		if(n) memcpy(buf.data() + off, p, n * sizeof(T));
		return off;
	}
};

struct Fixup { size_t off; const void **slot; };

}  // namespace

template<class Mark>
int plain_launch(cudaStream_t st, const Plan &P, const Job &J, Mark mark);

// Transfer mode of a context: "gpu:upload" = "copy" (cudaMemcpy from / to the
// caller's pageable buffers), "stage" (pinned staging with host copy threads)
// or "zero" (kernels read and write the caller's host buffers in place; needs
// pageable memory access, and is slow on the first touch of fresh pages).
// or "pull" (one image: a copy kernel reads the caller's input over the
// CPU-GPU link into device memory; needs pageable memory access).  Measured
// on GB300 (Grace, NVLink-C2C) for a freshly malloc'd 134 MB input: a kernel
// reads it at 143-161 GB/s, while a cudaMemcpyAsync from those fresh
// pageable pages ran near 60 GB/s (host copies into pinned memory top out
// near 95 GB/s with 8-16 threads).  Default: "pull" for one image where the
// GPU reads pageable memory, else "copy"; "stage" for batches on lane 0 (many
// pageable copies are slow one by one, and they synchronise with work
// already queued); "zero" on a server's scan lanes.  'resident' runs need
// the input on the device.
enum { UP_ZERO = 0, UP_COPY = 1, UP_STAGE = 2, UP_PULL = 3 };
static int upload_mode(iw_context *ctx, const DeviceState &S, bool resident, bool many = false, bool pull_many = false)
{
	const char *u = get_option(ctx, "gpu:upload");
	// scan lanes (a server's error-diffusion requests: small images, many
	// lanes) read and write the callers' buffers in place where the GPU can
	// (no pinned staging buffer per lane, no download stream); lane 0 stages
	// its batches
	int m = many ? (S.lane != 0 ? UP_ZERO : UP_STAGE) : UP_PULL;
	if(u && !strcmp(u, "copy")) m = UP_COPY;
	if(u && !strcmp(u, "stage")) m = UP_STAGE;
	else if(u && !strcmp(u, "zero")) m = UP_ZERO;
	else if(u && !strcmp(u, "pull")) m = UP_PULL;
	if(m == UP_PULL && many && pull_many && S.pageable) return m;   // a batch: one copy kernel for every image
	if(m == UP_PULL && (!S.pageable || many || ((uintptr_t)ctx->img1.pixels & 15))) m = UP_COPY;   // (a linearised copy is 16-byte aligned too)
	if(m == UP_ZERO && (!S.pageable || resident)) m = UP_COPY;
	return m;
}

// Fills the device job description of a planned image: geometry, flags and
// the tables (weights packed into 'pk' with fix-ups for their device
// addresses; decode and quantisation tables from the device table cache).
// Buffers (input, intermediate, output, dither scratch) are left to the caller.
static bool make_job(iw_context *ctx, const Plan &P, DeviceState &S, Packer &pk, std::vector<Fixup> &fix, Job &J)
{
	memset(&J, 0, sizeof(J));
	J.in_bpr = plan_in_bpr(P);
	J.in_depth = P.in_depth;
	J.in_float = P.lin_in ? 2 : (P.in_sampletype == IW_SAMPLETYPE_FLOATINGPOINT ? 1 : 0);
	J.in_nphys = P.in_nphys;
	J.orient = P.orient;
	J.img1_w = P.img1_w;
	J.img1_h = P.img1_h;
	J.crop_x = P.crop_x; J.crop_y = P.crop_y; J.crop_w = P.crop_w; J.crop_h = P.crop_h;
	J.in_alpha = P.in_alpha;
	J.mid_n = P.mid_n;
	J.mid_alpha = P.mid_alpha;
	J.mid_w = P.crop_w;
	J.mid_h = P.out_h;
	J.interm_plane = (unsigned long long)J.mid_w * J.mid_h;
	J.out_bpr = P.out_bpr;
	J.out_w = P.out_w; J.out_h = P.out_h; J.out_n = P.out_n; J.out_depth = P.out_depth;
	J.out_float = P.out_sampletype == IW_SAMPLETYPE_FLOATINGPOINT;
	J.apply_bk = P.apply_bk;
	J.bk_late = P.apply_bk && P.bk_strategy == BK_LATE;
	J.bk_early = P.apply_bk && P.bk_strategy == BK_EARLY;
	J.bk_checker = P.apply_bk && P.bk_checker;
	J.bk_trns = P.bk_trns;
	J.bk1_alpha = P.bk1_alpha; J.bk2_alpha = P.bk2_alpha;
	J.check_size = P.check_size < 1 ? 1 : P.check_size;
	J.check_ox = P.check_origin[0]; J.check_oy = P.check_origin[1];
	J.gsf = P.gsf;
	for(int k = 0; k < 3; k++) J.gsw[k] = P.gsw[k];
	J.intclamp = P.intclamp;
	J.negate = P.negate;
	J.blacken = P.blacken;
	J.seed = ctx->seed;

	// processing order: alpha first, then the others in channel order
	{
		int n = 0;
		if(P.mid_alpha >= 0) J.order[n++] = P.mid_alpha;
		for(int m = 0; m < P.mid_n; m++) if(m != P.mid_alpha) J.order[n++] = m;
	}

	// ---- tables ----
	auto put = [&](const void **slot, size_t off) { fix.push_back({off, slot}); };
	std::vector<std::vector<float>> wf_store;
	for(int d = 0; d < 2; d++) {
		for(size_t k = 0; k < P.wsets[d].size(); k++) {
			const Weights &W = *P.wsets[d][k];
			DWeights &D = d == 0 ? J.wh[k] : J.wv[k];
			D.kind = (int)W.kind;
			D.n_in = W.n_in;
			D.n_out = W.n_out;
			D.max_taps = W.max_taps;
			D.edge_value = W.edge_value;
			wf_store.emplace_back(W.w.begin(), W.w.end());
			put((const void **)&D.off, pk.add(W.off.data(), W.off.size()));
			put((const void **)&D.src, pk.add(W.src.data(), W.src.size()));
			put((const void **)&D.w, pk.add(W.w.data(), W.w.size()));
			put((const void **)&D.wf, pk.add(wf_store.back().data(), wf_store.back().size()));
			put((const void **)&D.pos, pk.add(W.pos.data(), W.pos.size()));
		}
	}
	// decode tables (cached): per input channel, with the transfer each
	// intermediate channel uses
	auto decode_tab = [&](int ch, bool linear) -> const double * {
		if(ch >= P.in_nphys || P.in_sampletype == IW_SAMPLETYPE_FLOATINGPOINT) return nullptr;
		int ncodes = 1 << P.in_depth;
		int maxcc = P.reduced_in ? (int)P.in_maxcc_d[ch] : P.in_max;
		return cached_table(S, input_table(P.cs_in.cstype, P.cs_in.gamma, maxcc, ncodes, linear));
	};
	for(int m = 0; m < P.mid_n; m++) {
		const MidChannel &mc = P.mid[m];
		DMid &D = J.mid[m];
		D.ctype = mc.ctype; D.in_ch = mc.in_ch; D.to_gray = mc.to_gray; D.out_ch = mc.out_ch;
		D.unassoc = mc.unassoc; D.wh = mc.wset_h; D.wv = mc.wset_v; D.bk_early = mc.bk_early;
		for(int t = 0; t < (mc.to_gray ? 3 : 1); t++) {
			D.tab[t] = decode_tab(mc.in_ch + t, mc.lin_cs);
			if(!D.tab[t] && mc.in_ch + t < P.in_nphys && P.in_sampletype != IW_SAMPLETYPE_FLOATINGPOINT) {
				iw_set_error(ctx, "Out of GPU memory (tables)");
				return false;
			}
		}
	}
	J.alpha_tab = decode_tab(P.in_alpha, true);
	if(!J.alpha_tab && P.in_alpha < P.in_nphys && P.in_sampletype != IW_SAMPLETYPE_FLOATINGPOINT &&
		IW_IMGTYPE_HAS_ALPHA(P.in_logtype)) {
		iw_set_error(ctx, "Out of GPU memory (tables)");
		return false;
	}

	bool any_scan = false;
	for(int oc = 0; oc < P.out_n; oc++) {
		const OutChannel &o = P.out[oc];
		DOut &D = J.outc[oc];
		D.ctype = o.ctype;
		D.maxcc = o.maxcc;
		D.bk1 = o.bk1;
		D.bk2 = o.bk2;
		const Quant &q = o.q;
		D.q.float_out = q.float_out;
		if(q.float_out) continue;
		D.q.use_nc = q.use_nc; D.q.dfam = q.dfam; D.q.dsub = q.dsub; D.q.maxcc = q.maxcc; D.q.P = q.P;
		D.q.U = cached_table(S, q.U);
		D.q.X = cached_table(S, q.X);
		D.q.code = cached_table(S, q.code);
		D.q.rev = cached_table(S, q.rev);
		D.q.nc = cached_table(S, q.nc);
		D.q.rec = cached_table(S, q.rec);
		D.q.lut = nullptr;
		if(!D.q.U || !D.q.X || !D.q.code || !D.q.rev || (q.use_nc && !D.q.nc) || (q.rec && !D.q.rec)) {
			iw_set_error(ctx, "Out of GPU memory (tables)");
			return false;
		}
		D.scan = q.dfam == IW_DITHERFAMILY_ERRDIFF || q.dfam == IW_DITHERFAMILY_RANDOM;
		if(D.scan) any_scan = true;
	}
	J.any_scan = any_scan;

	return true;
}

bool run_pipeline(iw_context *ctx, Plan &P, int warmup, int iters, int lane)
{
	DeviceState &S = state(lane);
	std::lock_guard<std::mutex> lk(S.mu);
	std::string err;
	if(!ensure_init(S, err)) {
		iw_set_error(ctx, err.c_str());
		return false;
	}

	// host output image, owned by the context
	ctx->img2.bpr = P.out_bpr;
	ctx->img2.pixels = (iw_byte *)iw_malloc_large(ctx, P.out_bpr, P.out_h);
	if(!ctx->img2.pixels) return false;

	Job J;
	Packer pk(S.staging);
	std::vector<Fixup> fix;
	if(!make_job(ctx, P, S, pk, fix, J)) return false;
	const int phys_h = P.orient >= 4 ? P.img1_w : P.img1_h;
	const size_t in_bytes = plan_in_bpr(P) * (size_t)phys_h;
	const bool any_scan = J.any_scan != 0;

	// ---- buffers ----
	// Zero copy: where the GPU can access pageable host memory coherently
	// (cudaDevAttrPageableMemoryAccess), the kernels read the caller's input
	// image and write the output image in place, over the CPU-GPU link, instead
	// of staging copies.  Timed runs keep the input resident in device memory.
	const int upmode = upload_mode(ctx, S, warmup > 0 || iters > 1);
	const bool zero_copy = upmode == UP_ZERO;
	const size_t interm_bytes = (size_t)P.mid_n * J.interm_plane * sizeof(float);
	const size_t out_bytes = P.out_bpr * (size_t)P.out_h;
	// failure tests: option gpu:fail_alloc=1 makes this call's device
	// allocation fail as cudaMalloc would when memory runs out
	const char *fa = get_option(ctx, "gpu:fail_alloc");
	const bool inject_oom = fa && !strcmp(fa, "1");
	if(inject_oom || (!zero_copy && (!S.in.ensure(in_bytes ? in_bytes : 16) || !S.out.ensure(out_bytes))) ||
		!S.interm.ensure(interm_bytes) || !S.params.ensure(S.staging.size() + 256)) {
		iw_set_error(ctx, "Out of GPU memory");
		return false;
	}
	if(any_scan) {
		if(!S.scan.ensure((size_t)P.out_n * P.out_w * P.out_h * sizeof(double)) ||
			!S.err.ensure((size_t)P.out_n * 5 * P.out_w * sizeof(double))) {
			iw_set_error(ctx, "Out of GPU memory");
			return false;
		}
		J.scanbuf = (double *)S.scan.p;
		J.errbuf = (double *)S.err.p;
	}
	J.in = zero_copy ? (const uint8_t *)plan_input(ctx, P) : (const uint8_t *)S.in.p;
	J.interm = (float *)S.interm.p;
	J.out = zero_copy ? (uint8_t *)ctx->img2.pixels : (uint8_t *)S.out.p;
	ctx->stats.zero_copy = zero_copy;
	for(const Fixup &f : fix) *f.slot = (const uint8_t *)S.params.p + f.off;

	cudaStream_t st = S.stream;
	// phase events: upload, device passes, download
	struct PhaseEvents {
		cudaEvent_t e[4] = {nullptr, nullptr, nullptr, nullptr};
		PhaseEvents() { for(cudaEvent_t &x : e) cudaEventCreate(&x); }
		~PhaseEvents() { for(cudaEvent_t x : e) if(x) cudaEventDestroy(x); }
	} phases;
	cudaEvent_t *const ph = phases.e;
	cudaEventRecord(ph[0], st);
	cudaMemcpyAsync(S.params.p, S.staging.data(), S.staging.size(), cudaMemcpyHostToDevice, st);
	if(upmode == UP_COPY) cudaMemcpyAsync(S.in.p, plan_input(ctx, P), in_bytes, cudaMemcpyHostToDevice, st);
	if(upmode == UP_PULL && in_bytes) {
		int sms = 152;
		cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, S.device);
		const size_t n16 = in_bytes / 16;
		const unsigned blocks = (unsigned)std::max<size_t>(1, std::min<size_t>((n16 + 1023) / 1024, (size_t)8 * sms));
		k_pull<<<blocks, 256, 0, st>>>((uint8_t *)S.in.p, (const uint8_t *)plan_input(ctx, P), in_bytes);
	}
	if(upmode == UP_STAGE &&
		!stage_h2d(S.stager, st, {Xfer{(uint8_t *)S.in.p, (uint8_t *)plan_input(ctx, P), in_bytes}})) {
		iw_set_error(ctx, "Out of pinned host memory");
		return false;
	}

	cudaEventRecord(ph[1], st);
	const char *prec = get_option(ctx, "gpu:precision");
	bool want_plain = prec && !strcmp(prec, "fp64");
	FastInfo fi;
	{
		const char *vt = get_option(ctx, "gpu:vertical");
		fi.tc_mode = (vt && !strcmp(vt, "cuda")) ? 0 : ((vt && !strcmp(vt, "tensor")) ? 2 : 1);
		const char *at = get_option(ctx, "gpu:autotune");
		fi.autotune = !(at && !strcmp(at, "off"));
		// the fused pass is measured slower than the two passes today (its
		// vertical and horizontal phases serialise inside each block): on
		// request only
		const char *fu = get_option(ctx, "gpu:fuse");
		fi.fuse_mode = (fu && !strcmp(fu, "on")) ? 1 : 0;
		// failure tests: gpu:wait_test=1 starves the bulk-copy pipeline (its
		// producer issues no copies, so no barrier it waits on ever
		// completes) and shortens its waits to a few thousand polls
		const char *wt = get_option(ctx, "gpu:wait_test");
		fi.starve = (wt && !strcmp(wt, "1")) ? 1 : 0;
		fi.wait_polls = fi.starve ? 4096 : 0;
	}
	bool fast = !want_plain && fast_eligible(P, J, fi);
	ctx->stats.form = fast ? 1 : 0;
	// Debug readback (option gpu:debug_values=1, one untimed pass): the
	// intermediate image and, per output sample, the value the tail quantises
	// (and, in the fast form, its error bound) are copied to the context.
	const char *dbgopt = get_option(ctx, "gpu:debug_values");
	const bool want_dbg = dbgopt && !strcmp(dbgopt, "1") && warmup == 0 && iters <= 1 && P.out_sampletype == IW_SAMPLETYPE_UINT;
	const size_t dbg_n = (size_t)P.out_n * P.out_w * P.out_h;
	ctx->dbg.clear();
	if(want_dbg) {
		if(!S.dbg.ensure(dbg_n * 8 + 16)) {
			iw_set_error(ctx, "Out of GPU memory");
			return false;
		}
		cudaMemsetAsync(S.dbg.p, 0xff, dbg_n * 8, st);   // NaN: no value
		if(fast) fi.dbg = (float *)S.dbg.p;
		else J.dbg = (double *)S.dbg.p;
	}
	ctx->stats.vertical_tensor = 0;
	if(fast && !fast_prepare(st, P, J, fi, err)) {
		iw_set_error(ctx, err.c_str());
		return false;
	}
	ctx->stats.vertical_tensor = fast ? fi.tc : 0;
	ctx->stats.fused = fast ? fi.fused : 0;

	// The device passes, launched warmup+iters times; the input stays resident.
	// Events bracket every launch group of the timed iterations.
	const int total_it = warmup + (iters < 1 ? 1 : iters);
	const int nt = total_it - warmup;
	std::vector<cudaEvent_t> ev;
	auto mark = [&](bool timed) {
		if(!timed) return;
		cudaEvent_t e;
		cudaEventCreate(&e);
		cudaEventRecord(e, st);
		ev.push_back(e);
	};
	int launches = 0, marks_per_it = 0;
	for(int it = 0; it < total_it; it++) {
		bool timed = it >= warmup;
		size_t before = ev.size();
		mark(timed);
		int l;
		if(fast) l = fast_launch(st, fi, [&]() { mark(timed); });
		else l = plain_launch(st, P, J, [&]() { mark(timed); });
		if(timed) marks_per_it = (int)(ev.size() - before);
		launches = l;
	}
	// Repeated passes of a resident image (the timed entry point): the fast
	// form's launches captured once as a CUDA graph and replayed nt times
	// between two events; that mean is the device time per pass.  The
	// per-launch breakdown comes from the directly launched passes above.
	float graph_ms = -1.0f;
	ctx->stats.graph = 0;
	if(fast && nt > 1) {
		cudaGraph_t g = nullptr;
		cudaGraphExec_t gx = nullptr;
		if(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed) == cudaSuccess) {
			fast_launch(st, fi, []() {});
			if(cudaStreamEndCapture(st, &g) != cudaSuccess || !g || cudaGraphInstantiate(&gx, g, 0) != cudaSuccess) gx = nullptr;
		}
		cudaGetLastError();
		if(gx) {
			cudaEvent_t ga, gb;
			cudaEventCreate(&ga);
			cudaEventCreate(&gb);
			cudaGraphLaunch(gx, st);   // warm-up replay
			cudaEventRecord(ga, st);
			bool ok = true;
			for(int it = 0; it < nt && ok; it++) ok = cudaGraphLaunch(gx, st) == cudaSuccess;
			cudaEventRecord(gb, st);
			if(ok && cudaEventSynchronize(gb) == cudaSuccess && cudaEventElapsedTime(&graph_ms, ga, gb) == cudaSuccess) {
				graph_ms /= (float)nt;
				ctx->stats.graph = 1;
			}
			else graph_ms = -1.0f;
			cudaEventDestroy(ga);
			cudaEventDestroy(gb);
			cudaGraphExecDestroy(gx);
		}
		if(g) cudaGraphDestroy(g);
		cudaGetLastError();
	}
	// The post-pass's property scan as a device reduction over the output,
	// where the host would scan it (16-bit, or 8-bit with more than one
	// channel; integer output at a full max code) and the output is in device
	// memory; the flags come back with the image.
	unsigned int prop_flags = 0;
	bool props = false;
	{
		const int ot = ctx->img2.imgtype, od = ctx->img2.bit_depth;
		const bool wide = od == 16;
		if(!zero_copy && ctx->img2.sampletype == IW_SAMPLETYPE_UINT && !ctx->reduced_out && (od == 8 || od == 16) &&
			!(ot == IW_IMGTYPE_GRAY && !wide) && P.out_w > 0 && P.out_h > 0 && S.flags.ensure(16)) {
			const int nch = iw_imgtype_num_channels(ot);
			cudaMemsetAsync(S.flags.p, 0, sizeof(unsigned int), st);
			const long long px = (long long)P.out_w * P.out_h;
			const unsigned blocks = (unsigned)std::min<long long>((px + 255) / 256, 4096);
			k_out_props<<<blocks, 256, 0, st>>>((const uint8_t *)S.out.p, P.out_w, P.out_h, (unsigned long long)P.out_bpr,
				nch, wide ? 1 : 0, IW_IMGTYPE_HAS_ALPHA(ot) ? 1 : 0, IW_IMGTYPE_IS_GRAY(ot) ? 0 : 1, (unsigned int *)S.flags.p);
			props = true;
		}
	}
	if(S.lane != 0) wait_stream(st, true);   // downloads queued once the kernels are done (as for batches)
	if(want_dbg) {
		// intermediate planes in intermediate-channel order, then the values
		// (and bounds): all as doubles on the host
		const size_t plane = (size_t)J.interm_plane;
		std::vector<float> im((size_t)P.mid_n * plane), fv(fast ? 2 * dbg_n : 0);
		std::vector<double> dv(fast ? 0 : dbg_n);
		for(int m = 0; m < P.mid_n; m++)
			cudaMemcpyAsync(im.data() + (size_t)m * plane, J.interm + (size_t)(fast ? fi.plane_of[m] : m) * plane,
				plane * sizeof(float), cudaMemcpyDeviceToHost, st);
		if(fast) cudaMemcpyAsync(fv.data(), S.dbg.p, 2 * dbg_n * sizeof(float), cudaMemcpyDeviceToHost, st);
		else cudaMemcpyAsync(dv.data(), S.dbg.p, dbg_n * sizeof(double), cudaMemcpyDeviceToHost, st);
		if(cudaStreamSynchronize(st) == cudaSuccess) {
			ctx->dbg.interm.assign(im.begin(), im.end());
			if(fast) {
				ctx->dbg.value.assign(fv.begin(), fv.begin() + dbg_n);
				ctx->dbg.bound.assign(fv.begin() + dbg_n, fv.end());
			}
			else {
				ctx->dbg.value = dv;
				ctx->dbg.bound.assign(dbg_n, 0.0);
			}
			ctx->dbg.dims[0] = P.mid_n; ctx->dbg.dims[1] = J.mid_h; ctx->dbg.dims[2] = J.mid_w;
			ctx->dbg.dims[3] = P.out_n; ctx->dbg.dims[4] = P.out_h; ctx->dbg.dims[5] = P.out_w;
		}
	}
	cudaEventRecord(ph[2], st);
	if(props) cudaMemcpyAsync(&prop_flags, S.flags.p, sizeof(unsigned int), cudaMemcpyDeviceToHost, st);
	if(upmode == UP_COPY || upmode == UP_PULL) cudaMemcpyAsync(ctx->img2.pixels, S.out.p, out_bytes, cudaMemcpyDeviceToHost, st);
	if(upmode == UP_STAGE) stage_d2h(S.stager, st, {Xfer{(uint8_t *)S.out.p, (uint8_t *)ctx->img2.pixels, out_bytes}});
	cudaEventRecord(ph[3], st);
	cudaError_t ce = wait_stream(st, S.lane != 0);
	for(int k = 0; k < 3; k++) {
		float v = 0.0f;
		ctx->stats.ms_phase[1 + k] = (ce == cudaSuccess && cudaEventElapsedTime(&v, ph[k], ph[k + 1]) == cudaSuccess) ? v : 0.0;
	}
	cudaGetLastError();
	if(ce == cudaSuccess) ce = cudaGetLastError();
	ctx->opt_dev_props = (ce == cudaSuccess && props) ? (int)(prop_flags | 0x100u) : 0;
	ctx->stats.flagged = 0;
	ctx->stats.flagged_exact = 0;
	if(ce == cudaSuccess && fast && fi.flag_count_dev) {
		int nflag[3] = {0, 0, 0};
		ce = cudaMemcpyAsync(nflag, fi.flag_count_dev, 3 * sizeof(int), cudaMemcpyDeviceToHost, st);
		if(ce == cudaSuccess) ce = cudaStreamSynchronize(st);
		ctx->stats.flagged = nflag[0];
		ctx->stats.flagged_exact = nflag[1];
		if(ce == cudaSuccess && nflag[2]) {
			fast_release(fi);
			for(cudaEvent_t e : ev) cudaEventDestroy(e);
			iw_set_error(ctx, nflag[2] == 2 ? "Internal: flag list overflow" : "A device wait ran out of time (vertical pass)");
			return false;
		}
	}
	double total_ms = 0, part[8] = {0, 0, 0, 0, 0, 0, 0, 0};
	if(ce == cudaSuccess && marks_per_it >= 2) {
		for(int it = 0; it < nt; it++) {
			cudaEvent_t *e = ev.data() + (size_t)it * marks_per_it;
			float ms = 0;
			cudaEventElapsedTime(&ms, e[0], e[marks_per_it - 1]);
			total_ms += ms;
			for(int k = 0; k + 1 < marks_per_it && k < 8; k++) {
				cudaEventElapsedTime(&ms, e[k], e[k + 1]);
				part[k] += ms;
			}
		}
	}
	for(cudaEvent_t e : ev) cudaEventDestroy(e);
	fast_release(fi);
	if(ce != cudaSuccess) {
		iw_set_errorf(ctx, "CUDA error: %s", cudaGetErrorString(ce));
		return false;
	}
	ctx->stats.ms_device = graph_ms > 0.0f ? (double)graph_ms : total_ms / nt;
	for(int k = 0; k < 4; k++) ctx->stats.ms_part[k] = part[k] / nt;
	ctx->stats.kernels = launches;
	return true;
}

// Batches of at least this many images prepare their jobs on the host pool
// (shared by all lanes, so a small serving batch would wait for it).
constexpr int kPoolMin = 16;

// make_job for the images 'which' on the host threads.  Each image packs its
// arrays into a buffer of its own; the buffers are then appended to
// S.staging in image order, each at a 256-byte boundary (as the packer aligns
// its arrays), and the image's fix-up offsets moved by its buffer's position,
// so the result equals packing them one after the other.  ok[k]: make_job's
// result for which[k].
static void make_jobs(const std::vector<iw_context *> &ctxs, const std::vector<Plan *> &plans, const std::vector<int> &which,
	DeviceState &S, std::vector<std::vector<Fixup>> &fixes, std::vector<Job> &jobs, std::vector<char> &ok)
{
	const int m = (int)which.size();
	std::vector<std::vector<uint8_t>> bufs(m);
	ok.assign(m, 0);
	auto one = [&](int k) {
		const int i = which[k];
		Packer pk(bufs[k]);
		ok[k] = make_job(ctxs[i], *plans[i], S, pk, fixes[i], jobs[i]) ? 1 : 0;
	};
	if(m < kPoolMin)   // small batches (serving): no wait for the shared pool
		for(int k = 0; k < m; k++) one(k);
	else
		host_pool().run(m, [&](int k) {
			cudaSetDevice(S.device);   // pool threads: the lane's device for the table uploads
			one(k);
		});
	S.staging.clear();
	for(int k = 0; k < m; k++) {
		if(!ok[k]) continue;
		const size_t base = (S.staging.size() + 255) & ~(size_t)255;
		S.staging.resize(base + bufs[k].size());
		if(!bufs[k].empty()) memcpy(S.staging.data() + base, bufs[k].data(), bufs[k].size());
		for(Fixup &f : fixes[which[k]]) f.off += base;
	}
}

// A batch of planned images.  The images the fast form takes run together:
// one launch per kernel variant for the vertical and horizontal passes, one
// exact re-evaluation launch for the flagged pixels of all of them.  Each
// image keeps its own tables and buffers, so its bytes equal a lone run's.
// status[i]: 1 done here, 0 left for the caller (run it alone), -1 failed
// (error set on the context).  'dev_ms' receives the batch's device time.
// Host wall time of run_batch's phases, summed over calls: job packing and
// the fast form's host preparation, uploads, the passes' launches, the
// fix-up's launch, the wait for the device with the downloads, the rest; and
// inside the passes' launches, the table upload and the attribute calls.
namespace {
std::mutex g_phase_mu;
double g_phase_ms[kBatchPhases] = {};
using PhaseClock = std::chrono::steady_clock;
struct PhaseTimer {
	PhaseClock::time_point t = PhaseClock::now();
	double d[6] = {0, 0, 0, 0, 0, 0};
	void mark(int k)
	{
		const PhaseClock::time_point n = PhaseClock::now();
		d[k] += std::chrono::duration<double, std::milli>(n - t).count();
		t = n;
	}
	~PhaseTimer()
	{
		mark(5);
		std::lock_guard<std::mutex> lk(g_phase_mu);
		for(int k = 0; k < 6; k++) g_phase_ms[k] += d[k];
	}
};
}  // namespace

void batch_phase_add(int k, double ms)
{
	std::lock_guard<std::mutex> lk(g_phase_mu);
	g_phase_ms[k] += ms;
}

void batch_phase_ms(double *out)
{
	std::lock_guard<std::mutex> lk(g_phase_mu);
	for(int k = 0; k < kBatchPhases; k++) out[k] = g_phase_ms[k];
}

bool run_batch(const std::vector<iw_context *> &ctxs, const std::vector<Plan *> &plans, std::vector<int> &status,
	double &dev_ms, int lane)
{
	DeviceState &S = state(lane);
	std::lock_guard<std::mutex> lk(S.mu);
	PhaseTimer pt;
	const int n = (int)ctxs.size();
	status.assign(n, 0);
	dev_ms = 0;
	std::string err;
	if(!ensure_init(S, err)) {
		for(int i = 0; i < n; i++) { iw_set_error(ctxs[i], err.c_str()); status[i] = -1; }
		return false;
	}
	std::vector<Job> jobs(n);                 // sized once: fix-ups point into it
	std::vector<std::vector<Fixup>> fixes(n);
	std::vector<int> cand, sel;
	for(int i = 0; i < n; i++) {
		const char *prec = get_option(ctxs[i], "gpu:precision");
		if(prec && !strcmp(prec, "fp64")) continue;
		// images the fast form cannot take are left to the plain-form batch
		// (which builds their jobs): decided from the plan, before packing
		FastInfo fi;
		if(!fast_eligible(*plans[i], jobs[i], fi)) continue;
		cand.push_back(i);
	}
	{
		std::vector<char> ok;
		make_jobs(ctxs, plans, cand, S, fixes, jobs, ok);
		for(size_t k = 0; k < cand.size(); k++) {
			const int i = cand[k];
			if(!ok[k]) { status[i] = -1; continue; }
			if(jobs[i].any_scan) continue;
			sel.push_back(i);
		}
	}
	if(sel.empty()) return true;

	// one transfer mode for the batch: the first image's
	const int upmode = upload_mode(ctxs[sel[0]], S, false, true, true);
	const bool zc = upmode == UP_ZERO;
	// buffers of every image, the packed weight lists and the flag list in one block
	size_t top = 0;
	auto take = [&](size_t bytes) { size_t at = (top + 255) & ~(size_t)255; top = at + bytes; return at; };
	const size_t o_par = take(S.staging.size());
	const size_t o_cnt = take(256);
	size_t nflag = 0;
	for(int i : sel) nflag += (size_t)plans[i]->out_w * plans[i]->out_h;
	const size_t o_flags = take(nflag * 16);
	std::vector<size_t> o_in(n, 0), o_mid(n, 0), o_out(n, 0), in_bytes(n, 0), out_bytes(n, 0);
	for(int i : sel) {
		const Plan &P = *plans[i];
		in_bytes[i] = plan_in_bpr(P) * (size_t)(P.orient >= 4 ? P.img1_w : P.img1_h);
		out_bytes[i] = P.out_bpr * (size_t)P.out_h;
		if(!zc) o_in[i] = take(in_bytes[i] ? in_bytes[i] : 16);
		o_mid[i] = take((size_t)P.mid_n * jobs[i].interm_plane * sizeof(float));
		if(!zc) o_out[i] = take(out_bytes[i]);
	}
	if(!S.batch_io.ensure(top)) {
		for(int i : sel) { iw_set_error(ctxs[i], "Out of GPU memory (batch)"); status[i] = -1; }
		return false;
	}
	uint8_t *base = (uint8_t *)S.batch_io.p;
	int *flag_count = (int *)(base + o_cnt);
	int *flag_list = (int *)(base + o_flags);

	// final device addresses, then the fast form's host preparation of every
	// image on the host threads (fast_batch_item is safe to call concurrently)
	std::vector<void *> items;
	std::vector<int> item_img;
	std::vector<int> ready;
	for(int i : sel) {
		iw_context *ctx = ctxs[i];
		const Plan &P = *plans[i];
		Job &J = jobs[i];
		for(const Fixup &f : fixes[i]) *f.slot = base + o_par + f.off;
		ctx->img2.bpr = P.out_bpr;
		ctx->img2.pixels = (iw_byte *)iw_malloc_large(ctx, P.out_bpr, P.out_h);
		if(!ctx->img2.pixels) { status[i] = -1; continue; }
		J.in = zc ? (const uint8_t *)plan_input(ctx, P) : base + o_in[i];
		J.interm = (float *)(base + o_mid[i]);
		J.out = zc ? (uint8_t *)ctx->img2.pixels : base + o_out[i];
		ready.push_back(i);
	}
	std::vector<void *> prepared(ready.size(), nullptr);
	auto prep = [&](int k) {
		std::string e2;
		prepared[k] = fast_batch_item(*plans[ready[k]], jobs[ready[k]], e2);
	};
	if((int)ready.size() < kPoolMin)   // small batches (serving): no wait for the shared pool
		for(int k = 0; k < (int)ready.size(); k++) prep(k);
	else
		host_pool().run((int)ready.size(), [&](int k) {
			cudaSetDevice(S.device);   // pool threads: the lane's device for the table uploads
			prep(k);
		});
	for(size_t k = 0; k < ready.size(); k++) {
		const int i = ready[k];
		if(!prepared[k]) {   // leave it to the caller's lone run
			iw_free(ctxs[i], ctxs[i]->img2.pixels);
			ctxs[i]->img2.pixels = nullptr;
			continue;
		}
		items.push_back(prepared[k]);
		item_img.push_back(i);
	}
	if(items.empty()) return true;
	const int m = (int)items.size();

	// per-image arrays of the fast form and the exact form's job array
	std::vector<uint8_t> tab;
	auto add = [&](const void *p, size_t bytes) {
		size_t at = (tab.size() + 255) & ~(size_t)255;
		tab.resize(at + bytes);
		if(bytes) memcpy(tab.data() + at, p, bytes);
		return at;
	};
	std::vector<size_t> o_blob(m);
	for(int k = 0; k < m; k++) o_blob[k] = add(fast_item_blob(items[k]), fast_item_blob_bytes(items[k]));
	std::vector<Job> djobs(m);
	for(int k = 0; k < m; k++) djobs[k] = jobs[item_img[k]];
	const size_t o_jobs = add(djobs.data(), djobs.size() * sizeof(Job));
	size_t o_pull = 0;
	if(upmode == UP_PULL) {
		std::vector<PullItem> pv(m);
		for(int k = 0; k < m; k++) {
			const int i = item_img[k];
			pv[k] = PullItem{base + o_in[i], (const uint8_t *)plan_input(ctxs[i], *plans[i]), (unsigned long long)in_bytes[i]};
		}
		o_pull = add(pv.data(), pv.size() * sizeof(PullItem));
	}
	auto fail_all = [&](const char *msg) {
		for(int k = 0; k < m; k++) {
			iw_set_error(ctxs[item_img[k]], msg);
			status[item_img[k]] = -1;
			fast_item_free(items[k]);
		}
		return false;
	};
	if(!S.batch_tab.ensure(tab.size())) return fail_all("Out of GPU memory (batch tables)");
	uint8_t *tbase = (uint8_t *)S.batch_tab.p;
	int maxt = 1, maxv = 1;
	for(int k = 0; k < m; k++) {
		fast_item_place(items[k], tbase + o_blob[k], flag_count, flag_list, k, nflag);
		maxt = std::max(maxt, fast_item_htaps(items[k]));
		maxv = std::max(maxv, fast_item_vtaps(items[k]));
		// the job record gets the image's placed double-float pointers
		fast_item_job_df(items[k], djobs[k]);
		memcpy(tab.data() + o_jobs + (size_t)k * sizeof(Job), &djobs[k], sizeof(Job));
	}

	cudaStream_t st = S.stream;
	cudaEvent_t e0, e1;
	cudaEventCreate(&e0);
	cudaEventCreate(&e1);
	pt.mark(0);
	cudaMemcpyAsync(base + o_par, S.staging.data(), S.staging.size(), cudaMemcpyHostToDevice, st);
	cudaMemcpyAsync(tbase, tab.data(), tab.size(), cudaMemcpyHostToDevice, st);
	if(upmode == UP_COPY)
		for(int k = 0; k < m; k++) {
			const int i = item_img[k];
			cudaMemcpyAsync(base + o_in[i], plan_input(ctxs[i], *plans[i]), in_bytes[i], cudaMemcpyHostToDevice, st);
		}
	if(upmode == UP_STAGE) {
		std::vector<Xfer> xs;
		for(int k = 0; k < m; k++) {
			const int i = item_img[k];
			xs.push_back({base + o_in[i], (uint8_t *)plan_input(ctxs[i], *plans[i]), in_bytes[i]});
		}
		if(!stage_h2d(S.stager, st, xs)) return fail_all("Out of pinned host memory");
	}
	if(upmode == UP_PULL) {
		int sms = 152;
		cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, S.device);
		k_pull_many<<<(unsigned)std::min(m, 8 * sms), 256, 0, st>>>((const PullItem *)(tbase + o_pull), m);
	}
	cudaMemsetAsync(flag_count, 0, 4 * sizeof(int), st);
	cudaEvent_t ev_h, ev_f;
	cudaEventCreate(&ev_h);
	cudaEventCreate(&ev_f);
	cudaEventRecord(e0, st);
	pt.mark(1);
	// vertical and horizontal groups, then the re-evaluation, launched
	// directly.  (Captured as one CUDA graph, the same launches gave correct
	// output for this batch but wrong output for the plain-form batch run on
	// the lane right after it; the cause was not found, so batches do not use
	// graphs.)
	const bool graphed = false;
	int launches = fast_launch_batch(st, items.data(), m, err, ev_h, ev_f, [&]() {
		return launch_fix_flagged_batch(st, (const Job *)(tbase + o_jobs), maxv, maxt, flag_count, flag_list,
			(int)std::min<size_t>(nflag, 0x7fffffff));
	}, nullptr);
	pt.mark(2);
	cudaEventRecord(e1, st);
	pt.mark(3);
	if(upmode == UP_COPY)
		for(int k = 0; k < m; k++) {
			const int i = item_img[k];
			cudaMemcpyAsync(ctxs[i]->img2.pixels, base + o_out[i], out_bytes[i], cudaMemcpyDeviceToHost, st);
		}
	if(upmode == UP_STAGE || upmode == UP_PULL) {
		std::vector<Xfer> xs;
		for(int k = 0; k < m; k++) {
			const int i = item_img[k];
			xs.push_back({base + o_out[i], (uint8_t *)ctxs[i]->img2.pixels, out_bytes[i]});
		}
		stage_d2h(S.stager, st, xs);
	}
	cudaError_t ce = wait_stream(st, S.lane != 0);
	if(ce == cudaSuccess) ce = cudaGetLastError();
	pt.mark(4);
	int nflagged[3] = {0, 0, 0};
	float ms = 0, ms_v = 0, ms_h = 0, ms_f = 0;
	if(ce == cudaSuccess) ce = cudaMemcpyAsync(nflagged, flag_count, 3 * sizeof(int), cudaMemcpyDeviceToHost, st);
	if(ce == cudaSuccess) ce = cudaStreamSynchronize(st);
	if(ce == cudaSuccess && nflagged[2]) {
		err = "A device wait ran out of time (vertical pass); nothing was written";
		launches = -1;
	}
	if(ce == cudaSuccess) {
		cudaEventElapsedTime(&ms, e0, e1);
		cudaEventElapsedTime(&ms_v, e0, ev_h);
		cudaEventElapsedTime(&ms_h, ev_h, ev_f);
		cudaEventElapsedTime(&ms_f, ev_f, e1);
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	cudaEventDestroy(ev_h);
	cudaEventDestroy(ev_f);
	if(launches < 0) return fail_all(err.c_str());
	if(ce != cudaSuccess) {
		std::string msg = std::string("CUDA error: ") + cudaGetErrorString(ce);
		return fail_all(msg.c_str());
	}
	dev_ms = ms;
	for(int k = 0; k < m; k++) {
		iw_context *ctx = ctxs[item_img[k]];
		ctx->stats.form = 1;
		ctx->stats.graph = graphed ? 1 : 0;
		ctx->stats.zero_copy = zc;
		ctx->stats.kernels = launches;
		ctx->stats.ms_device = ms;
		ctx->stats.ms_part[0] = ms_v;
		ctx->stats.ms_part[1] = ms_h;
		ctx->stats.ms_part[2] = ms_f;
		ctx->stats.flagged = nflagged[0];
		ctx->stats.flagged_exact = nflagged[1];
		status[item_img[k]] = 1;
		fast_item_free(items[k]);
	}
	return true;
}

// A batch in the plain (FP64) form: every image runs the reference's
// arithmetic through batched launches of the plain kernels, and the serial
// dither scans of all images run at once, one warp per channel.  For images
// the fast form does not take (error-diffusion / random dither, fp64
// requests, ...).  status / dev_ms as run_batch.
// Per-image completion flags of a scan lane: grow-only mapped host memory.
static bool ensure_done_flags(DeviceState &S, int n)
{
	if(n <= S.done_cap) return true;
	if(S.done_h) cudaFreeHost(S.done_h);
	S.done_h = nullptr;
	S.done_d = nullptr;
	S.done_cap = 0;
	const int cap = std::max(n, 256);
	if(cudaHostAlloc((void **)&S.done_h, cap * sizeof(int), cudaHostAllocMapped) != cudaSuccess ||
		cudaHostGetDevicePointer((void **)&S.done_d, S.done_h, 0) != cudaSuccess) {
		cudaGetLastError();
		if(S.done_h) cudaFreeHost(S.done_h);
		S.done_h = nullptr;
		S.done_d = nullptr;
		return false;
	}
	S.done_cap = cap;
	return true;
}

bool run_batch_plain(const std::vector<iw_context *> &ctxs, const std::vector<Plan *> &plans, std::vector<int> &status,
	double &dev_ms, int lane, const std::function<void(int)> &on_done)
{
	DeviceState &S = state(lane);
	std::lock_guard<std::mutex> lk(S.mu);
	const int n = (int)ctxs.size();
	status.assign(n, 0);
	dev_ms = 0;
	std::string err;
	if(!ensure_init(S, err)) {
		for(int i = 0; i < n; i++) { iw_set_error(ctxs[i], err.c_str()); status[i] = -1; }
		return false;
	}
	std::vector<Job> jobs(n);
	std::vector<std::vector<Fixup>> fixes(n);
	std::vector<int> all(n), sel;
	for(int i = 0; i < n; i++) all[i] = i;
	{
		std::vector<char> ok;
		make_jobs(ctxs, plans, all, S, fixes, jobs, ok);
		for(int i = 0; i < n; i++) {
			if(!ok[i]) { status[i] = -1; continue; }
			sel.push_back(i);
		}
	}
	if(sel.empty()) return true;
	const int upmode = upload_mode(ctxs[sel[0]], S, false, true);
	const bool zc = upmode == UP_ZERO;
	size_t top = 0;
	auto take = [&](size_t bytes) { size_t at = (top + 255) & ~(size_t)255; top = at + bytes; return at; };
	const size_t o_par = take(S.staging.size());
	std::vector<size_t> o_in(n, 0), o_mid(n, 0), o_out(n, 0), o_scan(n, 0), o_err(n, 0), in_bytes(n, 0), out_bytes(n, 0);
	for(int i : sel) {
		const Plan &P = *plans[i];
		in_bytes[i] = plan_in_bpr(P) * (size_t)(P.orient >= 4 ? P.img1_w : P.img1_h);
		out_bytes[i] = P.out_bpr * (size_t)P.out_h;
		if(!zc) o_in[i] = take(in_bytes[i] ? in_bytes[i] : 16);
		o_mid[i] = take((size_t)P.mid_n * jobs[i].interm_plane * sizeof(float));
		if(!zc) o_out[i] = take(out_bytes[i]);
		if(jobs[i].any_scan) {
			o_scan[i] = take((size_t)P.out_n * P.out_w * P.out_h * sizeof(double));
			o_err[i] = take((size_t)P.out_n * 5 * P.out_w * sizeof(double));
		}
	}
	if(!S.batch_io.ensure(top)) {
		for(int i : sel) { iw_set_error(ctxs[i], "Out of GPU memory (batch)"); status[i] = -1; }
		return false;
	}
	uint8_t *base = (uint8_t *)S.batch_io.p;
	std::vector<int> run;
	for(int i : sel) {
		iw_context *ctx = ctxs[i];
		const Plan &P = *plans[i];
		Job &J = jobs[i];
		for(const Fixup &f : fixes[i]) *f.slot = base + o_par + f.off;
		ctx->img2.bpr = P.out_bpr;
		ctx->img2.pixels = (iw_byte *)iw_malloc_large(ctx, P.out_bpr, P.out_h);
		if(!ctx->img2.pixels) { status[i] = -1; continue; }
		J.in = zc ? (const uint8_t *)plan_input(ctx, P) : base + o_in[i];
		J.interm = (float *)(base + o_mid[i]);
		J.out = zc ? (uint8_t *)ctx->img2.pixels : base + o_out[i];
		if(J.any_scan) {
			J.scanbuf = (double *)(base + o_scan[i]);
			J.errbuf = (double *)(base + o_err[i]);
		}
		run.push_back(i);
	}
	if(run.empty()) return true;
	const int m = (int)run.size();
	// per-image completion: a scan lane with a caller that takes images one by one
	const bool per_image = on_done && S.lane != 0 && ensure_done_flags(S, m);
	if(per_image) memset(S.done_h, 0, m * sizeof(int));
	// job array and block tables
	std::vector<Job> djobs(m);
	std::vector<int> sv(m), sh(m);
	long long bv = 0, bh = 0;
	int maxch = 1;
	for(int k = 0; k < m; k++) {
		const Job &J = jobs[run[k]];
		djobs[k] = J;
		djobs[k].done_flag = per_image ? S.done_d + k : nullptr;
		sv[k] = (int)bv;
		sh[k] = (int)bh;
		bv += (long long)((J.mid_w + 127) / 128) * J.mid_h;
		bh += (long long)((J.out_w + 127) / 128) * J.out_h;
		maxch = std::max(maxch, J.out_n);
	}
	auto fail_all = [&](const char *msg) {
		for(int i : run) { iw_set_error(ctxs[i], msg); status[i] = -1; }
		return false;
	};
	if(bv > 0x7fffffffLL || bh > 0x7fffffffLL) return fail_all("batch: too many blocks in one launch");
	std::vector<uint8_t> tab;
	auto add = [&](const void *p, size_t bytes) {
		size_t at = (tab.size() + 255) & ~(size_t)255;
		tab.resize(at + bytes);
		if(bytes) memcpy(tab.data() + at, p, bytes);
		return at;
	};
	const size_t o_jobs = add(djobs.data(), djobs.size() * sizeof(Job));
	const size_t o_sv = add(sv.data(), sv.size() * sizeof(int)), o_sh = add(sh.data(), sh.size() * sizeof(int));
	if(!S.batch_tab.ensure(tab.size())) return fail_all("Out of GPU memory (batch tables)");
	uint8_t *tbase = (uint8_t *)S.batch_tab.p;
	const Job *dj = (const Job *)(tbase + o_jobs);
	const int *dsv = (const int *)(tbase + o_sv), *dsh = (const int *)(tbase + o_sh);

	cudaStream_t st = S.stream;
	cudaEvent_t e0, e1;
	cudaEventCreate(&e0);
	cudaEventCreate(&e1);
	cudaMemcpyAsync(base + o_par, S.staging.data(), S.staging.size(), cudaMemcpyHostToDevice, st);
	cudaMemcpyAsync(tbase, tab.data(), tab.size(), cudaMemcpyHostToDevice, st);
	std::vector<Xfer> xin, xout;
	for(int i : run) {
		xin.push_back({base + o_in[i], (uint8_t *)plan_input(ctxs[i], *plans[i]), in_bytes[i]});
		xout.push_back({base + o_out[i], (uint8_t *)ctxs[i]->img2.pixels, out_bytes[i]});
	}
	if(upmode == UP_COPY)
		for(const Xfer &x : xin) cudaMemcpyAsync(x.dev, x.host, x.n, cudaMemcpyHostToDevice, st);
	if(upmode == UP_STAGE && !stage_h2d(S.stager, st, xin)) return fail_all("Out of pinned host memory");
	cudaEventRecord(e0, st);
	// lane 0 takes the whole GPU; the scan lanes' passes run on at most four
	// blocks per SM, so that lane 0's batches find room beside them
	int sms = 152;
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, S.device);
	const long long cap = S.lane == 0 ? 0x7fffffffLL : 4LL * sms;
	const int nv = (int)bv, nh = (int)bh;
	if(bv > 0) kb_vpass_exact<<<(unsigned)std::min<long long>(bv, cap), 128, 0, st>>>(dj, dsv, m, nv);
	if(bh > 0) kb_hpass_exact<<<(unsigned)std::min<long long>(bh, cap), 128, 0, st>>>(dj, dsh, m, nh);
	kb_scan<<<std::min(m, sms), 32 * maxch, 0, st>>>(dj, m);
	if(bh > 0 && !per_image) kb_finalize<<<(unsigned)std::min<long long>(bh, cap), 128, 0, st>>>(dj, dsh, m, nh);
	cudaEventRecord(e1, st);
	std::vector<char> reported(m, 0);
	if(per_image) {
		// take each image as its scan block reports it: download on the
		// lane's second stream, then hand it to the caller
		const volatile int *flags = S.done_h;
		int left = m;
		for(;;) {
			bool any = false;
			for(int k = 0; k < m; k++) {
				if(reported[k] || !flags[k]) continue;
				const int i = run[k];
				iw_context *ctx = ctxs[i];
				reported[k] = 1;
				left--;
				any = true;
				if(!zc) {
					cudaMemcpyAsync(ctx->img2.pixels, base + o_out[i], out_bytes[i], cudaMemcpyDeviceToHost, S.dl_stream);
					const cudaError_t de = cudaStreamSynchronize(S.dl_stream);
					if(de != cudaSuccess) {
						iw_set_error(ctx, (std::string("CUDA error: ") + cudaGetErrorString(de)).c_str());
						status[i] = -1;
						continue;
					}
				}
				ctx->stats.form = 0;
				ctx->stats.zero_copy = zc;
				ctx->stats.kernels = 3;
				ctx->stats.ms_device = 0;   // the batch's device time is not known yet
				ctx->stats.flagged = 0;
				status[i] = 1;
				on_done(i);
			}
			if(left == 0) break;
			if(cudaStreamQuery(st) != cudaErrorNotReady) {   // the kernels ended: a last look, then stop
				bool late = false;
				for(int k = 0; k < m; k++) if(!reported[k] && flags[k]) late = true;
				if(!late) break;
				continue;
			}
			if(!any) std::this_thread::sleep_for(std::chrono::microseconds(200));
		}
	}
	else {
		// A scan lane queues its downloads only once its kernels are done: a
		// copy queued behind a long scan can hold up other streams' copies.
		if(S.lane != 0) wait_event(e1, true);
		if(upmode == UP_COPY)
			for(const Xfer &x : xout) cudaMemcpyAsync(x.host, x.dev, x.n, cudaMemcpyDeviceToHost, st);
		if(upmode == UP_STAGE) stage_d2h(S.stager, st, xout);
	}
	cudaError_t ce = wait_stream(st, S.lane != 0);
	if(ce == cudaSuccess) ce = cudaGetLastError();
	float ms = 0;
	if(ce == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	if(ce == cudaSuccess && per_image)
		for(int k = 0; k < m; k++) if(!reported[k]) ce = cudaErrorUnknown;   // a block ended without its flag
	if(ce != cudaSuccess) {
		std::string msg = std::string("CUDA error: ") + cudaGetErrorString(ce);
		for(int k = 0; k < m; k++) {
			if(reported[k]) continue;   // already handed over, its bytes complete
			iw_set_error(ctxs[run[k]], msg.c_str());
			status[run[k]] = -1;
		}
		return false;
	}
	dev_ms = ms;
	if(per_image) return true;   // every image was handed over as it finished
	for(int i : run) {
		iw_context *ctx = ctxs[i];
		ctx->stats.form = 0;
		ctx->stats.zero_copy = zc;
		ctx->stats.kernels = 4;
		ctx->stats.ms_device = ms;
		ctx->stats.flagged = 0;
		status[i] = 1;
	}
	return true;
}

// The plain form's launches; 'mark' is called after each launch group.
template<class Mark>
int plain_launch(cudaStream_t st, const Plan &P, const Job &J, Mark mark)
{
	int launches = 0;
	dim3 bv(128), gv((J.mid_w + 127) / 128, J.mid_h);
	k_vpass_exact<<<gv, bv, 0, st>>>(J);
	mark();
	dim3 bh(128), gh((J.out_w + 127) / 128, J.out_h);
	k_hpass_exact<<<gh, bh, 0, st>>>(J);
	mark();
	launches += 2;
	if(J.any_scan) {
		k_scan<<<1, 32 * P.out_n, 0, st>>>(J);
		launches++;
		if(J.negate || J.blacken) { k_finalize<<<gh, bh, 0, st>>>(J); launches++; }
		mark();
	}
	return launches;
}

}  // namespace iwg

// ===== additive ABI (include/imagew_gb300.h) ================================

extern "C" int iwg_get_stats(struct iw_context *ctx, struct iwg_stats *out)
{
	out->ms_total = ctx->stats.ms_total;
	out->ms_device = ctx->stats.ms_device;
	for(int k = 0; k < 4; k++) out->ms_part[k] = ctx->stats.ms_part[k];
	out->flagged = ctx->stats.flagged;
	out->form = ctx->stats.form;
	out->kernels = ctx->stats.kernels;
	out->zero_copy = ctx->stats.zero_copy;
	out->flagged_exact = ctx->stats.flagged_exact;
	out->vertical_tensor = ctx->stats.vertical_tensor;
	out->graph = ctx->stats.graph;
	out->fused = ctx->stats.fused;
	for(int k = 0; k < 6; k++) out->ms_phase[k] = ctx->stats.ms_phase[k];
	return 1;
}

extern "C" long long iwg_debug_values(struct iw_context *ctx, int which, double *out, long long max_count, int *dims)
{
	const std::vector<double> *v = which == 0 ? &ctx->dbg.interm : which == 1 ? &ctx->dbg.value :
		which == 2 ? &ctx->dbg.bound : nullptr;
	if(!v) return -1;
	if(dims)
		for(int k = 0; k < 3; k++) dims[k] = ctx->dbg.dims[(which == 0 ? 0 : 3) + k];
	const long long n = (long long)v->size();
	if(out) memcpy(out, v->data(), (size_t)std::min(n, max_count < 0 ? 0 : max_count) * sizeof(double));
	return n;
}

extern "C" int iwg_device_info(char *buf, int buflen)
{
	int dev = 0, n = 0;
	if(buflen < 1) return 0;
	buf[0] = '\0';
	if(cudaGetDeviceCount(&n) != cudaSuccess || n < 1) return 0;
	cudaGetDevice(&dev);
	cudaDeviceProp p;
	if(cudaGetDeviceProperties(&p, dev) != cudaSuccess) return 0;
	int pageable = 0, hostpt = 0;
	cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev);
	cudaDeviceGetAttribute(&hostpt, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev);
	snprintf(buf, buflen, "%s sm_%d%d, %d SMs, %.1f GiB, pageable host memory access %d (host page tables %d)",
		p.name, p.major, p.minor, p.multiProcessorCount, p.totalGlobalMem / 1073741824.0, pageable, hostpt);
	return 1;
}
