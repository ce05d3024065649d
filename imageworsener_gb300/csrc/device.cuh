// device.cuh -- device-side job description and the exact (FP64) sample
// arithmetic shared by all kernels.
//
// Exactness rules: every double operation below is a separately rounded IEEE
// operation (__dadd_rn, __dmul_rn, ...), in the reference's order; the file is
// also compiled with -fmad=false so no multiply-add is ever fused.  Values that
// need a transcendental function come from host-built tables.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace iwg {
namespace dev {

constexpr int kMaxCh = 4;

struct DWeights {
	int kind;              // 0: weighted sum, 1: copy
	int n_in, n_out;
	int max_taps;
	double edge_value;
	const int *off;        // n_out + 1
	const int *src;        // -1: virtual pixel / no source
	const double *w;
	const float *wf;
	const int *pos;        // virtual input position per tap (streaming kernels)
};

struct DQuant {
	int float_out, use_nc, dfam, dsub, maxcc, P;
	const double *U;       // P+2
	const double *X;       // P+1
	const int *code;       // P+2
	const double *rev;     // maxcc+1
	const double *nc;      // 255
	const long long *rec;  // error diffusion: 8 words per bracket (P+1)
	const float *lut;      // or null: kBracketLutCells search start points for U[1..P]
	                       // (cell c: the count of float-rounded edges <= c / kBracketLutCells)
};

constexpr int kBracketLutCells = 1024;

struct DMid {
	int ctype, in_ch, to_gray, out_ch, unassoc, wh, wv;
	double bk_early;
	const double *tab[3];  // decode tables of the input channel(s) read
};

struct DOut {
	int ctype, maxcc, scan;
	double bk1, bk2;
	DQuant q;
};

struct Job {
	// input image (device copy of the caller's bytes)
	const uint8_t *in;
	unsigned long long in_bpr;
	int in_depth, in_float, in_nphys, orient, img1_w, img1_h;   // in_float: 1 float samples, 2 linearised doubles
	int crop_x, crop_y, crop_w, crop_h;
	int in_alpha;                 // logical alpha channel
	const double *alpha_tab;      // alpha code -> value, null if the alpha channel is virtual

	// intermediate: [m][row][x] float planes
	int mid_n, mid_alpha;
	DMid mid[kMaxCh];
	int order[kMaxCh];            // processing order: alpha first
	float *interm;
	unsigned long long interm_plane;
	int mid_w, mid_h;

	// output
	uint8_t *out;
	unsigned long long out_bpr;
	int out_w, out_h, out_n, out_depth, out_float;
	DOut outc[kMaxCh];
	int any_scan;
	volatile int *done_flag;      // batched scans: set in mapped host memory once the image's output is final (null: none)
	double *scanbuf;              // pre-quantisation values of dithered channels that scan serially
	double *errbuf;               // error rows for error diffusion: [channel][3][out_w]

	DWeights wh[kMaxCh], wv[kMaxCh];

	// background, gray, misc
	int apply_bk, bk_late, bk_early, bk_checker, bk_trns;
	double bk1_alpha, bk2_alpha;
	int check_size, check_ox, check_oy;
	int gsf;
	double gsw[3];
	int intclamp, negate, blacken;
	int seed;

	// double-float copies for the fast form's re-evaluation tier (null
	// otherwise): decode table per intermediate channel, alpha table, and the
	// weights of weight set 0 of each dimension, indexed like their CSR lists
	const float2 *df_tab[kMaxCh];
	const float2 *df_atab;
	const float2 *df_wv, *df_wh;

	// debug readback (null normally): the value each output sample is
	// quantised from, [out_n][out_h][out_w] (plain form)
	double *dbg;
};

// ---- double-float ("df") arithmetic ----
// A value hi + lo of two floats with |lo| <= ulp(hi)/2: 48 significant bits
// on the FP32 pipe.  Error-free transformations (Knuth's TwoSum, Dekker's
// Fast2Sum, the FMA product error) and the double-word algorithms of Joldes,
// Muller and Popescu ("Tight and rigorous error bounds for basic building
// blocks of double-word arithmetic", ACM TOMS 44(2), 2017), whose relative
// error bounds with u = 2^-24 are: DW+DW (accurate) 3u^2/(1-4u), DW*DW 5u^2,
// DW/FP 3.5u^2.  Every operation is a separately rounded IEEE FP32 operation.
struct dfl { float hi, lo; };

__device__ __forceinline__ dfl df_two_sum(float a, float b)
{
	const float s = __fadd_rn(a, b);
	const float bb = __fsub_rn(s, a);
	return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

__device__ __forceinline__ dfl df_fast_two_sum(float a, float b)   // |a| >= |b| or a == 0
{
	const float s = __fadd_rn(a, b);
	return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ dfl df_add(dfl x, dfl y)
{
	const dfl s = df_two_sum(x.hi, y.hi), t = df_two_sum(x.lo, y.lo);
	const dfl v = df_fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
	return df_fast_two_sum(v.hi, __fadd_rn(t.lo, v.lo));
}

// x + y with the error bounded by the operands' magnitudes rather than the
// result's: TwoSum of the high parts, the low parts added in FP32, one
// renormalisation.  |error| <= 2.01 u^2 (|x| + |y|) (one rounding of the
// low parts' sum, below u^2 (|x| + |y|), and one of its sum with the
// TwoSum error, below u^2 |x.hi + y.hi| (1 + u)^2).  Where a bound is
// stated in the sum of the terms' magnitudes -- a running sum of n terms
// gains at most 2.01 n u^2 of it -- this is as good as the accurate form
// in far fewer operations.
__device__ __forceinline__ dfl df_add_sloppy(dfl x, dfl y)
{
	const dfl s = df_two_sum(x.hi, y.hi);
	return df_fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo)));
}

// A float times a double-float: the exact product of the high parts
// (TwoProd by FMA) plus the low part's product; error below 2 u^2 |x y|.
__device__ __forceinline__ dfl df_mul_f(float x, dfl y)
{
	const float p = __fmul_rn(x, y.hi);
	const float e = __fmaf_rn(x, y.hi, -p);
	return df_fast_two_sum(p, __fmaf_rn(x, y.lo, e));
}

__device__ __forceinline__ dfl df_mul(dfl x, dfl y)
{
	const float ch = __fmul_rn(x.hi, y.hi);
	const float cl1 = __fmaf_rn(x.hi, y.hi, -ch);
	const float tl0 = __fmul_rn(x.lo, y.lo);
	const float tl1 = __fmaf_rn(x.hi, y.lo, tl0);
	const float cl2 = __fmaf_rn(x.lo, y.hi, tl1);
	return df_fast_two_sum(ch, __fadd_rn(cl1, cl2));
}

__device__ __forceinline__ dfl df_div_f(dfl x, float y)
{
	const float th = __fdiv_rn(x.hi, y);
	const float ph = __fmul_rn(th, y);
	const float pl = __fmaf_rn(th, y, -ph);
	const float dh = __fsub_rn(x.hi, ph);
	const float dt = __fsub_rn(dh, pl);
	const float d = __fadd_rn(dt, x.lo);
	return df_fast_two_sum(th, __fdiv_rn(d, y));
}

__device__ __forceinline__ dfl df_of(float2 v) { return {v.x, v.y}; }

// ---- exact double helpers ----
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// Logical (crop-relative) coordinates -> stored pixel (src/imagew-main.c:189-234).
__device__ __forceinline__ void phys_xy(const Job &J, int x, int y, int &px, int &py)
{
	int lx = J.crop_x + x, ly = J.crop_y + y;
	switch(J.orient) {
	case 0: px = lx; py = ly; break;
	case 1: px = J.img1_w - 1 - lx; py = ly; break;
	case 2: px = lx; py = J.img1_h - 1 - ly; break;
	case 3: px = J.img1_w - 1 - lx; py = J.img1_h - 1 - ly; break;
	case 4: px = ly; py = lx; break;
	case 5: px = ly; py = J.img1_w - 1 - lx; break;
	case 6: px = J.img1_h - 1 - ly; py = lx; break;
	case 7: px = J.img1_h - 1 - ly; py = J.img1_w - 1 - lx; break;
	default: px = 0; py = 0; break;
	}
}

__device__ __forceinline__ unsigned int raw_code(const Job &J, int px, int py, int ch)
{
	const uint8_t *row = J.in + (unsigned long long)py * J.in_bpr;
	switch(J.in_depth) {
	case 8: return row[J.in_nphys * px + ch];
	case 16: {
		const uint8_t *p = row + (size_t)(J.in_nphys * px + ch) * 2;
		return ((unsigned int)p[0] << 8) | p[1];
	}
	case 4: return (px & 1) ? (row[px / 2] & 0x0f) : (row[px / 2] >> 4);
	case 2: return (row[px / 4] >> ((3 - px % 4) * 2)) & 0x03;
	case 1: return (row[px / 8] & (1 << (7 - px % 8))) ? 1u : 0u;
	}
	return 0;
}

// Value of input channel 'ch' at logical (x,y) through table 'tab'
// (get_raw_sample + transfer function, src/imagew-main.c:257-383).
__device__ __forceinline__ double in_value(const Job &J, int x, int y, int ch, const double *tab)
{
	if(ch >= J.in_nphys) return 1.0;   // virtual alpha: opaque
	int px, py;
	phys_xy(J, x, y, px, py);
	if(J.in_float == 2) {   // float input linearised on the host: one double per sample
		const uint8_t *p = J.in + (unsigned long long)py * J.in_bpr + (size_t)(J.in_nphys * px + ch) * 8;
		double d;
		memcpy(&d, p, 8);
		return d;
	}
	if(J.in_float) {
		const uint8_t *p = J.in + (unsigned long long)py * J.in_bpr + (size_t)(J.in_nphys * px + ch) * 4;
		float f;
		memcpy(&f, p, 4);
		return (double)f;
	}
	return tab[raw_code(J, px, py, ch)];
}

__device__ __forceinline__ double gray_of(const Job &J, double r, double g, double b)
{
	if(J.gsf == IW_GSF_WEIGHTED) return dadd(dadd(dmul(J.gsw[0], r), dmul(J.gsw[1], g)), dmul(J.gsw[2], b));
	if(J.gsf == IW_GSF_ORDERBYVALUE) {
		double hi, mid, lo;
		if(g <= r) { hi = r; mid = g; } else { hi = g; mid = r; }
		if(b <= mid) lo = b;
		else {
			lo = mid;
			if(b <= hi) mid = b;
			else { mid = hi; hi = b; }
		}
		return dadd(dadd(dmul(J.gsw[0], hi), dmul(J.gsw[1], mid)), dmul(J.gsw[2], lo));
	}
	return 0.0;
}

// Linear-light input value of intermediate channel m at (x,y), premultiplied
// by alpha or composited over an early background (src/imagew-main.c:873-894).
__device__ __forceinline__ double decode_exact(const Job &J, const DMid &m, int x, int y)
{
	double s;
	if(m.to_gray) {
		double r = in_value(J, x, y, m.in_ch, m.tab[0]);
		double g = in_value(J, x, y, m.in_ch + 1, m.tab[1]);
		double b = in_value(J, x, y, m.in_ch + 2, m.tab[2]);
		s = gray_of(J, r, g, b);
	}
	else s = in_value(J, x, y, m.in_ch, m.tab[0]);
	if(m.unassoc) {
		s = dmul(s, in_value(J, x, y, J.in_alpha, J.alpha_tab));
	}
	else if(J.bk_early) {
		double a = in_value(J, x, y, J.in_alpha, J.alpha_tab);
		s = dadd(dmul(a, s), dmul(dsub(1.0, a), m.bk_early));
	}
	return s;
}

// Ordered-dither threshold ranks; threshold = (rank + 0.5) / 64 (8x8
// dispersed and "halftone" patterns of src/imagew-main.c:461-483).  In global
// memory (read through L1): lanes of a warp index different entries.
static __device__ const unsigned char kDitherRank[2][64] = {
	{0,48,12,60, 3,51,15,63, 32,16,44,28,35,19,47,31,  8,56, 4,52,11,59, 7,55, 40,24,36,20,43,27,39,23,
	 2,50,14,62, 1,49,13,61, 34,18,46,30,33,17,45,29, 10,58, 6,54, 9,57, 5,53, 42,26,38,22,41,25,37,21},
	{3, 9,17,27,25,15, 7, 1, 11,29,37,45,43,35,23, 5, 19,39,51,57,55,49,33,13, 31,47,59,63,61,53,41,21,
	 30,46,58,62,60,52,40,20, 18,38,50,56,54,48,32,12, 10,28,36,44,42,34,22, 4,  2, 8,16,26,24,14, 6, 0}};

__device__ __forceinline__ int dither_rank(int sub, int x, int y)
{
	return kDitherRank[sub ? 1 : 0][(x % 8) + 8 * (y % 8)];
}

// Number of entries of the ascending table t[0..n-1] that are <= v.
__device__ __forceinline__ int count_le(const double *t, int n, double v)
{
	int lo = 0, hi = n;
	while(lo < hi) {
		int mid = (lo + hi) >> 1;
		if(t[mid] <= v) lo = mid + 1; else hi = mid;
	}
	return lo;
}

struct Bracket {
	int lo, hi, exact;
	double d_lo, d_hi;
};

// The two codes around v and their distances in linear light
// (get_nearest_valid_colors, src/imagew-main.c:570-629), via the host tables.
__device__ __forceinline__ Bracket bracket_exact(const DQuant &q, double v)
{
	Bracket b;
	int k = count_le(q.U + 1, q.P, v);          // floor(from_linear(v) * P), clamped
	b.exact = (k == q.P) || (v < q.X[k]);
	b.lo = q.code[k];
	b.hi = q.code[k + 1];
	b.d_lo = b.d_hi = 0.0;
	if(!b.exact) {
		b.d_lo = dsub(v, q.rev[b.lo]);
		b.d_hi = dsub(q.rev[b.hi], v);
	}
	return b;
}

// Output code for one sample with no dither, a nearest-colour table, or
// ordered dither (put_sample_convert_from_linear, src/imagew-main.c:669-765).
__device__ __forceinline__ int quantize_exact(const DQuant &q, double v, int x, int y)
{
	if(v < 0.0) v = 0.0;
	if(v > 1.0) v = 1.0;
	if(v != v) return 0;   // NaN: both candidate codes convert to 0
	if(q.use_nc) return count_le(q.nc, 255, v);
	Bracket b = bracket_exact(q, v);
	if(b.exact) return b.lo;
	if(q.dfam == IW_DITHERFAMILY_ORDERED) {
		double f = ddiv(b.d_lo, dadd(b.d_lo, b.d_hi));
		double thr = ddiv((double)dither_rank(q.dsub, x, y) + 0.5, 64.0);
		return f >= thr ? b.hi : b.lo;
	}
	return b.d_hi <= b.d_lo ? b.hi : b.lo;
}

__device__ __forceinline__ void store_code(const Job &J, int ch, int x, int y, unsigned int code)
{
	uint8_t *row = J.out + (unsigned long long)y * J.out_bpr;
	if(J.out_depth == 8) row[J.out_n * x + ch] = (uint8_t)code;
	else {
		uint8_t *p = row + (size_t)(J.out_n * x + ch) * 2;
		p[0] = (uint8_t)(code >> 8);
		p[1] = (uint8_t)(code & 0xff);
	}
}

__device__ __forceinline__ unsigned int load_code(const Job &J, int ch, int x, int y)
{
	const uint8_t *row = J.out + (unsigned long long)y * J.out_bpr;
	if(J.out_depth == 8) return row[J.out_n * x + ch];
	const uint8_t *p = row + (size_t)(J.out_n * x + ch) * 2;
	return ((unsigned int)p[0] << 8) | p[1];
}

__device__ __forceinline__ void store_float(const Job &J, int ch, int x, int y, float f)
{
	uint8_t *p = J.out + (unsigned long long)y * J.out_bpr + (size_t)(J.out_n * x + ch) * 4;
	memcpy(p, &f, 4);
}

// Checkerboard cell parity at output (x,y) (src/imagew-main.c:1080-1083).
__device__ __forceinline__ int checker_alt(const Job &J, int x, int y)
{
	if(!J.bk_checker) return 0;
	return (((J.check_ox + x) / J.check_size) % 2) != (((J.check_oy + y) / J.check_size) % 2);
}

}  // namespace dev
}  // namespace iwg
