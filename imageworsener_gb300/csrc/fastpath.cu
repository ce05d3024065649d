// fastpath.cu -- FP32 + guard-band form of the pixel pipeline.
//
// The vertical and horizontal resampling run in FP32.  Every output sample
// carries a rigorous bound E on |v_fp32 - v_ref|, where v_ref is the value the
// reference computes in double precision (with its float intermediate).  The
// quantisation tail then decides the output code for the whole interval
// [v - E, v + E]; if a decision boundary of the reference (a code bracket
// edge, a nearest-colour midpoint, an ordered-dither threshold) lies inside,
// the pixel is flagged and recomputed exactly in FP64 by k_fix_flagged
// (pipeline.cu).  Output bytes therefore equal the plain form's.
//
// Error bound (u = 2^-24, per pass with n taps and weights w):
//   decode   |a' - a| <= e_dec + r_dec * a          (e_dec measured over every code)
//   vertical |I' - I_ref| <= e_dec*W1v + c1 * (|I'| + 2*Wneg_v)
//   horizontal |v' - v_ref| <= K0 + K1 * sum_k |I'_k||w_k|
// with c1 = (r_dec + 2u + gamma_nv + gamma_nv^(fp64)) and K0, K1 assembled on
// the host below; unassociating alpha divides by the float alpha, whose own
// bound is propagated.
#include "iwg_internal.h"
#include "device.cuh"
#include "fastpath.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

namespace iwg {

using namespace dev;

void launch_fix_flagged(cudaStream_t st, const Job &J, const int *count, const int *list);

namespace {

constexpr int kVThreads = 128;
constexpr int kHThreads = 128;
constexpr int kVPxThreads = 128;
constexpr int kMaxPlanes = 4;

struct FPlane {
	int src;          // physical channel, -1: virtual (value 1)
	int table;        // 1: decode through the shared table; 0: code * inv
	int premul;       // multiply by the alpha value
	float inv;        // 1 / maxcc for arithmetic decode
};

struct FTail {        // quantisation of one output channel, float tables
	int P, M, cc, use_nc, dfam, dsub;
	const float *U;   // P+2
	const float *X;   // P+1
	const int *code;  // P+2
	const float *rev; // M+1
	const float *nc;  // 255
};

struct FJob {
	// input
	const uint8_t *in;
	unsigned long long in_bpr;
	int crop_x, crop_y, nphys, depth;
	int alpha_src;    // physical alpha channel, -1 virtual/none
	float alpha_inv;
	int npl;
	FPlane pl[kMaxPlanes];
	int vec;                   // 8 / 4: pixels load as one aligned 8- / 4-byte word; 0: bytes
	const float *dec_tab;      // 8-bit: 256 floats; 16-bit: 4096 (T0, slope) pairs
	int dec_tab_floats;
	// vertical pass
	int mid_w, mid_h;
	float *interm;
	unsigned long long plane;
	// streaming
	int pmin, npos, ns;
	const int2 *pinfo;        // per position: (first row finalised, count)
	const float *sw;          // per position: ns slot weights (padded to 8)
	const int *srcrow;        // per position: input row, -1 virtual
	const int *first_pos, *last_pos;
	int rows_per_band;
	int in_rows;              // crop height: input rows of the vertical pass
	// gather (upscale) vertical pass
	const int *voff, *vsrc;
	const float *vw;
	// horizontal pass
	const int *hoff, *hsrc;
	const float *hw;
	int out_w, out_h, out_n, out_depth;
	uint8_t *out;
	unsigned long long out_bpr;
	// per processing slot k (alpha first), so kernels index these statically
	int mid_n;
	int k_plane[dev::kMaxCh];   // plane holding the channel's intermediate
	int k_out[dev::kMaxCh];     // output channel
	int k_alpha[dev::kMaxCh];   // 1: the alpha channel
	int k_unassoc[dev::kMaxCh]; // 1: colour channel divided by alpha
	int k_maxcc[dev::kMaxCh];   // output max code (negation)
	unsigned int k_bit[dev::kMaxCh];  // bit of the intermediate channel in re-evaluation masks
	int alpha_plane;
	const FTail *tail;         // per output channel (device memory)
	int negate, blacken;
	// error model
	float K0[kMaxPlanes], K1[kMaxPlanes];
	// flags
	int *flag_count;
	int *flag_list;
};

// ---------------------------------------------------------------------------
// decode
// ---------------------------------------------------------------------------

template<int DEPTH>
__device__ __forceinline__ unsigned int fetch_code(const uint8_t *px, int ch)
{
	if(DEPTH == 8) return px[ch];
	return ((unsigned int)px[2 * ch] << 8) | px[2 * ch + 1];
}

template<int DEPTH>
__device__ __forceinline__ float dec_table(const float *tab, unsigned int code)
{
	if(DEPTH == 8) return tab[code];
	float2 t = reinterpret_cast<const float2 *>(tab)[code >> 4];
	return __fmaf_rn((float)(code & 15u), t.y, t.x);
}

template<int NPL, int DEPTH>
__device__ __forceinline__ void decode_pixel(const FJob &F, const float *tab, const uint8_t *px, float *val)
{
	float a = 1.0f;
	if(F.alpha_src >= 0) a = __fmul_rn((float)fetch_code<DEPTH>(px, F.alpha_src), F.alpha_inv);
#pragma unroll
	for(int c = 0; c < NPL; c++) {
		const FPlane &P = F.pl[c];
		float v;
		if(P.src < 0) v = 1.0f;
		else {
			unsigned int code = fetch_code<DEPTH>(px, P.src);
			v = P.table ? dec_table<DEPTH>(tab, code) : __fmul_rn((float)code, P.inv);
		}
		val[c] = P.premul ? __fmul_rn(v, a) : v;
	}
}

// ---------------------------------------------------------------------------
// vertical pass, streaming: each thread owns one column; input rows are read
// once, in order, and accumulated into NS register slots, one per output row
// whose window is open (slot = row mod NS).
// ---------------------------------------------------------------------------
// Raw bytes of one input pixel (at most 8: four 16-bit channels).
struct Raw {
	uint32_t lo, hi;
};

__device__ __forceinline__ Raw load_raw(const FJob &F, const uint8_t *px, int bpp)
{
	Raw r{0u, 0u};
	if(F.vec == 8) {
		uint2 v = __ldg(reinterpret_cast<const uint2 *>(px));
		r.lo = v.x;
		r.hi = v.y;
	}
	else if(F.vec == 4) r.lo = __ldg(reinterpret_cast<const unsigned int *>(px));
	else {
		for(int b = 0; b < bpp; b++) {
			uint32_t byte = __ldg(px + b);
			if(b < 4) r.lo |= byte << (8 * b);
			else r.hi |= byte << (8 * (b - 4));
		}
	}
	return r;
}

__device__ __forceinline__ unsigned int raw_byte(const Raw &r, int b)
{
	return ((b < 4 ? (r.lo >> (8 * b)) : (r.hi >> (8 * (b - 4))))) & 0xffu;
}

template<int DEPTH>
__device__ __forceinline__ unsigned int raw_code(const Raw &r, int ch)
{
	if(DEPTH == 8) return raw_byte(r, ch);
	return (raw_byte(r, 2 * ch) << 8) | raw_byte(r, 2 * ch + 1);   // big-endian samples
}

template<int NPL, int DEPTH>
__device__ __forceinline__ void decode_raw(const FJob &F, const float *tab, const Raw &px, float *val)
{
	float a = 1.0f;
	if(F.alpha_src >= 0) a = __fmul_rn((float)raw_code<DEPTH>(px, F.alpha_src), F.alpha_inv);
#pragma unroll
	for(int c = 0; c < NPL; c++) {
		const FPlane &P = F.pl[c];
		float v;
		if(P.src < 0) v = 1.0f;
		else {
			unsigned int code = raw_code<DEPTH>(px, P.src);
			v = P.table ? dec_table<DEPTH>(tab, code) : __fmul_rn((float)code, P.inv);
		}
		val[c] = P.premul ? __fmul_rn(v, a) : v;
	}
}

// Vertical pass, streaming.  Each thread owns one column and walks the input
// rows of its band once, in order, keeping PF rows of loads in flight; every
// row is decoded once and accumulated into NS register slots, one per output
// row whose window is open (slot = row mod NS).  A slot is stored and cleared
// when its row's window closes.
template<int NS, int NPL, int DEPTH>
__global__ void __launch_bounds__(kVThreads) k_vstream(FJob F)
{
	constexpr int PF = 8;
	extern __shared__ float s_tab[];
	for(int k = threadIdx.x; k < F.dec_tab_floats; k += blockDim.x) s_tab[k] = F.dec_tab[k];
	__syncthreads();

	const int x = blockIdx.x * blockDim.x + threadIdx.x;
	const bool active = x < F.mid_w;
	const int jb = blockIdx.y * F.rows_per_band;
	const int je = min(jb + F.rows_per_band, F.mid_h);
	if(jb >= je) return;
	const int p0 = F.first_pos[jb], p1 = F.last_pos[je - 1];
	const int bpp = F.nphys * (DEPTH / 8);
	const uint8_t *colbase = F.in + (size_t)(F.crop_x + (active ? x : 0)) * bpp +
		(unsigned long long)F.crop_y * F.in_bpr;

	float acc[NS][NPL];
#pragma unroll
	for(int s = 0; s < NS; s++)
#pragma unroll
		for(int c = 0; c < NPL; c++) acc[s][c] = 0.0f;

	Raw buf[PF];
	int rows[PF];
#pragma unroll
	for(int u = 0; u < PF; u++) {
		const int p = p0 + u;
		const int r = p <= p1 ? __ldg(F.srcrow + (p - F.pmin)) : -1;
		rows[u] = r;
		buf[u] = (r >= 0 && active) ? load_raw(F, colbase + (unsigned long long)r * F.in_bpr, bpp) : Raw{0u, 0u};
	}

	for(int p = p0; p <= p1; p += PF) {
#pragma unroll
		for(int u = 0; u < PF; u++) {
			const int pp = p + u;
			if(pp > p1) break;
			const Raw cur = buf[u];
			const int row = rows[u];
			{   // refill this slot of the ring with the row PF positions ahead
				const int pn = pp + PF;
				const int r = pn <= p1 ? __ldg(F.srcrow + (pn - F.pmin)) : -1;
				rows[u] = r;
				buf[u] = (r >= 0 && active) ? load_raw(F, colbase + (unsigned long long)r * F.in_bpr, bpp) : Raw{0u, 0u};
			}
			const int q = pp - F.pmin;
			float val[NPL];
			if(row >= 0 && active) decode_raw<NPL, DEPTH>(F, s_tab, cur, val);
			else {
#pragma unroll
				for(int c = 0; c < NPL; c++) val[c] = 0.0f;   // transparent edge: value 0
			}
			const float4 *w4 = reinterpret_cast<const float4 *>(F.sw + (size_t)q * 8);
			const float4 wa = __ldg(w4), wb = __ldg(w4 + 1);
			const float ws[8] = {wa.x, wa.y, wa.z, wa.w, wb.x, wb.y, wb.z, wb.w};
#pragma unroll
			for(int s = 0; s < NS; s++)
#pragma unroll
				for(int c = 0; c < NPL; c++) acc[s][c] = __fmaf_rn(val[c], ws[s], acc[s][c]);
			const int2 fin = __ldg(F.pinfo + q);
			for(int k = 0; k < fin.y; k++) {
				const int j = fin.x + k;
				const int sj = j % NS;
#pragma unroll
				for(int s = 0; s < NS; s++) {
					if(s == sj) {
						if(active && j >= jb && j < je) {
#pragma unroll
							for(int c = 0; c < NPL; c++)
								F.interm[(unsigned long long)c * F.plane + (unsigned long long)j * F.mid_w + x] = acc[s][c];
						}
#pragma unroll
						for(int c = 0; c < NPL; c++) acc[s][c] = 0.0f;
					}
				}
			}
		}
	}
}

// Exact float of a small unsigned integer (< 2^23) without an I2F: the code
// is placed in the mantissa of 2^23 and 2^23 is subtracted.
__device__ __forceinline__ float u2f(unsigned int v)
{
	return __fsub_rn(__uint_as_float(0x4b000000u | v), 8388608.0f);
}


// Vertical pass, streaming, PX pixels per thread.  Same scheme as
// k_vstream, arranged for memory-level parallelism and few instructions
// per sample:
//   * each thread reads PX adjacent pixels of a row as one aligned 4/8/16-byte
//     word group, and keeps PF rows of those loads in flight;
//   * a row's address is computed from its position (positions map to rows by
//     clamping, which the host checked for this weight set), so no load waits
//     on another load;
//   * the band's schedule (slot weights, rows finished per position) is staged
//     in shared memory once per block.
template<int NS, int NCH, bool ALPHA, int DEPTH, int PX>
__global__ void __launch_bounds__(kVPxThreads) k_vstream_px(FJob F)
{
	constexpr int PF = 8;
	constexpr int BPP = NCH * (DEPTH / 8);
	constexpr int NW = PX * BPP / 4;              // 32-bit words per thread per row
	static_assert(PX * BPP % 4 == 0, "thread group must be whole words");
	extern __shared__ float s_dyn[];
	float *s_tab = s_dyn;
	const int jb = blockIdx.y * F.rows_per_band;
	const int je = min(jb + F.rows_per_band, F.mid_h);
	if(jb >= je) return;
	const int p0 = F.first_pos[jb], p1 = F.last_pos[je - 1];
	const int nq = p1 - p0 + 1;
	float *s_w = s_dyn + F.dec_tab_floats;         // nq * NS
	int2 *s_fin = reinterpret_cast<int2 *>(s_w + (size_t)nq * NS);
	for(int k = threadIdx.x; k < F.dec_tab_floats; k += blockDim.x) s_tab[k] = F.dec_tab[k];
	for(int k = threadIdx.x; k < nq * NS; k += blockDim.x) {
		const int q = k / NS, sl = k - q * NS;
		s_w[k] = F.sw[(size_t)(p0 - F.pmin + q) * 8 + sl];
	}
	for(int k = threadIdx.x; k < nq; k += blockDim.x) s_fin[k] = F.pinfo[p0 - F.pmin + k];
	__syncthreads();

	const int x0 = (blockIdx.x * blockDim.x + threadIdx.x) * PX;
	if(x0 >= F.mid_w) return;
	const bool full = x0 + PX <= F.mid_w;
	const int valid_bytes = (F.mid_w - x0) * BPP;
	const uint8_t *colbase = F.in + (size_t)(F.crop_x + x0) * BPP + (unsigned long long)F.crop_y * F.in_bpr;
	const int last_row = F.in_rows - 1;
	const float ainv = F.alpha_inv;

	float acc[NS][PX][NCH];
#pragma unroll
	for(int s = 0; s < NS; s++)
#pragma unroll
		for(int px = 0; px < PX; px++)
#pragma unroll
			for(int c = 0; c < NCH; c++) acc[s][px][c] = 0.0f;

	auto load_row = [&](int p, uint32_t *w) {
		const int row = min(max(p, 0), last_row);
		const uint8_t *a = colbase + (unsigned long long)row * F.in_bpr;
		if(full) {
			if(NW % 4 == 0) {
#pragma unroll
				for(int k = 0; k < NW; k += 4) {
					const uint4 v = __ldcs(reinterpret_cast<const uint4 *>(a) + k / 4);
					w[k] = v.x; w[k + 1] = v.y; w[k + 2] = v.z; w[k + 3] = v.w;
				}
			}
			else if(NW % 2 == 0) {
#pragma unroll
				for(int k = 0; k < NW; k += 2) {
					const uint2 v = __ldcs(reinterpret_cast<const uint2 *>(a) + k / 2);
					w[k] = v.x; w[k + 1] = v.y;
				}
			}
			else {
#pragma unroll
				for(int k = 0; k < NW; k++) w[k] = __ldcs(reinterpret_cast<const unsigned int *>(a) + k);
			}
		}
		else {
#pragma unroll
			for(int k = 0; k < NW; k++)
				w[k] = 4 * k < valid_bytes ? __ldcs(reinterpret_cast<const unsigned int *>(a) + k) : 0u;
		}
	};

	uint32_t ring[PF][NW];
#pragma unroll
	for(int u = 0; u < PF; u++) {
		if(p0 + u <= p1) load_row(p0 + u, ring[u]);
		else {
#pragma unroll
			for(int k = 0; k < NW; k++) ring[u][k] = 0u;
		}
	}

	for(int p = p0; p <= p1; p += PF) {
#pragma unroll
		for(int u = 0; u < PF; u++) {
			const int pp = p + u;
			if(pp > p1) break;
			uint32_t cur[NW];
#pragma unroll
			for(int k = 0; k < NW; k++) cur[k] = ring[u][k];
			if(pp + PF <= p1) load_row(pp + PF, ring[u]);
			const int q = pp - p0;
			float val[PX][NCH];
#pragma unroll
			for(int px = 0; px < PX; px++) {
				float a = 1.0f;
#pragma unroll
				for(int c = 0; c < NCH; c++) {
					const int sidx = px * NCH + c;      // sample index within the group
					unsigned int code;
					if(DEPTH == 8) code = __byte_perm(cur[sidx >> 2], 0u, 0x4440u + (sidx & 3));
					else code = __byte_perm(cur[sidx >> 1], 0u, (sidx & 1) ? 0x4423u : 0x4401u);
					if(ALPHA && c == NCH - 1) {
						a = __fmul_rn(u2f(code), ainv);
						val[px][c] = a;
					}
					else val[px][c] = dec_table<DEPTH>(s_tab, code);
				}
				if(ALPHA) {
#pragma unroll
					for(int c = 0; c < NCH - 1; c++) val[px][c] = __fmul_rn(val[px][c], a);
				}
			}
			float ws[NS];
			if(NS == 4) {
				const float4 w4 = reinterpret_cast<const float4 *>(s_w)[q];
				ws[0] = w4.x; ws[1] = w4.y; ws[2] = w4.z; ws[3] = w4.w;
			}
			else {
#pragma unroll
				for(int s = 0; s < NS; s += 2) {
					const float2 w2 = reinterpret_cast<const float2 *>(s_w)[(q * NS + s) / 2];
					ws[s] = w2.x; ws[s + 1] = w2.y;
				}
			}
#pragma unroll
			for(int s = 0; s < NS; s++)
#pragma unroll
				for(int px = 0; px < PX; px++)
#pragma unroll
					for(int c = 0; c < NCH; c++) acc[s][px][c] = __fmaf_rn(val[px][c], ws[s], acc[s][px][c]);
			const int2 fin = s_fin[q];
			for(int k = 0; k < fin.y; k++) {
				const int j = fin.x + k;
				const int sj = j % NS;
				const bool keep = j >= jb && j < je;
#pragma unroll
				for(int s = 0; s < NS; s++) {
					if(s == sj) {
						if(keep) {
							float *o = F.interm + (unsigned long long)j * F.mid_w + x0;
#pragma unroll
							for(int px = 0; px < PX; px++) {
								if(full || x0 + px < F.mid_w) {
#pragma unroll
									for(int c = 0; c < NCH; c++) o[(unsigned long long)c * F.plane + px] = acc[s][px][c];
								}
							}
						}
#pragma unroll
						for(int px = 0; px < PX; px++)
#pragma unroll
							for(int c = 0; c < NCH; c++) acc[s][px][c] = 0.0f;
					}
				}
			}
		}
	}
}

// vertical pass, gather (upsampling or wide windows): one thread per (x, j).
template<int NPL, int DEPTH>
__global__ void __launch_bounds__(kVThreads) k_vgather(FJob F)
{
	extern __shared__ float s_tab[];
	for(int k = threadIdx.x; k < F.dec_tab_floats; k += blockDim.x) s_tab[k] = F.dec_tab[k];
	__syncthreads();
	const int x = blockIdx.x * blockDim.x + threadIdx.x;
	const int j = blockIdx.y;
	if(x >= F.mid_w || j >= F.mid_h) return;
	const int bpp = F.nphys * (DEPTH / 8);
	const uint8_t *colbase = F.in + (size_t)(F.crop_x + x) * bpp;
	float acc[NPL];
#pragma unroll
	for(int c = 0; c < NPL; c++) acc[c] = 0.0f;
	for(int t = F.voff[j]; t < F.voff[j + 1]; t++) {
		int row = F.vsrc[t];
		if(row < 0) continue;   // transparent edge contributes 0
		float val[NPL];
		decode_pixel<NPL, DEPTH>(F, s_tab, colbase + (unsigned long long)(F.crop_y + row) * F.in_bpr, val);
		float w = F.vw[t];
#pragma unroll
		for(int c = 0; c < NPL; c++) acc[c] = __fmaf_rn(val[c], w, acc[c]);
	}
#pragma unroll
	for(int c = 0; c < NPL; c++) F.interm[(unsigned long long)c * F.plane + (unsigned long long)j * F.mid_w + x] = acc[c];
}

// ---------------------------------------------------------------------------
// horizontal pass + guarded quantisation
// ---------------------------------------------------------------------------

__device__ __forceinline__ int count_le_f(const float *t, int n, float v)
{
	int lo = 0, hi = n;
	while(lo < hi) {
		int mid = (lo + hi) >> 1;
		if(t[mid] <= v) lo = mid + 1; else hi = mid;
	}
	return lo;
}

// Decides the output code for every value in [v - E, v + E]; returns -1 if
// the interval straddles a decision of the reference.
__device__ __forceinline__ int quantize_guarded(const FTail &T, float v, float E, int x, int y)
{
	v = fminf(fmaxf(v, 0.0f), 1.0f);
	// slack for float rounding of the tables and of this arithmetic
	const float Ep = __fmaf_rn(E, 1.0000001f, __fmaf_rn(fabsf(v), 2.4e-7f, 1e-37f));
	const float lo_v = __fsub_rn(v, Ep), hi_v = __fadd_rn(v, Ep);
	if(T.use_nc) {
		int c = count_le_f(T.nc, 255, v);
		if(c > 0 && !(T.nc[c - 1] < lo_v)) return -1;
		if(c < 255 && !(T.nc[c] > hi_v)) return -1;
		return c;
	}
	int k = count_le_f(T.U + 1, T.P, v);
	bool near_lo = k > 0 && !(T.U[k] < lo_v);          // v within E of the bracket's lower edge
	bool near_hi = k < T.P && !(T.U[k + 1] > hi_v);    // ... or of the next bracket
	if(near_lo || near_hi) {
		// With all codes available, the code at a bracket edge U[k] is k from
		// both sides (the fraction is ~0 above it and ~1 below it), provided
		// the uncertainty is far smaller than the distance to the thresholds.
		if(T.cc != 0 || (near_lo && near_hi)) return -1;
		int kk = near_lo ? k : k + 1;
		// distance to the neighbouring codes on both sides of code kk
		float step = fminf(__fsub_rn(T.rev[kk], T.rev[kk - 1]), kk < T.M ? __fsub_rn(T.rev[kk + 1], T.rev[kk]) : 1.0f);
		if(!(__fmul_rn(Ep, 512.0f) < step)) return -1;
		return T.code[kk];
	}
	const int lo = T.code[k], hi = T.code[k + 1];
	if(k == T.P) return lo;
	const float a = T.rev[lo], b = T.rev[hi];
	const float den = __fsub_rn(b, a);
	const float f = __fdiv_rn(__fsub_rn(v, a), den);
	const float mf = __fdiv_rn(__fmaf_rn(fabsf(a) + fabsf(b), 1.2e-7f, Ep), den) + 1e-6f;
	float thr = 0.5f;
	if(T.dfam == IW_DITHERFAMILY_ORDERED) thr = ((float)dither_rank(T.dsub, x, y) + 0.5f) * 0.015625f;
	int decided;
	if(f >= thr + mf) decided = hi;
	else if(f < thr - mf) decided = lo;
	else return -1;
	// inside the exactly-representable region the reference always picks lo
	if(decided != lo && !(T.X[k] <= lo_v)) return -1;
	return decided;
}

__device__ __forceinline__ void store_code_f(const FJob &F, int ch, int x, int y, unsigned int code)
{
	uint8_t *row = F.out + (unsigned long long)y * F.out_bpr;
	if(F.out_depth == 8) row[F.out_n * x + ch] = (uint8_t)code;
	else {
		uint8_t *p = row + (size_t)(F.out_n * x + ch) * 2;
		p[0] = (uint8_t)(code >> 8);
		p[1] = (uint8_t)(code & 0xff);
	}
}

template<int NPL>
__global__ void __launch_bounds__(kHThreads) k_hpass_fast(FJob F)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	const int j = blockIdx.y;
	if(i >= F.out_w || j >= F.out_h) return;
	float v[NPL], T[NPL];
#pragma unroll
	for(int c = 0; c < NPL; c++) { v[c] = 0.0f; T[c] = 0.0f; }
	const int t0 = F.hoff[i], t1 = F.hoff[i + 1];
	for(int t = t0; t < t1; t++) {
		const int src = __ldg(F.hsrc + t);
		if(src < 0) continue;   // transparent edge: value 0
		const float w = __ldg(F.hw + t), aw = fabsf(w);
#pragma unroll
		for(int c = 0; c < NPL; c++) {
			const float I = __ldg(F.interm + (unsigned long long)c * F.plane + (unsigned long long)j * F.mid_w + src);
			v[c] = __fmaf_rn(I, w, v[c]);
			T[c] = __fmaf_rn(fabsf(I), aw, T[c]);
		}
	}
	float E[NPL];
#pragma unroll
	for(int c = 0; c < NPL; c++) E[c] = __fmaf_rn(F.K1[c], T[c], F.K0[c]);

	// Decide every sample; 'redo' collects the intermediate channels that
	// must be re-evaluated exactly.  An undecided colour sample needs its own
	// channel and the exact alpha (the reference divides by the float alpha);
	// an undecided alpha makes blackening undecided, so the whole pixel is redone.
	// codes are kept per processing slot k (registers); out_of maps k to the channel
	int codes[dev::kMaxCh];
	int alpha_code = -1;
	unsigned int redo = 0;
	const unsigned int all = (1u << F.mid_n) - 1u;
	float A = 0.0f, EA = 0.0f;
#pragma unroll
	for(int k = 0; k < dev::kMaxCh; k++) {
		codes[k] = -1;
		if(k >= F.mid_n || redo == all) continue;
		const int pl = F.k_plane[k];
		float val = 0.0f, err = 0.0f;
#pragma unroll
		for(int c = 0; c < NPL; c++) if(c == pl) { val = v[c]; err = E[c]; }
		const int oc = F.k_out[k];
		const bool is_alpha = F.k_alpha[k];
		if(is_alpha) {
			A = val;
			// the reference divides by the float-rounded alpha: widen by one rounding
			EA = __fmaf_rn(fabsf(val) + err, 6.0e-8f, err);
		}
		else if(F.k_unassoc[k]) {
			if(alpha_code == 0 && F.blacken) { codes[k] = 0; continue; }
			const float den = __fsub_rn(A, EA);
			if(!(den > 0.0f)) { redo |= F.k_bit[k] | F.k_bit[0]; continue; }
			const float q = __fdiv_rn(val, A);
			err = __fdiv_rn(__fmaf_rn(fabsf(q), EA, err), den);
			err = __fmaf_rn(fabsf(q), 1.2e-7f, err);
			val = q;
		}
		const int c = quantize_guarded(F.tail[oc], val, err, i, j);
		if(c < 0) {
			if(is_alpha) redo = all;
			else redo |= F.k_bit[k] | (F.k_unassoc[k] ? F.k_bit[0] : 0u);
			continue;
		}
		if(is_alpha) alpha_code = c;
		codes[k] = c;
	}
	if(redo) {
		const int slot = atomicAdd(F.flag_count, 1);
		F.flag_list[2 * slot] = j * F.out_w + i;
		F.flag_list[2 * slot + 1] = (int)redo;
		if(redo == all) return;
	}
#pragma unroll
	for(int k = 0; k < dev::kMaxCh; k++) {
		if(k >= F.mid_n) continue;
		if(redo & F.k_bit[k]) continue;
		int c = codes[k];
		if(!F.k_alpha[k]) {
			if(F.negate) c = F.k_maxcc[k] - c;
			if(F.blacken && alpha_code == 0) c = 0;
		}
		store_code_f(F, F.k_out[k], i, j, (unsigned int)c);
	}
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

// Device copies of host tables.  The host tables are cached process-wide
// (tables.cpp), so keying by their address is stable; derived float versions
// are cached under (address, kind) together with a reference that keeps the
// source alive.
struct Cache {
	std::mutex mu;
	struct Entry { std::shared_ptr<const void> keep; std::shared_ptr<const void> derived; void *dev; };
	std::map<std::pair<const void *, int>, Entry> dev;
	void *scratch = nullptr;
	size_t scratch_cap = 0;
};

Cache &cache()
{
	static Cache *c = new Cache();
	return *c;
}

template<class T>
const T *upload_vec(const std::vector<T> &v)
{
	void *d = nullptr;
	if(cudaMalloc(&d, std::max<size_t>(16, v.size() * sizeof(T))) != cudaSuccess) return nullptr;
	cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
	return (const T *)d;
}

// Device copy of a persistent host table.
template<class T>
const T *dev_table(const std::shared_ptr<const std::vector<T>> &v)
{
	Cache &C = cache();
	auto key = std::make_pair((const void *)v.get(), 0);
	auto it = C.dev.find(key);
	if(it != C.dev.end()) return (const T *)it->second.dev;
	const T *d = upload_vec(*v);
	if(d) C.dev[key] = {std::static_pointer_cast<const void>(v), nullptr, (void *)d};
	return d;
}

// Device copy of a float table derived from a persistent double table.
template<class Fn>
const float *dev_derived(const std::shared_ptr<const std::vector<double>> &v, int kind, Fn make)
{
	Cache &C = cache();
	auto key = std::make_pair((const void *)v.get(), kind);
	auto it = C.dev.find(key);
	if(it != C.dev.end()) return (const float *)it->second.dev;
	std::shared_ptr<std::vector<float>> f = make(*v);
	const float *d = upload_vec(*f);
	if(d) C.dev[key] = {std::static_pointer_cast<const void>(v), std::static_pointer_cast<const void>(f), (void *)d};
	return d;
}

std::shared_ptr<std::vector<float>> as_float(const std::vector<double> &v)
{
	auto f = std::make_shared<std::vector<float>>(v.size());
	for(size_t i = 0; i < v.size(); i++) (*f)[i] = (float)v[i];   // +-inf stay infinite
	return f;
}

// Decode table for the fast form, and its exactly measured error against the
// double table (every code is evaluated with the same float operations the
// device uses).
struct DecodeTab {
	std::shared_ptr<std::vector<float>> f;
	double err = 0;
};

DecodeTab make_decode_tab(const std::vector<double> &t, int depth)
{
	DecodeTab r;
	auto f = std::make_shared<std::vector<float>>();
	if(depth == 8) {
		f->resize(256);
		for(int c = 0; c < 256; c++) {
			(*f)[c] = (float)t[c];
			r.err = std::max(r.err, fabs((double)(*f)[c] - t[c]));
		}
	}
	else {
		f->resize(8192);
		for(int s = 0; s < 4096; s++) {
			double a = t[s * 16], b = s < 4095 ? t[s * 16 + 16] : t[65535] + (t[65535] - t[65535 - 15]) / 15.0;
			(*f)[2 * s] = (float)a;
			(*f)[2 * s + 1] = (float)((b - a) / 16.0);
		}
		for(int c = 0; c < 65536; c++) {
			float v = fmaf((float)(c & 15), (*f)[2 * (c >> 4) + 1], (*f)[2 * (c >> 4)]);
			r.err = std::max(r.err, fabs((double)v - t[c]));
		}
	}
	r.f = f;
	return r;
}

// Streaming layout of a vertical weight set.
struct StreamTab {
	bool ok = false;
	bool arith = false;         // every referenced position p reads row clamp(p, 0, n_in-1)
	int pmin = 0, npos = 0, ns = 0;
	std::vector<int> first_pos, last_pos, srcrow;
	std::vector<int> pinfo;     // pairs
	std::vector<float> sw;      // npos * 8
};

StreamTab make_stream(const Weights &W)
{
	StreamTab S;
	if(W.kind != RowKind::Sum) return S;
	const int n = W.n_out;
	S.first_pos.resize(n);
	S.last_pos.resize(n);
	int pmin = INT32_MAX, pmax = INT32_MIN;
	for(int j = 0; j < n; j++) {
		if(W.off[j + 1] == W.off[j]) return S;   // empty window: use the gather kernel
		int a = INT32_MAX, b = INT32_MIN;
		for(int t = W.off[j]; t < W.off[j + 1]; t++) { a = std::min(a, W.pos[t]); b = std::max(b, W.pos[t]); }
		S.first_pos[j] = a;
		S.last_pos[j] = b;
		if(j > 0 && (a < S.first_pos[j - 1] || b < S.last_pos[j - 1])) return S;   // not monotone
		pmin = std::min(pmin, a);
		pmax = std::max(pmax, b);
	}
	S.pmin = pmin;
	S.npos = pmax - pmin + 1;
	// widest set of simultaneously open windows
	int ns = 0;
	{
		int lo = 0;
		for(int j = 0; j < n; j++) {
			while(S.last_pos[lo] < S.first_pos[j]) lo++;
			ns = std::max(ns, j - lo + 1);
		}
	}
	if(ns > 8) return S;
	S.ns = ns <= 4 ? 4 : (ns <= 6 ? 6 : 8);
	S.srcrow.assign(S.npos, -1);
	S.sw.assign((size_t)S.npos * 8, 0.0f);
	S.pinfo.assign((size_t)S.npos * 2, 0);
	for(int j = 0; j < n; j++) {
		for(int t = W.off[j]; t < W.off[j + 1]; t++) {
			int q = W.pos[t] - pmin;
			S.srcrow[q] = W.src[t];
			S.sw[(size_t)q * 8 + (j % S.ns)] = (float)W.w[t];
		}
		int q = S.last_pos[j] - pmin;
		if(S.pinfo[2 * q + 1] == 0) S.pinfo[2 * q] = j;
		S.pinfo[2 * q + 1]++;
	}
	S.arith = true;
	for(int q = 0; q < S.npos && S.arith; q++) {
		bool used = false;
		for(int k = 0; k < S.ns; k++) used = used || S.sw[(size_t)q * 8 + k] != 0.0f;
		const int row = std::min(std::max(q + pmin, 0), W.n_in - 1);
		if(used && S.srcrow[q] != row) S.arith = false;
	}
	S.ok = true;
	return S;
}

double gamma_n(int n, double u) { return n * u / (1.0 - n * u); }

}  // namespace

bool fast_eligible(const Plan &P, const Job &J, FastInfo &fi)
{
	if(P.in_sampletype != IW_SAMPLETYPE_UINT || (P.in_depth != 8 && P.in_depth != 16)) return false;
	if(P.orient != 0 || P.reduced_in || P.apply_bk || P.intclamp) return false;
	if(P.out_sampletype != IW_SAMPLETYPE_UINT || P.wsets[0].size() != 1 || P.wsets[1].size() != 1) return false;
	for(int m = 0; m < P.mid_n; m++) {
		if(P.mid[m].to_gray || P.mid[m].out_ch < 0) return false;
	}
	for(int oc = 0; oc < P.out_n; oc++) {
		int f = P.out[oc].q.dfam;
		if(f != IW_DITHERFAMILY_NONE && f != IW_DITHERFAMILY_ORDERED) return false;
		if(P.out[oc].q.P > 65535) return false;
	}
	if(P.wsets[0][0]->edge_value != 0.0 || P.wsets[1][0]->edge_value != 0.0) return false;
	(void)J;
	fi.streaming = 0;
	fi.slots = 0;
	return true;
}

struct FastState {
	FJob F;
	Job J;
	const void *vkernel = nullptr, *hkernel = nullptr;
	dim3 vgrid, hgrid;
	int vthreads = kVThreads;
	size_t vsmem = 0;
};

void fast_launch_impl(cudaStream_t st, void *state, void (*mark)(void *), void *markarg)
{
	FastState &S = *static_cast<FastState *>(state);
	cudaMemsetAsync(S.F.flag_count, 0, sizeof(int), st);
	void *fargs[] = {&S.F};
	cudaLaunchKernel(S.vkernel, S.vgrid, dim3(S.vthreads), fargs, S.vsmem, st);
	mark(markarg);
	cudaLaunchKernel(S.hkernel, S.hgrid, dim3(kHThreads), fargs, 0, st);
	mark(markarg);
	// exact re-evaluation of flagged pixels (recomputes the vertical pass too)
	launch_fix_flagged(st, S.J, S.F.flag_count, S.F.flag_list);
	mark(markarg);
}

void fast_release(FastInfo &fi)
{
	delete static_cast<FastState *>(fi.state);
	fi.state = nullptr;
}

bool fast_prepare(cudaStream_t st, const Plan &P, Job &J, FastInfo &fi, std::string &err)
{
	Cache &C = cache();
	std::lock_guard<std::mutex> lk(C.mu);
	FJob F;
	memset(&F, 0, sizeof(F));
	const Weights &WV = *P.wsets[1][0], &WH = *P.wsets[0][0];

	// ---- planes: distinct (input channel, transfer, premultiply) combinations
	int nplanes = 0;
	int plane_of[dev::kMaxCh] = {0, 0, 0, 0};
	struct PK { int src, lin, premul; };
	PK keys[kMaxPlanes];
	std::shared_ptr<const std::vector<double>> coltab;
	int alpha_plane = -1;
	for(int m = 0; m < P.mid_n; m++) {
		const MidChannel &mc = P.mid[m];
		PK k{mc.in_ch < P.in_nphys ? mc.in_ch : -1, mc.lin_cs || P.cs_in.cstype == IW_CSTYPE_LINEAR, mc.unassoc};
		int found = -1;
		for(int q = 0; q < nplanes; q++)
			if(keys[q].src == k.src && keys[q].lin == k.lin && keys[q].premul == k.premul) found = q;
		if(found < 0) {
			found = nplanes++;
			keys[found] = k;
			FPlane &pl = F.pl[found];
			pl.src = k.src;
			pl.premul = k.premul;
			pl.table = !k.lin && k.src >= 0;
			pl.inv = (float)(1.0 / (double)P.in_max);
			if(pl.table) coltab = input_table(P.cs_in.cstype, P.cs_in.gamma, P.in_max, 1 << P.in_depth, false);
		}
		plane_of[m] = found;
		if(mc.ctype == IW_CHANNELTYPE_ALPHA) alpha_plane = found;
	}
	F.npl = nplanes;
	F.alpha_plane = alpha_plane;
	F.alpha_src = (IW_IMGTYPE_HAS_ALPHA(P.in_logtype) && P.in_alpha < P.in_nphys) ? P.in_alpha : -1;
	F.alpha_inv = (float)(1.0 / (double)P.in_max);

	// decode error: table interpolation / rounding, or code*inv rounding
	double e_dec = 0.0;
	const double u = 1.0 / 16777216.0, ud = 1.0 / 9007199254740992.0;
	const float *dec_tab = nullptr;
	int dec_floats = 0;
	if(coltab) {
		static std::map<std::pair<const void *, int>, double> dec_err;   // measured once per table
		double e = 0.0;
		dec_tab = dev_derived(coltab, 100 + P.in_depth, [&](const std::vector<double> &t) {
			DecodeTab dt = make_decode_tab(t, P.in_depth);
			e = dt.err;
			dec_err[std::make_pair((const void *)coltab.get(), P.in_depth)] = dt.err;
			return dt.f;
		});
		e_dec = dec_err[std::make_pair((const void *)coltab.get(), P.in_depth)];
		dec_floats = P.in_depth == 8 ? 256 : 8192;
		if(!dec_tab) { err = "Out of GPU memory (fast tables)"; return false; }
	}
	e_dec = std::max(e_dec, 2.0 * u);   // code*inv: 1/maxcc rounded, product rounded
	F.dec_tab = dec_tab;
	F.dec_tab_floats = dec_floats;

	// ---- error model constants per plane
	const int nv = std::max(1, WV.max_taps), nh = std::max(1, WH.max_taps);
	const double W1v = WV.kind == RowKind::Copy ? 1.0 : WV.wsum_abs_max, W1h = WH.kind == RowKind::Copy ? 1.0 : WH.wsum_abs_max;
	const double Wnv = WV.kind == RowKind::Copy ? 0.0 : WV.wsum_neg_max;
	for(int q = 0; q < nplanes; q++) {
		double r_dec = keys[q].premul ? 3.0 * u : 0.0;
		double c1 = (r_dec + 2.0 * u + gamma_n(nv + 1, u) + gamma_n(nv + 1, ud)) * 1.01;
		double c2 = (u + gamma_n(nh + 1, u) + gamma_n(nh + 1, ud)) * 1.01;
		double ed = e_dec * (keys[q].premul ? 1.0 : 1.0);
		double K0 = (ed * W1v * W1h + 2.02 * c1 * Wnv * W1h) * 1.05;
		double K1 = (1.01 * c1 + c2) * 1.05;
		F.K0[q] = (float)K0;
		F.K1[q] = (float)K1;
	}

	// ---- geometry and buffers (shared with the plain form's Job)
	F.in = J.in;
	F.in_bpr = J.in_bpr;
	F.crop_x = P.crop_x;
	F.crop_y = P.crop_y;
	F.nphys = P.in_nphys;
	F.depth = P.in_depth;
	{
		const int bpp = P.in_nphys * P.in_depth / 8;
		const uintptr_t base = (uintptr_t)J.in + (uintptr_t)P.crop_x * bpp + (uintptr_t)P.crop_y * P.in_bpr;
		F.vec = 0;
		if((bpp == 8 || bpp == 4) && base % bpp == 0 && P.in_bpr % bpp == 0) F.vec = bpp;
	}
	F.mid_w = J.mid_w;
	F.mid_h = J.mid_h;
	F.in_rows = P.crop_h;
	F.interm = J.interm;
	F.plane = J.interm_plane;
	F.out_w = J.out_w; F.out_h = J.out_h; F.out_n = J.out_n; F.out_depth = J.out_depth;
	F.out = J.out;
	F.out_bpr = J.out_bpr;
	F.mid_n = P.mid_n;
	for(int k = 0; k < P.mid_n; k++) {
		const int m = J.order[k];
		const MidChannel &mc = P.mid[m];
		F.k_plane[k] = plane_of[m];
		F.k_out[k] = mc.out_ch;
		F.k_alpha[k] = mc.ctype == IW_CHANNELTYPE_ALPHA;
		F.k_unassoc[k] = mc.unassoc;
		F.k_maxcc[k] = P.out[mc.out_ch].maxcc;
		F.k_bit[k] = 1u << m;
	}
	F.negate = P.negate;
	F.blacken = P.blacken;

	// ---- per-call device arrays (weights, streaming tables)
	StreamTab S = make_stream(WV);
	std::vector<uint8_t> blob;
	auto add = [&](const void *p, size_t n) {
		size_t off = (blob.size() + 255) & ~(size_t)255;
		blob.resize(off + n);
		if(n) memcpy(blob.data() + off, p, n);
		return off;
	};
	std::vector<float> hwf(WH.w.begin(), WH.w.end()), vwf(WV.w.begin(), WV.w.end());
	size_t o_hoff = add(WH.off.data(), WH.off.size() * 4), o_hsrc = add(WH.src.data(), WH.src.size() * 4);
	size_t o_hw = add(hwf.data(), hwf.size() * 4);
	size_t o_voff = add(WV.off.data(), WV.off.size() * 4), o_vsrc = add(WV.src.data(), WV.src.size() * 4);
	size_t o_vw = add(vwf.data(), vwf.size() * 4);
	size_t o_fp = 0, o_lp = 0, o_src = 0, o_pi = 0, o_sw = 0;
	if(S.ok) {
		o_fp = add(S.first_pos.data(), S.first_pos.size() * 4);
		o_lp = add(S.last_pos.data(), S.last_pos.size() * 4);
		o_src = add(S.srcrow.data(), S.srcrow.size() * 4);
		o_pi = add(S.pinfo.data(), S.pinfo.size() * 4);
		o_sw = add(S.sw.data(), S.sw.size() * 4);
	}
	const size_t flag_bytes = 256 + (size_t)J.out_w * J.out_h * 8;
	size_t need = blob.size() + 256 + flag_bytes + 256 + sizeof(FTail) * dev::kMaxCh;
	if(need > C.scratch_cap) {
		if(C.scratch) cudaFree(C.scratch);
		C.scratch = nullptr;
		C.scratch_cap = 0;
		if(cudaMalloc(&C.scratch, need + need / 8) != cudaSuccess) { err = "Out of GPU memory (fast form)"; return false; }
		C.scratch_cap = need + need / 8;
	}
	uint8_t *base = (uint8_t *)C.scratch;
	cudaMemcpyAsync(base, blob.data(), blob.size(), cudaMemcpyHostToDevice, st);
	size_t flag_off = (blob.size() + 255) & ~(size_t)255;
	F.flag_count = (int *)(base + flag_off);
	F.flag_list = (int *)(base + flag_off + 256);
	F.hoff = (const int *)(base + o_hoff);
	F.hsrc = (const int *)(base + o_hsrc);
	F.hw = (const float *)(base + o_hw);
	F.voff = (const int *)(base + o_voff);
	F.vsrc = (const int *)(base + o_vsrc);
	F.vw = (const float *)(base + o_vw);
	if(S.ok) {
		F.first_pos = (const int *)(base + o_fp);
		F.last_pos = (const int *)(base + o_lp);
		F.srcrow = (const int *)(base + o_src);
		F.pinfo = (const int2 *)(base + o_pi);
		F.sw = (const float *)(base + o_sw);
		F.pmin = S.pmin;
		F.npos = S.npos;
		F.ns = S.ns;
	}

	// ---- quantisation tables (float copies, cached)
	FTail tails[dev::kMaxCh];
	memset(tails, 0, sizeof(tails));
	for(int oc = 0; oc < P.out_n; oc++) {
		const Quant &q = P.out[oc].q;
		FTail &T = tails[oc];
		T.P = q.P; T.M = q.maxcc; T.cc = q.cc; T.use_nc = q.use_nc; T.dfam = q.dfam; T.dsub = q.dsub;
		T.U = dev_derived(q.U, 1, as_float);
		T.X = dev_derived(q.X, 1, as_float);
		T.code = dev_table(q.code);
		T.rev = dev_derived(q.rev, 1, as_float);
		T.nc = q.use_nc ? dev_derived(q.nc, 1, as_float) : nullptr;
		if(!T.U || !T.X || !T.code || !T.rev || (q.use_nc && !T.nc)) { err = "Out of GPU memory (fast tables)"; return false; }
	}
	{
		const size_t tail_off = (flag_off + 256 + flag_bytes + 255) & ~(size_t)255;
		cudaMemcpyAsync(base + tail_off, tails, sizeof(tails), cudaMemcpyHostToDevice, st);
		F.tail = (const FTail *)(base + tail_off);
	}

	// ---- kernel selection
	auto *FS = new FastState();
	const int gx = (F.mid_w + kVThreads - 1) / kVThreads;
	FS->vsmem = (size_t)dec_floats * sizeof(float);
	FS->vgrid = dim3(gx, F.mid_h);
#define IWG_VSTREAM(NS_, NPL_, D_) \
	if(!FS->vkernel && S.ns == NS_ && nplanes == NPL_ && P.in_depth == D_) { \
		int bands = std::max(1, std::min(F.mid_h, (4 * 152 + gx - 1) / gx)); \
		F.rows_per_band = (F.mid_h + bands - 1) / bands; \
		bands = (F.mid_h + F.rows_per_band - 1) / F.rows_per_band; \
		FS->vkernel = (const void *)k_vstream<NS_, NPL_, D_>; \
		FS->vgrid = dim3(gx, bands); \
	}
#define IWG_VGATHER(NPL_, D_) \
	if(!FS->vkernel && nplanes == NPL_ && P.in_depth == D_) FS->vkernel = (const void *)k_vgather<NPL_, D_>;
	// identity layout: plane c reads input channel c, the last one alpha when present
	bool ident = S.ok && nplanes == P.in_nphys && dec_tab != nullptr;
	for(int q = 0; q < nplanes && ident; q++) {
		bool is_a = (F.alpha_src >= 0 && q == nplanes - 1);
		if(F.pl[q].src != q) ident = false;
		else if(is_a && (F.pl[q].table || F.pl[q].premul)) ident = false;
		else if(!is_a && (!F.pl[q].table || F.pl[q].premul != (F.alpha_src >= 0))) ident = false;
	}
	if(F.alpha_src >= 0 && F.alpha_src != nplanes - 1) ident = false;
	// PX pixels per thread, one aligned word group per row
	const int v_bpp = P.in_nphys * P.in_depth / 8;
	const uintptr_t v_base = (uintptr_t)J.in + (uintptr_t)P.crop_x * v_bpp + (uintptr_t)P.crop_y * P.in_bpr;
#define IWG_VPX(NS_, NCH_, A_, D_, PX_) \
	if(!FS->vkernel && ident && S.arith && S.ns == NS_ && nplanes == NCH_ && (F.alpha_src >= 0) == A_ && \
		P.in_depth == D_) { \
		constexpr int nw_ = PX_ * NCH_ * (D_ / 8) / 4; \
		constexpr uintptr_t va_ = nw_ % 4 == 0 ? 16 : (nw_ % 2 == 0 ? 8 : 4); \
		if(v_base % va_ == 0 && P.in_bpr % va_ == 0) { \
			const int threads_ = (F.mid_w + PX_ - 1) / PX_; \
			const int gxp_ = (threads_ + kVPxThreads - 1) / kVPxThreads; \
			int bands = std::max(1, std::min(F.mid_h, (5 * 152 + gxp_ / 2) / gxp_)); \
			F.rows_per_band = (F.mid_h + bands - 1) / bands; \
			bands = (F.mid_h + F.rows_per_band - 1) / F.rows_per_band; \
			int nq_max = 0; \
			for(int b_ = 0; b_ < bands; b_++) { \
				const int jb_ = b_ * F.rows_per_band, je_ = std::min(jb_ + F.rows_per_band, F.mid_h); \
				nq_max = std::max(nq_max, S.last_pos[je_ - 1] - S.first_pos[jb_] + 1); \
			} \
			const size_t sm_ = (size_t)dec_floats * sizeof(float) + (size_t)nq_max * (NS_ * sizeof(float) + sizeof(int2)); \
			const void *k_ = (const void *)k_vstream_px<NS_, NCH_, A_, D_, PX_>; \
			if(sm_ <= 48 * 1024 || (sm_ <= 200 * 1024 && \
				cudaFuncSetAttribute(k_, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_) == cudaSuccess)) { \
				FS->vkernel = k_; \
				FS->vgrid = dim3(gxp_, bands); \
				FS->vthreads = kVPxThreads; \
				FS->vsmem = sm_; \
			} \
		} \
	}
	{
		IWG_VPX(4, 4, true, 16, 2) IWG_VPX(6, 4, true, 16, 2) IWG_VPX(8, 4, true, 16, 2)
		IWG_VPX(4, 3, false, 16, 2) IWG_VPX(6, 3, false, 16, 2) IWG_VPX(8, 3, false, 16, 2)
		IWG_VPX(4, 2, true, 16, 4) IWG_VPX(6, 2, true, 16, 4) IWG_VPX(8, 2, true, 16, 4)
		IWG_VPX(4, 1, false, 16, 8) IWG_VPX(6, 1, false, 16, 8) IWG_VPX(8, 1, false, 16, 8)
		IWG_VPX(4, 4, true, 8, 2) IWG_VPX(6, 4, true, 8, 2) IWG_VPX(8, 4, true, 8, 2)
		IWG_VPX(4, 3, false, 8, 4)
		IWG_VPX(4, 2, true, 8, 4) IWG_VPX(6, 2, true, 8, 4) IWG_VPX(8, 2, true, 8, 4)
		IWG_VPX(4, 1, false, 8, 8) IWG_VPX(6, 1, false, 8, 8) IWG_VPX(8, 1, false, 8, 8)
	}
#undef IWG_VPX
	if(S.ok) {
		IWG_VSTREAM(4, 1, 8) IWG_VSTREAM(4, 2, 8) IWG_VSTREAM(4, 3, 8) IWG_VSTREAM(4, 4, 8)
		IWG_VSTREAM(6, 1, 8) IWG_VSTREAM(6, 2, 8) IWG_VSTREAM(6, 3, 8) IWG_VSTREAM(6, 4, 8)
		IWG_VSTREAM(8, 1, 8) IWG_VSTREAM(8, 2, 8) IWG_VSTREAM(8, 3, 8) IWG_VSTREAM(8, 4, 8)
		IWG_VSTREAM(4, 1, 16) IWG_VSTREAM(4, 2, 16) IWG_VSTREAM(4, 3, 16) IWG_VSTREAM(4, 4, 16)
		IWG_VSTREAM(6, 1, 16) IWG_VSTREAM(6, 2, 16) IWG_VSTREAM(6, 3, 16) IWG_VSTREAM(6, 4, 16)
		IWG_VSTREAM(8, 1, 16) IWG_VSTREAM(8, 2, 16) IWG_VSTREAM(8, 3, 16) IWG_VSTREAM(8, 4, 16)
	}
	IWG_VGATHER(1, 8) IWG_VGATHER(2, 8) IWG_VGATHER(3, 8) IWG_VGATHER(4, 8)
	IWG_VGATHER(1, 16) IWG_VGATHER(2, 16) IWG_VGATHER(3, 16) IWG_VGATHER(4, 16)
#undef IWG_VSTREAM
#undef IWG_VGATHER
	if(!FS->vkernel) { delete FS; err = "fast form: no kernel for this layout"; return false; }
	switch(nplanes) {
	case 1: FS->hkernel = (const void *)k_hpass_fast<1>; break;
	case 2: FS->hkernel = (const void *)k_hpass_fast<2>; break;
	case 3: FS->hkernel = (const void *)k_hpass_fast<3>; break;
	default: FS->hkernel = (const void *)k_hpass_fast<4>; break;
	}
	FS->hgrid = dim3((F.out_w + kHThreads - 1) / kHThreads, F.out_h);
	FS->F = F;
	FS->J = J;
	fi.state = FS;
	fi.launches = 3;
	fi.launch_fn = fast_launch_impl;
	fi.streaming = S.ok;
	fi.slots = S.ns;
	fi.flag_count_dev = F.flag_count;
	return true;
}

}  // namespace iwg
