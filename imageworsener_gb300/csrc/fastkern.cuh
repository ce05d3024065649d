// fastkern.cuh -- device side of the FP32 + guard-band form: the job layout
// (FJob) and the per-tile bodies of its kernels.  Included by fastpath.cu
// (one launch per image) and fastbatch.cu (one launch per kernel variant for
// a whole batch of images); both wrap the same bodies.
#pragma once

#include "iwg_internal.h"
#include "device.cuh"
#include "tcvert.cuh"

#include <cstdint>
#include <vector>

namespace iwg {
namespace fp {

using namespace dev;

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
	const float *lut; // kLutCells: entries of the searched table (nc, or U[1..P]) <= cell/kLutCells
};

constexpr int kLutCells = 1024;
constexpr int kHBlock = 4;    // horizontal taps per partial sum (blocked summation: about sqrt(n) is best)

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
	FTail k_tail[dev::kMaxCh];  // quantisation of the output channel of slot k
	int negate, blacken;
	// error model
	float K0[kMaxPlanes], K1[kMaxPlanes];
	// flags
	int *flag_count;
	int *flag_list;            // entries (pixel, mask, image, 0)
	int flag_cap;              // entries the list holds
	int img;                   // index of the image in a batch (0 alone)
	int *err_flag;             // set by a kernel whose bounded wait ran out
	int wait_polls;            // polls of a pipeline wait before it gives up (kWaitPolls; failure tests shorten it)
	int starve;                // failure tests: the producer issues no copies, so every pipeline wait runs out
	int vgx, vgy, hgx;         // blocks of the vertical pass (x, bands or rows), horizontal pass (x)
	// debug readback (null normally): per output sample, the FP32 value the
	// tail quantises and its error bound, [2][out_n][out_h][out_w]; NaN where
	// the tail decided without a value (blackened, undecidable alpha)
	float *dbg;
};
static_assert(sizeof(FJob) <= 4096, "FJob is passed by value as a kernel parameter");

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
__device__ __forceinline__ void vstream_tile(const FJob &F, float *s_tab, int bx, int band)
{
	constexpr int PF = 8;
	for(int k = threadIdx.x; k < F.dec_tab_floats; k += blockDim.x) s_tab[k] = F.dec_tab[k];
	__syncthreads();

	const int x = bx * blockDim.x + threadIdx.x;
	const bool active = x < F.mid_w;
	const int jb = band * F.rows_per_band;
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
// Two floats in one 64-bit register pair, and Blackwell's paired FP32
// operations on them: each half is rounded exactly like __fmaf_rn /
// __fmul_rn, in half the instructions.
__device__ __forceinline__ unsigned long long f2_pack(float lo, float hi)
{
	unsigned long long d;
	asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(lo), "f"(hi));
	return d;
}

__device__ __forceinline__ void f2_unpack(unsigned long long v, float &lo, float &hi)
{
	asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}

__device__ __forceinline__ unsigned long long f2_fma(unsigned long long a, unsigned long long b, unsigned long long c)
{
	unsigned long long d;
	asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
	return d;
}

__device__ __forceinline__ unsigned long long f2_mul(unsigned long long a, unsigned long long b)
{
	unsigned long long d;
	asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
	return d;
}

__device__ __forceinline__ float u2f(unsigned int v)
{
	return __fsub_rn(__uint_as_float(0x4b000000u | v), 8388608.0f);
}


// ---- asynchronous bulk copies and mbarriers (inline PTX, sm_90 and later) ----
__device__ __forceinline__ unsigned smem_u32(const void *p)
{
	return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(unsigned long long *bar)
{
	asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Waits for the phase of 'parity' to complete; gives up (false) after a
// bounded number of polls (each poll may suspend the thread briefly).  The
// pipeline's waits take the job's limit (FJob::wait_polls: a failure test
// shortens it); the final wait for a block's own copies in flight always
// takes the full limit.
constexpr int kWaitPolls = 1 << 21;

__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity, int polls = kWaitPolls)
{
	for(int it = 0; it < polls; it++) {
		unsigned done;
		asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
			: "=r"(done) : "r"(smem_u32(bar)), "r"(parity) : "memory");
		if(done) return true;
	}
	return false;
}

// Global -> shared copy of 'bytes' (multiple of 16, both addresses 16-byte
// aligned) that counts its bytes on 'bar'.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar)
{
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
		::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}

constexpr int kBulkConsumers = 256;   // threads that decode and accumulate
constexpr int kBulkThreads = kBulkConsumers + 32;   // plus one producer warp
constexpr int kBulkStages = 8;        // rows in flight per block

// Vertical pass, streaming, with the rows of a strip staged in shared memory
// by asynchronous bulk copies.  A producer warp keeps kBulkStages rows of the
// block's strip (kBulkConsumers * PX pixels) in flight; consumer threads
// read their PX pixels of a row from shared memory, then decode and
// accumulate exactly as vstream_px_tile (same slot scheme, same results).
// Every wait is bounded: a wait that runs out sets F.err_flag, the producer
// waits (bounded) for the copies it issued, and the block returns.
template<int NS, int NCH, bool ALPHA, int DEPTH, int PX>
__device__ __forceinline__ void vbulk_tile(const FJob &F, unsigned char *s_raw, int bx, int band)
{
	constexpr int BPP = NCH * (DEPTH / 8);
	constexpr int NW = PX * BPP / 4;
	static_assert(NW == 4, "one 16-byte group per consumer and row");
	constexpr int STRIP = kBulkConsumers * PX * BPP;     // bytes of a full strip row
	unsigned char *ring = s_raw;                          // kBulkStages * STRIP
	unsigned long long *full = reinterpret_cast<unsigned long long *>(s_raw + kBulkStages * STRIP);
	unsigned long long *empty = full + kBulkStages;
	int *abort_flag = reinterpret_cast<int *>(empty + kBulkStages);
	float *s_tab = reinterpret_cast<float *>(s_raw + kBulkStages * STRIP + 256);
	const int jb = band * F.rows_per_band;
	const int je = min(jb + F.rows_per_band, F.mid_h);
	if(jb >= je) return;
	const int p0 = F.first_pos[jb], p1 = F.last_pos[je - 1];
	const int nq = p1 - p0 + 1;
	float *s_w = s_tab + F.dec_tab_floats;
	int2 *s_fin = reinterpret_cast<int2 *>(s_w + (size_t)nq * NS);
	for(int k = threadIdx.x; k < F.dec_tab_floats; k += blockDim.x) s_tab[k] = F.dec_tab[k];
	for(int k = threadIdx.x; k < nq * NS; k += blockDim.x) {
		const int q = k / NS, sl = k - q * NS;
		s_w[k] = F.sw[(size_t)(p0 - F.pmin + q) * 8 + sl];
	}
	for(int k = threadIdx.x; k < nq; k += blockDim.x) s_fin[k] = F.pinfo[p0 - F.pmin + k];
	if(threadIdx.x == 0) {
		for(int k = 0; k < kBulkStages; k++) {
			mbar_init(full + k, 1);
			mbar_init(empty + k, kBulkConsumers / 32);
		}
		*abort_flag = 0;
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	__syncthreads();

	const int strip_x = bx * kBulkConsumers * PX;        // first pixel of the strip
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	if(warp == kBulkConsumers / 32) {
		// producer
		if(lane != 0) return;
		const uint8_t *base = F.in + (size_t)(F.crop_x + strip_x) * BPP + (unsigned long long)F.crop_y * F.in_bpr;
		const int strip_px = min(kBulkConsumers * PX, F.mid_w - strip_x);
		const unsigned bytes = (unsigned)((strip_px * BPP + 15) & ~15);
		const int last_row = F.in_rows - 1;
		int issued = 0;
		bool ok = true;
		for(int q = 0; q < nq && ok && !F.starve; q++) {
			const int st = q % kBulkStages, use = q / kBulkStages;
			if(use > 0 && !mbar_wait(empty + st, (use - 1) & 1, F.wait_polls)) { ok = false; break; }
			if(*(volatile int *)abort_flag) { ok = false; break; }
			const int row = min(max(p0 + q, 0), last_row);
			mbar_expect_tx(full + st, bytes);
			bulk_g2s(ring + (size_t)st * STRIP, base + (unsigned long long)row * F.in_bpr, bytes, full + st);
			issued = q + 1;
		}
		if(!ok) {
			atomicExch(F.err_flag, 1);
			*(volatile int *)abort_flag = 1;
		}
		// every issued copy lands before the block's shared memory goes away
		for(int q = max(0, issued - kBulkStages); q < issued; q++) mbar_wait(full + q % kBulkStages, (q / kBulkStages) & 1);
		return;
	}

	// consumers
	const int x0 = strip_x + threadIdx.x * PX;
	const bool any = x0 < F.mid_w;
	const bool full_px = x0 + PX <= F.mid_w;
	const float ainv = F.alpha_inv;
	const unsigned long long plane = F.plane;
	const int mid_w = F.mid_w;
	float *const interm = F.interm;
	static_assert(PX == 2, "accumulators pair the thread's two pixels");
	static_assert(NS == 4, "one 16-byte load of the slot weights per row (16-byte aligned: the decode table before them holds 256 or 8192 floats)");
	unsigned long long acc[NS][NCH];   // (pixel 0, pixel 1) per slot and channel
#pragma unroll
	for(int s = 0; s < NS; s++)
#pragma unroll
		for(int c = 0; c < NCH; c++) acc[s][c] = 0ULL;

	for(int q = 0; q < nq; q++) {
		const int st = q % kBulkStages, use = q / kBulkStages;
		if(!mbar_wait(full + st, use & 1, F.wait_polls)) {
			atomicExch(F.err_flag, 1);
			*(volatile int *)abort_flag = 1;
			return;
		}
		uint32_t cur[NW];
		{
			const uint4 v = reinterpret_cast<const uint4 *>(ring + (size_t)st * STRIP)[threadIdx.x];
			cur[0] = v.x; cur[1] = v.y; cur[2] = v.z; cur[3] = v.w;
		}
		__syncwarp();
		if(lane == 0) mbar_arrive(empty + st);
		float val[PX][NCH], a[PX];
#pragma unroll
		for(int px = 0; px < PX; px++) {
			a[px] = 1.0f;
#pragma unroll
			for(int c = 0; c < NCH; c++) {
				const int sidx = px * NCH + c;
				unsigned int code;
				if(DEPTH == 8) code = __byte_perm(cur[sidx >> 2], 0u, 0x4440u + (sidx & 3));
				else code = __byte_perm(cur[sidx >> 1], 0u, (sidx & 1) ? 0x4423u : 0x4401u);
				if(ALPHA && c == NCH - 1) {
					a[px] = __fmul_rn(u2f(code), ainv);
					val[px][c] = a[px];
				}
				else val[px][c] = dec_table<DEPTH>(s_tab, code);
			}
		}
		unsigned long long v2[NCH];
#pragma unroll
		for(int c = 0; c < NCH; c++) v2[c] = f2_pack(val[0][c], val[1][c]);
		if(ALPHA) {
			const unsigned long long a2 = f2_pack(a[0], a[1]);
#pragma unroll
			for(int c = 0; c < NCH - 1; c++) v2[c] = f2_mul(v2[c], a2);   // premultiply
		}
		const float4 wq = *reinterpret_cast<const float4 *>(s_w + q * NS);
		const float wsv[4] = {wq.x, wq.y, wq.z, wq.w};
#pragma unroll
		for(int s = 0; s < NS; s++) {
			const unsigned long long w2 = f2_pack(wsv[s], wsv[s]);
#pragma unroll
			for(int c = 0; c < NCH; c++) acc[s][c] = f2_fma(v2[c], w2, acc[s][c]);
		}
		const int2 fin = s_fin[q];
		for(int k = 0; k < fin.y; k++) {
			const int j = fin.x + k;
			const int sj = j % NS;
			const bool keep = any && j >= jb && j < je;
#pragma unroll
			for(int s = 0; s < NS; s++) {
				if(s == sj) {
					if(keep) {
						float *o = interm + (unsigned long long)j * mid_w + x0;
#pragma unroll
						for(int c = 0; c < NCH; c++) {
							float lo, hi;
							f2_unpack(acc[s][c], lo, hi);
							o[(unsigned long long)c * plane] = lo;
							if(full_px) o[(unsigned long long)c * plane + 1] = hi;
						}
					}
#pragma unroll
					for(int c = 0; c < NCH; c++) acc[s][c] = 0ULL;
				}
			}
		}
	}
}

// ---------------------------------------------------------------------------
// Fused vertical + horizontal pass (one launch, no intermediate image in
// device memory).  A block owns a tile of output columns [i0, i1) and a band
// of output rows.  Its producer warp streams the rows of the input columns
// the tile's horizontal windows read ([xa, xa + nc)) into a shared-memory
// ring with bulk copies (as vbulk_tile); the consumers decode and accumulate
// the vertical sums exactly as vbulk_tile does (same operations, same order,
// so the same float intermediates), but a finished intermediate row goes to
// a small ring of rows in shared memory instead of device memory.  Every
// second finished row, the consumers synchronise and run the horizontal sums
// and the guarded quantisation tail of those rows' output pixels from shared
// memory (same operations and order as hpass_pixel, so the same values,
// bounds, codes and flags as the two-kernel form).
// Rows are summed horizontally two at a time, as soon as the second one
// finishes, wherever they finish (several rows can finish at one input
// position where the image's last row ends their windows): the four-row
// ring then always holds the two rows being summed and at most two filling.
// Requirements (checked by the host): the tile's input columns fit one strip
// of kBulkConsumers * PX pixels, every horizontal source of the tile lies in
// [xa, xa + nc), rows 16-byte aligned, nc * bytes per pixel a multiple of 16.
// ---------------------------------------------------------------------------
template<int NPL>
__device__ __forceinline__ void hpass_tail(const FJob &F, int i, int j, const float (&v)[NPL], const float (&T)[NPL]);

struct FuseTile {
	int xa, nc;       // first input column of the tile's strip, columns
	int i0, i1;       // output columns
};
constexpr int kFuseRows = 4;   // intermediate rows in shared memory (two being summed, two filling)

template<int NS, int NCH, bool ALPHA, int DEPTH, int PX>
__device__ __forceinline__ void vhfuse_tile(const FJob &F, const FuseTile *tiles, unsigned char *s_raw, int tile, int band)
{
	constexpr int BPP = NCH * (DEPTH / 8);
	constexpr int NW = PX * BPP / 4;
	static_assert(NW == 4, "one 16-byte group per consumer and row");
	static_assert(NCH == 4, "the row ring holds one float4 per column");
	constexpr int STRIP = kBulkConsumers * PX * BPP;
	constexpr int MIDW = kBulkConsumers * PX;              // columns of a ring row
	unsigned char *ring = s_raw;                           // kBulkStages * STRIP
	float4 *mid = reinterpret_cast<float4 *>(s_raw + kBulkStages * STRIP);   // kFuseRows * MIDW
	unsigned char *after = s_raw + kBulkStages * STRIP + (size_t)kFuseRows * MIDW * sizeof(float4);
	unsigned long long *full = reinterpret_cast<unsigned long long *>(after);
	unsigned long long *empty = full + kBulkStages;
	int *abort_flag = reinterpret_cast<int *>(empty + kBulkStages);
	float *s_tab = reinterpret_cast<float *>(after + 256);
	const FuseTile T = tiles[tile];
	const int jb = band * F.rows_per_band;
	const int je = min(jb + F.rows_per_band, F.mid_h);
	if(jb >= je) return;
	const int p0 = F.first_pos[jb], p1 = F.last_pos[je - 1];
	const int nq = p1 - p0 + 1;
	float *s_w = s_tab + F.dec_tab_floats;
	int2 *s_fin = reinterpret_cast<int2 *>(s_w + (size_t)nq * NS);
	for(int k = threadIdx.x; k < F.dec_tab_floats; k += blockDim.x) s_tab[k] = F.dec_tab[k];
	for(int k = threadIdx.x; k < nq * NS; k += blockDim.x) {
		const int q = k / NS, sl = k - q * NS;
		s_w[k] = F.sw[(size_t)(p0 - F.pmin + q) * 8 + sl];
	}
	for(int k = threadIdx.x; k < nq; k += blockDim.x) s_fin[k] = F.pinfo[p0 - F.pmin + k];
	if(threadIdx.x == 0) {
		for(int k = 0; k < kBulkStages; k++) {
			mbar_init(full + k, 1);
			mbar_init(empty + k, kBulkConsumers / 32);
		}
		*abort_flag = 0;
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	__syncthreads();

	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	if(warp == kBulkConsumers / 32) {
		// producer
		if(lane != 0) return;
		const uint8_t *base = F.in + (size_t)(F.crop_x + T.xa) * BPP + (unsigned long long)F.crop_y * F.in_bpr;
		const unsigned bytes = (unsigned)(T.nc * BPP);
		const int last_row = F.in_rows - 1;
		int issued = 0;
		bool ok = true;
		for(int q = 0; q < nq && ok && !F.starve; q++) {
			const int st = q % kBulkStages, use = q / kBulkStages;
			if(use > 0 && !mbar_wait(empty + st, (use - 1) & 1, F.wait_polls)) { ok = false; break; }
			if(*(volatile int *)abort_flag) { ok = false; break; }
			const int row = min(max(p0 + q, 0), last_row);
			mbar_expect_tx(full + st, bytes);
			bulk_g2s(ring + (size_t)st * STRIP, base + (unsigned long long)row * F.in_bpr, bytes, full + st);
			issued = q + 1;
		}
		if(!ok) {
			atomicExch(F.err_flag, 1);
			*(volatile int *)abort_flag = 1;
		}
		// every issued copy lands before the block's shared memory goes away
		for(int q = max(0, issued - kBulkStages); q < issued; q++) mbar_wait(full + q % kBulkStages, (q / kBulkStages) & 1);
		return;
	}

	// consumers
	const int x0 = threadIdx.x * PX;                  // first column of this thread (tile-local)
	const bool any = x0 < T.nc;
	const float ainv = F.alpha_inv;
	static_assert(PX == 2, "accumulators pair the thread's two pixels");
	static_assert(NS == 4, "one 16-byte load of the slot weights per row");
	unsigned long long acc[NS][NCH];
#pragma unroll
	for(int s = 0; s < NS; s++)
#pragma unroll
		for(int c = 0; c < NCH; c++) acc[s][c] = 0ULL;
	const int tw = T.i1 - T.i0;
	int pending = 0, jh = jb;                         // finished rows not yet summed horizontally, the first of them
	bool failed = false;

	// Horizontal sums + tail of the output pixels of rows jh .. jh + nrows - 1
	// (a consumer barrier first: their intermediate rows are complete).
	auto horizontal = [&](int nrows) {
		asm volatile("bar.sync 1, %0;" ::"n"(kBulkConsumers) : "memory");
		for(int k = threadIdx.x; k < nrows * tw; k += kBulkConsumers) {
			const int r = k / tw;
			const int j = jh + r, i = T.i0 + (k - r * tw);
			const float4 *row = mid + (size_t)(j % kFuseRows) * MIDW;
			float v[NCH], Tm[NCH];
#pragma unroll
			for(int c = 0; c < NCH; c++) { v[c] = 0.0f; Tm[c] = 0.0f; }
			const int t0 = __ldg(F.hoff + i), t1 = __ldg(F.hoff + i + 1);
			// blocked sums in hpass_pixel's order (partial sums of kHBlock taps)
			int t = t0;
			while(t < t1) {
				const int tb = min(t + kHBlock, t1);
				float pp[NCH];
#pragma unroll
				for(int c = 0; c < NCH; c++) pp[c] = 0.0f;
				for(; t < tb; t++) {
					const int src = __ldg(F.hsrc + t);
					if(src < 0) continue;   // transparent edge: value 0
					const float w = __ldg(F.hw + t), aw = fabsf(w);
					const float4 I4 = row[src - T.xa];
					const float I[4] = {I4.x, I4.y, I4.z, I4.w};
#pragma unroll
					for(int c = 0; c < NCH; c++) {
						pp[c] = __fmaf_rn(I[c], w, pp[c]);
						Tm[c] = __fmaf_rn(fabsf(I[c]), aw, Tm[c]);
					}
				}
#pragma unroll
				for(int c = 0; c < NCH; c++) v[c] = __fadd_rn(v[c], pp[c]);
			}
			hpass_tail<NCH>(F, i, j, v, Tm);
		}
	};

	for(int q = 0; q < nq; q++) {
		const int st = q % kBulkStages, use = q / kBulkStages;
		if(!failed && !mbar_wait(full + st, use & 1, F.wait_polls)) {
			atomicExch(F.err_flag, 1);
			*(volatile int *)abort_flag = 1;
			failed = true;   // keep to the barrier schedule; no more sums are taken
		}
		uint32_t cur[NW];
		{
			const uint4 v = reinterpret_cast<const uint4 *>(ring + (size_t)st * STRIP)[threadIdx.x];
			cur[0] = v.x; cur[1] = v.y; cur[2] = v.z; cur[3] = v.w;
		}
		__syncwarp();
		if(lane == 0 && !failed) mbar_arrive(empty + st);
		float val[PX][NCH], a[PX];
#pragma unroll
		for(int px = 0; px < PX; px++) {
			a[px] = 1.0f;
#pragma unroll
			for(int c = 0; c < NCH; c++) {
				const int sidx = px * NCH + c;
				unsigned int code;
				if(DEPTH == 8) code = __byte_perm(cur[sidx >> 2], 0u, 0x4440u + (sidx & 3));
				else code = __byte_perm(cur[sidx >> 1], 0u, (sidx & 1) ? 0x4423u : 0x4401u);
				if(ALPHA && c == NCH - 1) {
					a[px] = __fmul_rn(u2f(code), ainv);
					val[px][c] = a[px];
				}
				else val[px][c] = dec_table<DEPTH>(s_tab, code);
			}
		}
		unsigned long long v2[NCH];
#pragma unroll
		for(int c = 0; c < NCH; c++) v2[c] = f2_pack(val[0][c], val[1][c]);
		if(ALPHA) {
			const unsigned long long a2 = f2_pack(a[0], a[1]);
#pragma unroll
			for(int c = 0; c < NCH - 1; c++) v2[c] = f2_mul(v2[c], a2);   // premultiply
		}
		const float4 wq = *reinterpret_cast<const float4 *>(s_w + q * NS);
		const float wsv[4] = {wq.x, wq.y, wq.z, wq.w};
#pragma unroll
		for(int s = 0; s < NS; s++) {
			const unsigned long long w2 = f2_pack(wsv[s], wsv[s]);
#pragma unroll
			for(int c = 0; c < NCH; c++) acc[s][c] = f2_fma(v2[c], w2, acc[s][c]);
		}
		const int2 fin = s_fin[q];
		for(int k = 0; k < fin.y; k++) {
			const int j = fin.x + k;
			const int sj = j % NS;
			const bool keep = j >= jb && j < je;
#pragma unroll
			for(int s = 0; s < NS; s++) {
				if(s == sj) {
					if(keep && any) {
						float4 *o = mid + (size_t)(j % kFuseRows) * MIDW + x0;
						float lo[NCH], hi[NCH];
#pragma unroll
						for(int c = 0; c < NCH; c++) f2_unpack(acc[s][c], lo[c], hi[c]);
						o[0] = make_float4(lo[0], lo[1], lo[2], lo[3]);
						o[1] = make_float4(hi[0], hi[1], hi[2], hi[3]);
					}
#pragma unroll
					for(int c = 0; c < NCH; c++) acc[s][c] = 0ULL;
				}
			}
			if(keep && ++pending == 2) {
				if(!failed) horizontal(2);
				else asm volatile("bar.sync 1, %0;" ::"n"(kBulkConsumers) : "memory");
				jh += 2;
				pending = 0;
			}
		}
	}
	if(pending > 0) {
		if(!failed) horizontal(pending);
		else asm volatile("bar.sync 1, %0;" ::"n"(kBulkConsumers) : "memory");
	}
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
__device__ __forceinline__ void vstream_px_tile(const FJob &F, float *s_dyn, int bx, int band)
{
	constexpr int PF = 8;
	constexpr int BPP = NCH * (DEPTH / 8);
	constexpr int NW = PX * BPP / 4;              // 32-bit words per thread per row
	static_assert(PX * BPP % 4 == 0, "thread group must be whole words");
	float *s_tab = s_dyn;
	const int jb = band * F.rows_per_band;
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

	const int x0 = (bx * blockDim.x + threadIdx.x) * PX;
	if(x0 >= F.mid_w) return;
	const bool full = x0 + PX <= F.mid_w;
	const int valid_bytes = (F.mid_w - x0) * BPP;
	const uint8_t *colbase = F.in + (size_t)(F.crop_x + x0) * BPP + (unsigned long long)F.crop_y * F.in_bpr;
	const int last_row = F.in_rows - 1;
	const float ainv = F.alpha_inv;
	const unsigned long long bpr = F.in_bpr, plane = F.plane;
	const int mid_w = F.mid_w;
	float *const interm = F.interm;

	float acc[NS][PX][NCH];
#pragma unroll
	for(int s = 0; s < NS; s++)
#pragma unroll
		for(int px = 0; px < PX; px++)
#pragma unroll
			for(int c = 0; c < NCH; c++) acc[s][px][c] = 0.0f;

	auto load_row = [&](int p, uint32_t *w) {
		const int row = min(max(p, 0), last_row);
		const uint8_t *a = colbase + (unsigned long long)row * bpr;
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
			const uint32_t *cur = ring[u];
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
			// the row is decoded: its ring slot takes the row PF positions ahead
			if(pp + PF <= p1) load_row(pp + PF, ring[u]);
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
							float *o = interm + (unsigned long long)j * mid_w + x0;
#pragma unroll
							for(int px = 0; px < PX; px++) {
								if(full || x0 + px < mid_w) {
#pragma unroll
									for(int c = 0; c < NCH; c++) o[(unsigned long long)c * plane + px] = acc[s][px][c];
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
__device__ __forceinline__ void vgather_tile(const FJob &F, float *s_tab, int bx, int j)
{
	for(int k = threadIdx.x; k < F.dec_tab_floats; k += blockDim.x) s_tab[k] = F.dec_tab[k];
	__syncthreads();
	const int x = bx * blockDim.x + threadIdx.x;
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

// count_le_f for v in [0, 1], starting from the count at the start of v's
// cell (v * kLutCells is exact, so the cell's start is <= v) and stepping up.
__device__ __forceinline__ int count_le_lut(const float *t, int n, const float *lut, float v)
{
	const int cell = min(max((int)__fmul_rn(v, (float)kLutCells), 0), kLutCells - 1);
	int k = (int)__ldg(lut + cell);
	while(k < n && __ldg(t + k) <= v) k++;
	return k;
}

__device__ __forceinline__ int count_le_f(const float *t, int n, float v)
{
	int lo = 0, hi = n;
	while(lo < hi) {
		int mid = (lo + hi) >> 1;
		if(__ldg(t + mid) <= v) lo = mid + 1; else hi = mid;
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
		int c = count_le_lut(T.nc, 255, T.lut, v);
		if(c > 0 && !(T.nc[c - 1] < lo_v)) return -1;
		if(c < 255 && !(T.nc[c] > hi_v)) return -1;
		return c;
	}
	int k = count_le_lut(T.U + 1, T.P, T.lut, v);
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
	// one correctly rounded reciprocal for both quotients: f is within 1.5 ulp
	// (< 2e-7) of the rounded division, well inside the 1e-6 slack of mf
	const float rd = __frcp_rn(den);
	const float f = __fmul_rn(__fsub_rn(v, a), rd);
	const float mf = __fmaf_rn(__fmul_rn(__fmaf_rn(fabsf(a) + fabsf(b), 1.2e-7f, Ep), rd), 1.0000004f, 1e-6f);
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
__device__ __forceinline__ void hpass_tail(const FJob &F, int i, int j, const float (&v)[NPL], const float (&T)[NPL]);

// Horizontal pass + tail for output pixel (i, j).
template<int NPL>
__device__ __forceinline__ void hpass_pixel(const FJob &F, int i, int j)
{
	if(i >= F.out_w || j >= F.out_h) return;
	float v[NPL], T[NPL];
#pragma unroll
	for(int c = 0; c < NPL; c++) { v[c] = 0.0f; T[c] = 0.0f; }
	const int t0 = F.hoff[i], t1 = F.hoff[i + 1];
	const float *rowp[NPL];
#pragma unroll
	for(int c = 0; c < NPL; c++) rowp[c] = F.interm + (unsigned long long)c * F.plane + (unsigned long long)j * F.mid_w;
	// Taps are summed in blocks of kHBlock: a block's products are accumulated
	// into a partial sum (fused multiply-adds from 0) that is then added to the
	// total, so a product passes through at most kHBlock + ceil(n / kHBlock)
	// roundings instead of n (the host's bound uses that count).  Within a
	// block, four taps at a time: their sources, weights and samples are all
	// loaded before the first multiply-add, then accumulated in tap order.  A
	// transparent edge tap (source -1) reads column 0 and contributes 0.
	int t = t0;
	while(t < t1) {
		const int tb = min(t + kHBlock, t1);
		float p[NPL];
#pragma unroll
		for(int c = 0; c < NPL; c++) p[c] = 0.0f;
		for(; t + 4 <= tb; t += 4) {
			int src[4];
			float w[4], I[4][NPL];
#pragma unroll
			for(int u = 0; u < 4; u++) {
				src[u] = __ldg(F.hsrc + t + u);
				w[u] = __ldg(F.hw + t + u);
			}
#pragma unroll
			for(int u = 0; u < 4; u++) {
				const int sc = src[u] < 0 ? 0 : src[u];
#pragma unroll
				for(int c = 0; c < NPL; c++) I[u][c] = __ldg(rowp[c] + sc);
			}
#pragma unroll
			for(int u = 0; u < 4; u++) {
				const float aw = fabsf(w[u]);
#pragma unroll
				for(int c = 0; c < NPL; c++) {
					const float x = src[u] < 0 ? 0.0f : I[u][c];
					p[c] = __fmaf_rn(x, w[u], p[c]);
					T[c] = __fmaf_rn(fabsf(x), aw, T[c]);
				}
			}
		}
		for(; t < tb; t++) {
			const int src = __ldg(F.hsrc + t);
			if(src < 0) continue;   // transparent edge: value 0
			const float w = __ldg(F.hw + t), aw = fabsf(w);
#pragma unroll
			for(int c = 0; c < NPL; c++) {
				const float I = __ldg(rowp[c] + src);
				p[c] = __fmaf_rn(I, w, p[c]);
				T[c] = __fmaf_rn(fabsf(I), aw, T[c]);
			}
		}
#pragma unroll
		for(int c = 0; c < NPL; c++) v[c] = __fadd_rn(v[c], p[c]);
	}
	hpass_tail<NPL>(F, i, j, v, T);
}

// Horizontal pass for wide windows, a warp per output pixel (i, j): lane l
// accumulates taps l, l+32, ... (fused multiply-adds from 0), then a butterfly
// of five additions gives every lane the same total, so a product passes
// through at most ceil(n / 32) + 5 roundings (the host's bound uses that
// count).  Lane 0 decides the codes.
template<int NPL>
__device__ __forceinline__ void hpass_pixel_warp(const FJob &F, int i, int j, int lane)
{
	if(i >= F.out_w || j >= F.out_h) return;
	float v[NPL], T[NPL];
#pragma unroll
	for(int c = 0; c < NPL; c++) { v[c] = 0.0f; T[c] = 0.0f; }
	const int t0 = F.hoff[i], t1 = F.hoff[i + 1];
	const float *rowp[NPL];
#pragma unroll
	for(int c = 0; c < NPL; c++) rowp[c] = F.interm + (unsigned long long)c * F.plane + (unsigned long long)j * F.mid_w;
	for(int t = t0 + lane; t < t1; t += 32) {
		const int src = __ldg(F.hsrc + t);
		const float w = __ldg(F.hw + t), aw = fabsf(w);
		if(src < 0) continue;   // transparent edge: value 0
#pragma unroll
		for(int c = 0; c < NPL; c++) {
			const float I = __ldg(rowp[c] + src);
			v[c] = __fmaf_rn(I, w, v[c]);
			T[c] = __fmaf_rn(fabsf(I), aw, T[c]);
		}
	}
#pragma unroll
	for(int off = 16; off > 0; off >>= 1) {
#pragma unroll
		for(int c = 0; c < NPL; c++) {
			v[c] = __fadd_rn(v[c], __shfl_xor_sync(0xffffffffu, v[c], off));
			T[c] = __fadd_rn(T[c], __shfl_xor_sync(0xffffffffu, T[c], off));
		}
	}
	if(lane == 0) hpass_tail<NPL>(F, i, j, v, T);
}

// Quantisation tail of output pixel (i, j) from its horizontal sums v and
// their magnitude sums T (error bound E = K0 + K1 * T per plane).
template<int NPL>
__device__ __forceinline__ void hpass_tail(const FJob &F, int i, int j, const float (&v)[NPL], const float (&T)[NPL])
{
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
	float A = 0.0f, EA = 0.0f, rA = 0.0f, rden = 0.0f;
#pragma unroll
	for(int k = 0; k < dev::kMaxCh; k++) {
		codes[k] = -1;
		if(k >= F.mid_n || redo == all) continue;
		const int pl = F.k_plane[k];
		float val = 0.0f, err = 0.0f;
#pragma unroll
		for(int c = 0; c < NPL; c++) if(c == pl) { val = v[c]; err = E[c]; }
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
			if(rA == 0.0f) { rA = __frcp_rn(A); rden = __frcp_rn(den); }   // shared by the colour channels
			// q within 1.5 ulp of val/A; the bound's quotient rounded up by its own error
			const float q = __fmul_rn(val, rA);
			err = __fmul_rn(__fmul_rn(__fmaf_rn(fabsf(q), EA, err), rden), 1.0000004f);
			err = __fmaf_rn(fabsf(q), 2.4e-7f, err);
			val = q;
		}
		if(F.dbg) {
			const unsigned long long di = ((unsigned long long)F.k_out[k] * F.out_h + j) * F.out_w + i;
			const unsigned long long dn = (unsigned long long)F.out_n * F.out_h * F.out_w;
			F.dbg[di] = val;
			F.dbg[dn + di] = err;
		}
		const int c = quantize_guarded(F.k_tail[k], val, err, i, j);
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
		if(slot < F.flag_cap) reinterpret_cast<int4 *>(F.flag_list)[slot] = make_int4(j * F.out_w + i, (int)redo, F.img, 0);
		else atomicExch(F.err_flag, 2);   // more entries than pixels: never in a correct run
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



// Vertical kernel variant of a prepared image (which template instance).
struct VVariant {
	int kind = 0;    // 1: k_vstream_px, 2: k_vstream, 3: k_vgather, 4: k_vbulk
	int ns = 0, nch = 0, alpha = 0, depth = 0, px = 0;
	bool operator==(const VVariant &o) const
	{
		return kind == o.kind && ns == o.ns && nch == o.nch && alpha == o.alpha && depth == o.depth && px == o.px;
	}
};

// Host-side state of one prepared image of the fast form.
struct FastState {
	FJob F;
	Job J;
	const void *vkernel = nullptr, *hkernel = nullptr;
	dim3 vgrid, hgrid;
	int vthreads = kVThreads;
	size_t vsmem = 0;
	VVariant vv;
	// per-image arrays, laid out in 'blob' (copied to the device as one block)
	std::vector<uint8_t> blob;
	size_t o_hoff = 0, o_hsrc = 0, o_hw = 0, o_voff = 0, o_vsrc = 0, o_vw = 0;
	size_t o_fp = 0, o_lp = 0, o_src = 0, o_pi = 0, o_sw = 0;
	bool streaming = false;
	size_t flag_entries = 0;   // capacity of the flag list (one entry per output pixel)
	// double-float tier of the re-evaluation: tables (cached device copies)
	// and weights (in the blob)
	const float2 *df_tab[dev::kMaxCh] = {nullptr, nullptr, nullptr, nullptr};
	const float2 *df_atab = nullptr;
	size_t o_wvdf = 0, o_whdf = 0;
	bool df = false;
	// band tuning (fastpath.cu): the streaming schedule's windows (host
	// copies) and the vertical kernel's shared memory as a function of the
	// positions a band spans (vsmem = vsmem_fixed + positions * vsmem_per_pos)
	std::vector<int> first_pos, last_pos;
	size_t vsmem_fixed = 0, vsmem_per_pos = 0;
	bool in_device = false;
	// fused vertical + horizontal pass (k_vhfuse, vkernel; no hkernel): its
	// column tiles (device copy in the blob)
	bool fuse = false;
	size_t o_fuse = 0;
	const FuseTile *fuse_tiles = nullptr;
	// vertical pass on the tensor cores (tcvert.cu) instead of vkernel's FJob launch
	bool tc = false;
	tc::TcJob T;
	size_t o_tct = 0, o_tcb = 0, o_tcl = 0;
};

// Template instances of the vertical kernels, shared by the per-image and
// batch launchers: (NS, channels, alpha, depth, pixels per thread).
#define IWG_VPX_VARIANTS(X) \
	X(4, 4, true, 16, 2) X(6, 4, true, 16, 2) X(8, 4, true, 16, 2) \
	X(4, 3, false, 16, 2) X(6, 3, false, 16, 2) X(8, 3, false, 16, 2) \
	X(4, 2, true, 16, 4) X(6, 2, true, 16, 4) X(8, 2, true, 16, 4) \
	X(4, 1, false, 16, 8) X(6, 1, false, 16, 8) X(8, 1, false, 16, 8) \
	X(4, 4, true, 8, 2) X(6, 4, true, 8, 2) X(8, 4, true, 8, 2) \
	X(4, 3, false, 8, 4) X(6, 3, false, 8, 4) X(8, 3, false, 8, 4) \
	X(4, 2, true, 8, 4) X(6, 2, true, 8, 4) X(8, 2, true, 8, 4) \
	X(4, 1, false, 8, 8) X(6, 1, false, 8, 8) X(8, 1, false, 8, 8)
// Instances of the bulk-copy vertical kernel: (NS, channels, alpha, depth, PX)
// with one 16-byte group per consumer thread and row.
// (more slots or more pixels per thread spill registers at this block size)
#define IWG_VBULK_VARIANTS(X) X(4, 4, true, 16, 2)
// (NS, planes, depth)
#define IWG_VSTREAM_VARIANTS(X) \
	X(4, 1, 8) X(4, 2, 8) X(4, 3, 8) X(4, 4, 8) X(6, 1, 8) X(6, 2, 8) X(6, 3, 8) X(6, 4, 8) \
	X(8, 1, 8) X(8, 2, 8) X(8, 3, 8) X(8, 4, 8) \
	X(4, 1, 16) X(4, 2, 16) X(4, 3, 16) X(4, 4, 16) X(6, 1, 16) X(6, 2, 16) X(6, 3, 16) X(6, 4, 16) \
	X(8, 1, 16) X(8, 2, 16) X(8, 3, 16) X(8, 4, 16)
// (planes, depth)
#define IWG_VGATHER_VARIANTS(X) X(1, 8) X(2, 8) X(3, 8) X(4, 8) X(1, 16) X(2, 16) X(3, 16) X(4, 16)

}  // namespace fp
}  // namespace iwg
