// tcvert.cu -- vertical pass on the tensor cores (tcgen05, TMEM), exact
// integer digit products on bf16 operands.  The scheme, the operand layouts
// and the error bound are described in tcvert.cuh.
#include "tcvert.cuh"
#include "iwg_internal.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>

namespace iwg {
namespace tc {
namespace {

// ---------------------------------------------------------------------------
// inline PTX wrappers (sm_100 family)
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned saddr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void bar_init(unsigned long long *b, unsigned count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(b)), "r"(count) : "memory");
}

// Waits for the phase of 'parity' to complete; false after a bounded number
// of polls (each poll may suspend the thread for a short time).
__device__ __forceinline__ bool bar_wait(unsigned long long *b, unsigned parity)
{
	for(int it = 0; it < (1 << 21); it++) {
		unsigned done;
		asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
			: "=r"(done) : "r"(saddr(b)), "r"(parity) : "memory");
		if(done) return true;
	}
	return false;
}

__device__ __forceinline__ void tmem_alloc(unsigned *slot, unsigned ncols)
{
	asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(slot)), "r"(ncols) : "memory");
	asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_free(unsigned taddr, unsigned ncols)
{
	asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes -> visible to the tensor core (async proxy)
__device__ __forceinline__ void proxy_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Shared-memory matrix descriptor: canonical K-major layout without swizzle,
// K-adjacent core matrices 128 bytes apart, 8-row groups 'sbo' bytes apart,
// descriptor version 1 (bits 46-47).
__device__ __forceinline__ unsigned long long sdesc(unsigned addr, unsigned sbo)
{
	return (unsigned long long)((addr >> 4) & 0x3FFFu) | ((unsigned long long)(128u >> 4) << 16) |
		((unsigned long long)(sbo >> 4) << 32) | (1ull << 46);
}

// Instruction descriptor, kind::f16: FP32 accumulator (bits 4-5 = 1), A and B
// bf16 (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr unsigned idesc(int n)
{
	return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(n >> 3) << 17) | ((unsigned)(kM >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(unsigned d, unsigned long long a, unsigned long long b, unsigned id, int accumulate)
{
	asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
		"tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
		::"r"(d), "l"(a), "l"(b), "r"(id), "r"(accumulate) : "memory");
}

// Arrives on 'b' once every tcgen05 operation this thread issued so far is done.
__device__ __forceinline__ void mma_commit(unsigned long long *b)
{
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(b)) : "memory");
}

// 16 consecutive 32-bit TMEM columns of this thread's lane; the wait takes the
// registers as operands so no use of them can move above it.
__device__ __forceinline__ void tmem_ld16(unsigned taddr, uint32_t (&v)[16])
{
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
		: "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
		  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
		: "r"(taddr) : "memory");
	asm volatile("tcgen05.wait::ld.sync.aligned;"
		: "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3]), "+r"(v[4]), "+r"(v[5]), "+r"(v[6]), "+r"(v[7]),
		  "+r"(v[8]), "+r"(v[9]), "+r"(v[10]), "+r"(v[11]), "+r"(v[12]), "+r"(v[13]), "+r"(v[14]), "+r"(v[15])
		:: "memory");
}

__device__ __forceinline__ void tmem_ld8(unsigned taddr, uint32_t (&v)[8])
{
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
		: "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
		: "r"(taddr) : "memory");
	asm volatile("tcgen05.wait::ld.sync.aligned;"
		: "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3]), "+r"(v[4]), "+r"(v[5]), "+r"(v[6]), "+r"(v[7])
		:: "memory");
}

// ---------------------------------------------------------------------------
// kernel
// ---------------------------------------------------------------------------

// This thread's codes for one stage: its 2 byte columns (from cbase) in the
// 8 input rows from row0, one row per element (column cbase in bits 0-7,
// cbase + 1 in bits 8-15; rows past the crop repeat the last row, their
// weights are zero).  Columns past the image read as code 0 (their results
// are never stored).  VEC: the two bytes are one aligned 16-bit word.
template<bool VEC>
__device__ __forceinline__ void load_words(uint32_t (&raw)[8], const TcJob &T, int cbase, bool full, int row0)
{
	const int last = T.in_rows - 1;
	const uint8_t *base = T.in + cbase;
#pragma unroll
	for(int r = 0; r < 8; r++) {
		const uint8_t *p = base + (unsigned long long)min(row0 + r, last) * T.in_bpr;
		if(VEC && full) raw[r] = __ldg(reinterpret_cast<const unsigned short *>(p));
		else {
			uint32_t w = 0;
#pragma unroll
			for(int c = 0; c < 2; c++)
				if(cbase + c < T.cols) w |= (uint32_t)__ldg(p + c) << (8 * c);
			raw[r] = w;
		}
	}
}

// This thread's share of a stage's two weight tiles (2 * 3072 bytes = 384 x
// 16 bytes): pieces tid and tid + 256 (the second for tid < 128 only).
constexpr int kTilePieces = 2 * kTileBytes / 16;
__device__ __forceinline__ void load_tiles(uint4 (&bt)[2], const uint4 *tiles, int stage, int tid)
{
	const uint4 *g = tiles + (size_t)stage * kTilePieces;
	bt[0] = __ldg(g + tid);
	bt[1] = tid + kThreads < kTilePieces ? __ldg(g + tid + kThreads) : make_uint4(0, 0, 0, 0);
}

// Digit-product sums of block b -> float intermediate: this thread's byte
// column (TMEM lane) and output rows 8h..8h+7 of the block (h = warp / 4;
// warps w and w + 4 share lanes 32(w % 4)..).  Columns 0..127 of the block's
// TMEM region hold X2*(W2,W1,W0), X1*(W2,W1,W0), X0*(W2,W1), 16 rows each;
// the weights of the digit products are 2^(8*(i+j)) with the digits' positions i, j.
__device__ __forceinline__ void write_block(const TcJob &T, unsigned tmem, int b, int warp, int col, bool colok, int ch)
{
	const int h = warp >> 2;
	const unsigned base = tmem + ((unsigned)((warp & 3) * 32) << 16) + (unsigned)(b & 1) * 128u + (unsigned)h * 8u;
	long long acc[8];
#pragma unroll
	for(int r = 0; r < 8; r++) acc[r] = 0;
#pragma unroll
	for(int q = 0; q < 8; q++) {
		uint32_t v[8];
		tmem_ld8(base + q * 16, v);
		const int sh = q == 0 ? 32 : ((q == 1 || q == 3) ? 24 : ((q == 5 || q == 7) ? 8 : 16));
#pragma unroll
		for(int r = 0; r < 8; r++) acc[r] += (long long)__float2int_rz(__uint_as_float(v[r])) * (1LL << sh);
	}
	if(!colok) return;
	float *o = T.interm + (unsigned long long)ch * T.plane + col / T.nphys;
#pragma unroll
	for(int r = 0; r < 8; r++) {
		const int j = b * kR + h * 8 + r;
		if(j < T.mid_h) o[(unsigned long long)j * T.mid_w] = __fmul_rn(__ll2float_rn(acc[r]), T.scale);
	}
}

template<bool VEC>
__global__ void __launch_bounds__(kThreads, 2) k_vtc(const __grid_constant__ TcJob T)
{
	extern __shared__ __align__(128) unsigned char smem[];
	unsigned char *sA = smem;                                   // kStages x 3 digits x kPieceBytes
	unsigned char *sB = sA + kStages * 3 * kPieceBytes;         // kStages x 2 tiles x kTileBytes
	// digit table split in two so that nearby codes fall on different banks
	// (or share a word): X2 | X1 << 16 (4 bytes), X0 (2 bytes)
	uint32_t *sLutHi = reinterpret_cast<uint32_t *>(sB + kStages * 2 * kTileBytes);
	unsigned short *sLutLo = reinterpret_cast<unsigned short *>(sLutHi + T.nphys * 256);
	unsigned long long *bar = reinterpret_cast<unsigned long long *>(sLutLo + T.nphys * 256);
	unsigned *s_tmem = reinterpret_cast<unsigned *>(bar + kStages);
	int *s_abort = reinterpret_cast<int *>(s_tmem + 1);

	const int tid = threadIdx.x, warp = tid >> 5;
	const int b0 = blockIdx.y * T.blocks_per_band;
	const int b1 = min(b0 + T.blocks_per_band, T.nblk);
	if(b0 >= b1) return;                                        // whole block, before any allocation

	for(int k = tid; k < T.nphys * 256; k += kThreads) {
		const uint2 e = T.lut[k];
		sLutHi[k] = e.x;
		sLutLo[k] = (unsigned short)e.y;
	}
	if(tid == 0) {
		for(int s = 0; s < kStages; s++) bar_init(bar + s, 1);
		*s_abort = 0;
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	if(warp == 0) tmem_alloc(s_tmem, kTmemCols);
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const unsigned tmem = *s_tmem;

	// epilogue: thread tid owns TMEM lane 32 (warp % 4) + lane = byte column col
	const int col = blockIdx.x * kM + (warp & 3) * 32 + (tid & 31);
	const bool colok = col < T.cols;
	const int ch = colok ? col % T.nphys : 0;
	// decode: warp w takes rows 8(w / 2)..+7 of each stage and the 64 byte
	// columns (w % 2) * 64.. of the strip, lane l two of them (one 64-byte
	// segment per row and warp); each (column, 8 rows) is one 16-byte
	// core-matrix row per digit
	const int lane = tid & 31;
	const int rg = warp >> 1;
	const int m0 = (warp & 1) * 64 + lane * 2;          // first of the thread's columns in the strip
	const int cbase = blockIdx.x * kM + m0;
	const bool full = cbase + 1 < T.cols;
	int lofs[2];
#pragma unroll
	for(int c = 0; c < 2; c++) lofs[c] = ((cbase + c) % T.nphys) * 256;
	const int t0 = T.blk[b0].x, t1 = T.blk[b1 - 1].y;

	uint32_t raw[8];
	uint4 bt[2];
	load_words<VEC>(raw, T, cbase, full, t0 * kRows + rg * 8);
	load_tiles(bt, T.tiles, t0, tid);
	int done_b = b0;       // first block of the band not yet written out
	int issued = -1;       // last stage whose operations were committed
	bool pending = false;  // operations of 'issued' not yet seen complete
	for(int t = t0; t < t1; t++) {
		const int i = t - t0, s = i % kStages, use = i / kStages;
		uint32_t nraw[8];
		uint4 nbt[2];
		if(t + 1 < t1) {
			load_words<VEC>(nraw, T, cbase, full, (t + 1) * kRows + rg * 8);
			load_tiles(nbt, T.tiles, t + 1, tid);
		}
		// the stage buffer is free once the MMAs that read it (kStages stages ago) are done
		if(use > 0 && !bar_wait(bar + s, (use - 1) & 1)) {
			atomicExch(T.err_flag, 1);
			*(volatile int *)s_abort = 1;
		}
		// per column: the 8 rows' digits as one core-matrix row (16 bytes) per digit
		unsigned char *A = sA + s * 3 * kPieceBytes;
		uint32_t hi[2][8], lo[2][8];   // all 32 table lookups of the stage first (independent)
#pragma unroll
		for(int c = 0; c < 2; c++)
#pragma unroll
			for(int q = 0; q < 8; q++) {
				const int code = lofs[c] + (int)__byte_perm(raw[q], 0u, 0x4440u + c);
				hi[c][q] = sLutHi[code];
				lo[c][q] = sLutLo[code];
			}
#pragma unroll
		for(int c = 0; c < 2; c++) {
			uint4 d2, d1, d0;
			d2.x = __byte_perm(hi[c][0], hi[c][1], 0x5410); d2.y = __byte_perm(hi[c][2], hi[c][3], 0x5410);
			d2.z = __byte_perm(hi[c][4], hi[c][5], 0x5410); d2.w = __byte_perm(hi[c][6], hi[c][7], 0x5410);
			d1.x = __byte_perm(hi[c][0], hi[c][1], 0x7632); d1.y = __byte_perm(hi[c][2], hi[c][3], 0x7632);
			d1.z = __byte_perm(hi[c][4], hi[c][5], 0x7632); d1.w = __byte_perm(hi[c][6], hi[c][7], 0x7632);
			d0.x = __byte_perm(lo[c][0], lo[c][1], 0x5410); d0.y = __byte_perm(lo[c][2], lo[c][3], 0x5410);
			d0.z = __byte_perm(lo[c][4], lo[c][5], 0x5410); d0.w = __byte_perm(lo[c][6], lo[c][7], 0x5410);
			const int m = m0 + c;
			const int off = (m >> 3) * kSboA + rg * 128 + (m & 7) * 16;
			*reinterpret_cast<uint4 *>(A + off) = d2;
			*reinterpret_cast<uint4 *>(A + kPieceBytes + off) = d1;
			*reinterpret_cast<uint4 *>(A + 2 * kPieceBytes + off) = d0;
		}
		uint4 *Bs = reinterpret_cast<uint4 *>(sB + s * 2 * kTileBytes);
		Bs[tid] = bt[0];
		if(tid + kThreads < kTilePieces) Bs[tid + kThreads] = bt[1];
		proxy_fence();
		__syncthreads();
		if(*(volatile int *)s_abort) break;
		if(tid == 0) {
			tc_fence_after();
			const unsigned a0 = saddr(A);
			for(int b = done_b; b < b1; b++) {
				const int4 bi = T.blk[b];
				if(bi.x > t) break;
				const unsigned d = tmem + (unsigned)(b & 1) * 128u;
				const unsigned bs = saddr(sB + (s * 2 + (b & 1)) * kTileBytes);
#pragma unroll
				for(int ks = 0; ks < 2; ks++) {
					const unsigned long long bd = sdesc(bs + ks * 256, 512);
					const int acc = (t != bi.x || ks) ? 1 : 0;
					mma_bf16(d, sdesc(a0 + ks * 256, kSboA), bd, idesc(48), acc);
					mma_bf16(d + 48, sdesc(a0 + kPieceBytes + ks * 256, kSboA), bd, idesc(48), acc);
					mma_bf16(d + 96, sdesc(a0 + 2 * kPieceBytes + ks * 256, kSboA), bd, idesc(32), acc);
				}
			}
			mma_commit(bar + s);
		}
		__syncwarp();
		issued = t;
		pending = true;
		// blocks whose last stage this was: wait for the stage, read TMEM, write rows
		bool waited = false;
		while(done_b < b1 && T.blk[done_b].y - 1 == t) {
			if(!waited) {
				if(!bar_wait(bar + s, use & 1)) {
					atomicExch(T.err_flag, 1);
					*(volatile int *)s_abort = 1;
				}
				tc_fence_after();
				waited = true;
				pending = false;
			}
			write_block(T, tmem, done_b, warp, col, colok, ch);
			done_b++;
		}
		if(waited) tc_fence_before();    // TMEM reads ordered before the next barrier and the MMAs after it
#pragma unroll
		for(int k = 0; k < 8; k++) raw[k] = nraw[k];
		bt[0] = nbt[0];
		bt[1] = nbt[1];
	}
	// A stop on a timed-out wait can leave committed operations running: wait
	// (bounded) for the last commit before the tensor memory is released.
	if(pending && issued >= t0) {
		const int i = issued - t0;
		bar_wait(bar + i % kStages, (i / kStages) & 1);
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	if(warp == 0) tmem_free(tmem, kTmemCols);
}

uint16_t bf16_of_int(int v)
{
	const float f = (float)v;   // |v| <= 256: exact, and exact in bf16
	uint32_t b;
	memcpy(&b, &f, 4);
	return (uint16_t)(b >> 16);
}

}  // namespace

size_t tc_smem_bytes(int nphys)
{
	return (size_t)kStages * 3 * kPieceBytes + (size_t)kStages * 2 * kTileBytes + (size_t)nphys * 256 * 6 +
		kStages * 8 + 16;
}

const void *tc_kernel(bool vec) { return vec ? (const void *)k_vtc<true> : (const void *)k_vtc<false>; }

bool tc_build(const Weights &WV, int in_rows, int nphys, const std::vector<const std::vector<double> *> &tabs,
	TcBuild &B)
{
	if(WV.kind != RowKind::Sum) return false;
	const int n = WV.n_out;
	if(n <= 0 || in_rows <= 0 || nphys < 1 || nphys > 4 || (int)tabs.size() != nphys) return false;

	// largest per-source sum of |w| in one row; entries and distinct sources per row
	std::vector<int> mark(in_rows, -1);
	std::vector<double> absum(in_rows, 0.0);
	double wmax = 0.0;
	int ent_max = 0, nz_max = 0;
	for(int j = 0; j < n; j++) {
		int nz = 0;
		for(int t = WV.off[j]; t < WV.off[j + 1]; t++) {
			const int k = WV.src[t];
			if(k < 0 || k >= in_rows || !std::isfinite(WV.w[t])) return false;
			if(mark[k] != j) { mark[k] = j; absum[k] = 0.0; nz++; }
			absum[k] += std::fabs(WV.w[t]);
			wmax = std::max(wmax, absum[k]);
		}
		ent_max = std::max(ent_max, WV.off[j + 1] - WV.off[j]);
		nz_max = std::max(nz_max, nz);
	}
	if(wmax <= 0.0 || nz_max >= 512) return false;
	int S = (int)std::floor(std::log2((8388608.0 - 65536.0) / wmax));
	S = std::min(S, 100);
	while(std::ldexp(wmax, S) + 0.5 * ent_max > 8388608.0 - 32768.0) S--;

	// blocks of 16 output rows: stage ranges
	const int nstages = (in_rows + kRows - 1) / kRows;
	const int nblk = (n + kR - 1) / kR;
	B.blk.assign(nblk, make_int4(0, 0, 0, 0));
	for(int b = 0; b < nblk; b++) {
		int klo = INT32_MAX, khi = -1;
		for(int j = b * kR; j < std::min(n, (b + 1) * kR); j++)
			for(int t = WV.off[j]; t < WV.off[j + 1]; t++) { klo = std::min(klo, WV.src[t]); khi = std::max(khi, WV.src[t]); }
		if(khi < 0) return false;
		B.blk[b] = make_int4(klo / kRows, (khi + kRows) / kRows, 0, 0);
		if(b > 0 && (B.blk[b].x < B.blk[b - 1].x || B.blk[b].y < B.blk[b - 1].y)) return false;
		if(b >= 2 && B.blk[b].x < B.blk[b - 2].y) return false;   // at most two blocks open at once
	}

	// weight tiles: per stage, one tile per block parity
	B.tiles.assign((size_t)nstages * 2 * kTileBytes, 0);
	std::vector<long long> wint(in_rows, 0);
	for(int j = 0; j < n; j++) {
		for(int t = WV.off[j]; t < WV.off[j + 1]; t++) wint[WV.src[t]] = 0;
		for(int t = WV.off[j]; t < WV.off[j + 1]; t++) wint[WV.src[t]] += std::llround(std::ldexp(WV.w[t], S));
		const int b = j / kR, r = j % kR;
		for(int t = WV.off[j]; t < WV.off[j + 1]; t++) {
			const int k = WV.src[t];
			const long long W = wint[k];
			if(W == LLONG_MIN) continue;          // written already (repeated source)
			wint[k] = LLONG_MIN;
			const int d0 = (int)(((W & 255) ^ 128) - 128);
			const long long W1r = (W - d0) / 256;
			const int d1 = (int)(((W1r & 255) ^ 128) - 128);
			const long long d2 = (W1r - d1) / 256;
			if(d2 < -128 || d2 > 128) return false;
			const int st = k / kRows, kk = k % kRows;
			uint8_t *tile = B.tiles.data() + ((size_t)st * 2 + (b & 1)) * kTileBytes;
			const int digit[3] = {(int)d2, d1, d0};
			for(int q = 0; q < 3; q++) {
				const int nrow = q * kR + r;
				const size_t off = (size_t)(nrow >> 3) * 512 + (kk >> 3) * 128 + (nrow & 7) * 16 + (kk & 7) * 2;
				const uint16_t h = bf16_of_int(digit[q]);
				memcpy(tile + off, &h, 2);
			}
		}
	}

	// decode table: bf16 digits of X = round(x * 2^24)
	double e_x = 0.0;
	B.lut.assign((size_t)nphys * 256, make_uint2(0, 0));
	for(int c = 0; c < nphys; c++) {
		const std::vector<double> &tab = *tabs[c];
		if(tab.size() < 256) return false;
		for(int code = 0; code < 256; code++) {
			const double x = tab[code];
			if(!(x >= 0.0 && x <= 1.0)) return false;
			const long long X = std::llround(std::ldexp(x, 24));
			e_x = std::max(e_x, std::fabs(std::ldexp((double)X, -24) - x));
			const int x2 = (int)(X >> 16), x1 = (int)((X >> 8) & 255), x0 = (int)(X & 255);
			B.lut[(size_t)c * 256 + code] = make_uint2((uint32_t)bf16_of_int(x2) | ((uint32_t)bf16_of_int(x1) << 16),
				(uint32_t)bf16_of_int(x0));
		}
	}

	// |sum X*W*2^-(24+S) - sum x*w| <= e_x*W1 + (entries)*2^-(S+1) + (sources)*255*128*2^-(24+S) + cross term
	const double q_w = std::ldexp(1.0, -(S + 1));
	const double W1 = std::max(WV.wsum_abs_max, 0.0);
	B.e_abs = (e_x * W1 + ent_max * q_w + nz_max * 255.0 * 128.0 * std::ldexp(1.0, -(24 + S)) + e_x * ent_max * q_w) * 1.01;
	B.S = S;
	B.scale = std::ldexp(1.0f, -(24 + S));
	B.nblk = nblk;
	B.nstages = nstages;
	return true;
}

void tc_geometry(const TcBuild &B, int cols, int sms, int &strips, int &bands, int &bpb)
{
	strips = (cols + kM - 1) / kM;
	const long long slots = 2LL * std::max(1, sms);
	double best = 1e300;
	bpb = B.nblk;
	for(int bb = 1; bb <= B.nblk; bb++) {
		const int nb = (B.nblk + bb - 1) / bb;
		int maxst = 0;
		for(int q = 0; q < nb; q++) {
			const int lo = q * bb, hi = std::min(lo + bb, B.nblk);
			maxst = std::max(maxst, B.blk[hi - 1].y - B.blk[lo].x);
		}
		const long long ctas = (long long)strips * nb;
		const double cost = (double)((ctas + slots - 1) / slots) * maxst;
		if(cost < best) { best = cost; bpb = bb; }
	}
	bands = (B.nblk + bpb - 1) / bpb;
}

}  // namespace tc
}  // namespace iwg
