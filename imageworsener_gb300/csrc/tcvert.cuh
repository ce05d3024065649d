// tcvert.cuh -- vertical pass of the FP32 + guard-band form on the tensor
// cores (tcgen05), for 8-bit inputs whose columns are decoded through a table
// (no alpha).  Used for downscales, where each output row sums tens to
// hundreds of input rows and the pass is a block-banded matrix product:
//
//     I[j][c] = sum_k W[j][k] * x[k][c]     (j: output row, k: input row, c: byte column)
//
// Exact integer arithmetic on bf16 operands.  Each decoded sample x (a double
// in [0,1] from the reference's input table) is held as the 24-bit fixed-point
// integer X = round(x * 2^24) and each weight as W = round(w * 2^S) (S chosen
// per image so |W| < 2^23).  Both are split into 8-bit digits,
//     X = X2*2^16 + X1*2^8 + X0          (0 <= X2 <= 256, 0 <= X1, X0 <= 255)
//     W = W2*2^16 + W1*2^8 + W0          (balanced: -128 <= W1, W0 <= 127, |W2| <= 128)
// every digit is an integer of at most 9 significant bits, exact in bf16, and
// every digit product is exact in FP32.  A column's sum of digit products
// over one output row's window (at most 511 taps) stays below 2^24 in
// magnitude, so every partial sum the tensor core forms is an integer that
// FP32 holds exactly, whatever order or rounding the hardware uses for its
// additions.  The epilogue recombines the eight digit-product sums used (the
// X0*W0 sum, below 2^-(9+S) per tap, is dropped and bounded) in 64-bit
// integers and rounds once to float.  The result's error against the
// reference's double sum comes only from the fixed-point quantisation of x
// and w, which the host bounds per image (TcBuild::e_abs).
//
// MMA layout (cta_group::1, kind::f16 with bf16 operands, FP32 accumulators):
//   A = decoded input, M = 128 byte columns of a strip, K = 32 input rows per
//       stage; three A operands per stage, one per X digit, written by 8
//       decoding warps (2 columns x 8 rows per thread, one 16-byte core-matrix
//       row per column and digit) from a digit table split into a 4-byte
//       (X2, X1) and a 2-byte (X0) part, whose lookups rarely collide on a bank.
//   B = weights, N = 48 rows: the W2, W1, W0 digits of 16 output rows (a
//       block).  The X0 operand uses the first 32 (W2, W1) only.
//   D = TMEM, 128 lanes (columns) x 128 FP32 columns per block: the sums
//       X2*(W2,W1,W0), X1*(W2,W1,W0), X0*(W2,W1), 16 output rows each.
// Both operands are K-major in the canonical no-swizzle layout: 8 x 16-byte
// core matrices, K-adjacent core matrices 128 bytes apart (leading byte
// offset), 8-row groups 528 (A) or 512 (B) bytes apart (stride byte offset;
// the 16 spare bytes per group of A spread a warp's transposing 16-byte
// stores over all shared-memory banks).
#pragma once

#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

namespace iwg {

struct Weights;

namespace tc {

constexpr int kRows = 32;                  // input rows per stage (two K = 16 MMA steps)
constexpr int kM = 128;                    // byte columns per strip
constexpr int kR = 16;                     // output rows per block
constexpr int kStages = 3;                 // stages in flight
constexpr int kSboA = 528;                 // A: bytes between 8-row groups (512 + 16: conflict-free stores)
constexpr int kPieceBytes = (kM / 8) * kSboA;  // one X digit of a stage: 8448
constexpr int kTileBytes = 48 * kRows * 2;      // one block's W digits of a stage: 3072
constexpr int kTmemCols = 256;             // two live blocks of 128 columns
constexpr int kThreads = 256;             // 8 warps: warp w decodes rows 8(w/2).. of 64 columns of a stage

struct TcJob {
	const uint8_t *in;            // input at the crop origin
	unsigned long long in_bpr;
	int in_rows;                  // crop height
	int cols;                     // byte columns: crop width * channels
	int nphys;                    // channels per pixel (1 byte each)
	int mid_w, mid_h;
	float *interm;                // planar float intermediate, plane c = channel c
	unsigned long long plane;     // floats per plane
	const uint2 *lut;             // nphys * 256: bf16 digits (X2 | X1 << 16, X0) per code
	const int4 *blk;              // per block: first stage, end stage
	const uint4 *tiles;           // per stage: 2 x kTileBytes (block parity 0, 1)
	int nblk, blocks_per_band;
	float scale;                  // 2^-(24+S)
	int *err_flag;                // set when a bounded wait runs out
};

// Host preparation.  Fills the per-image arrays and the error bound; false if
// the weights do not fit the scheme (virtual taps, non-monotone windows, more
// than two blocks open at once, windows of 512 or more rows).
struct TcBuild {
	std::vector<uint8_t> tiles;   // nstages * 2 * kTileBytes
	std::vector<int4> blk;        // nblk
	std::vector<uint2> lut;       // nphys * 256
	float scale = 0.0f;
	int S = 0;
	int nblk = 0, nstages = 0;
	double e_abs = 0.0;           // |I_tc - sum x*w| bound (before float rounding), absolute
};

// 'tabs' holds, per channel, the 256 doubles the reference decodes codes to.
bool tc_build(const Weights &WV, int in_rows, int nphys, const std::vector<const std::vector<double> *> &tabs,
	TcBuild &out);

// Launch geometry for a prepared image on 'sms' multiprocessors (two blocks
// per multiprocessor): strips x bands, the bands 'blocks_per_band' blocks tall.
void tc_geometry(const TcBuild &B, int cols, int sms, int &strips, int &bands, int &blocks_per_band);

size_t tc_smem_bytes(int nphys);
// k_vtc, for cudaLaunchKernel with a TcJob argument; 'vec': the input at the
// crop origin and its row stride are 2-byte aligned (16-bit loads)
const void *tc_kernel(bool vec);

}  // namespace tc
}  // namespace iwg
