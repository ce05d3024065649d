// tc_emul.cpp -- CPU check of the tensor-core vertical pass's host side
// (imageworsener_gb300/csrc/tcvert.cu tc_build): builds the digit tiles and the
// digit table for a real weight list, replays the digit-product sums the MMAs
// form (in the operand layout the kernel's descriptors describe) in exact
// arithmetic, recombines them as the kernel's epilogue does, and compares each
// result with the reference's double sum rounded to float.  Exit status 0 when
// every digit sum is an integer below 2^24 and every error is within the bound
// the error model uses: e_abs * 1.01 + (2u + gamma_(n+1)(2^-53)) * (|I| + 2 Wneg).
//
//   tc_emul <n_in> <n_out> [resize family] [p1] [columns]
#include "imagew.h"
#include "iwg_internal.h"
#include "tcvert.cuh"
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
using namespace iwg;
static int bf2int(uint16_t h) { uint32_t b = (uint32_t)h << 16; float f; memcpy(&f, &b, 4); return (int)f; }
int main(int argc, char **argv) {
	int n_in = argc > 1 ? atoi(argv[1]) : 8192, n_out = argc > 2 ? atoi(argv[2]) : 256;
	int fam = argc > 3 ? atoi(argv[3]) : IW_RESIZETYPE_LANCZOS;
	double p1 = argc > 4 ? atof(argv[4]) : 3.0;
	int cols = argc > 5 ? atoi(argv[5]) : 384;
	iw_context *ctx = iw_create_context(NULL);
	DimRequest d; d.family = fam; d.p1 = p1; d.p2 = 0; d.blur = 1.0; d.true_size = n_out;
	if(fam == IW_RESIZETYPE_CUBIC) { d.p1 = 1.0/3; d.p2 = 1.0/3; }
	auto W = build_weights(ctx, d, IW_CHANNELTYPE_RED, n_in, n_out, 0.0);
	if(!W) { printf("no weights\n"); return 1; }
	std::vector<double> tab(256);
	for(int c = 0; c < 256; c++) { double v = c / 255.0; tab[c] = v <= 0.04045 ? v / 12.92 : pow((v + 0.055) / 1.055, 2.4); }
	std::vector<const std::vector<double>*> tabs(3, &tab);
	tc::TcBuild B;
	if(!tc::tc_build(*W, n_in, 3, tabs, B)) { printf("tc_build refused\n"); return 1; }
	printf("S=%d nblk=%d nstages=%d e_abs=%.3e max_taps=%d W1=%.4f Wneg=%.4f\n", B.S, B.nblk, B.nstages, B.e_abs, W->max_taps, W->wsum_abs_max, W->wsum_neg_max);
	std::mt19937 rng(1);
	std::vector<uint8_t> img((size_t)n_in * cols);
	for(auto &v : img) v = rng() & 255;
	const double u = 1.0 / 16777216.0, ud = 1.0 / 9007199254740992.0;
	double nv = W->max_taps;
	double g = (nv + 1) * ud / (1 - (nv + 1) * ud);
	double c1 = (2 * u + g) * 1.01;
	double worst = 0, maxerr = 0; long long bad = 0, nonint = 0, big = 0;
	for(int c = 0; c < cols; c++) {
		int ch = c % 3;
		for(int b = 0; b < B.nblk; b++) {
			double D[128]; for(auto &x : D) x = 0;
			for(int t = B.blk[b].x; t < B.blk[b].y; t++) {
				const uint8_t *tile = B.tiles.data() + ((size_t)t * 2 + (b & 1)) * tc::kTileBytes;
				for(int kk = 0; kk < 32; kk++) {
					int k = std::min(t * 32 + kk, n_in - 1);
					uint2 L = B.lut[ch * 256 + img[(size_t)k * cols + c]];
					int X[3] = {bf2int(L.x & 0xffff), bf2int(L.x >> 16), bf2int(L.y & 0xffff)};
					for(int p = 0; p < 3; p++) {
						int N = p < 2 ? 48 : 32;
						for(int n = 0; n < N; n++) {
							size_t off = (size_t)(n >> 3) * 512 + (kk >> 3) * 128 + (n & 7) * 16 + (kk & 7) * 2;
							uint16_t h; memcpy(&h, tile + off, 2);
							D[p * 48 + n] += (double)X[p] * bf2int(h);
							if(fabs(D[p * 48 + n]) >= 16777216.0) big++;
						}
					}
				}
			}
			for(int r = 0; r < 16; r++) {
				int j = b * 16 + r; if(j >= n_out) break;
				const int colq[8] = {0, 16, 32, 48, 64, 80, 96, 112};
				const int sh[8] = {32, 24, 16, 24, 16, 8, 16, 8};
				long long acc = 0;
				for(int q = 0; q < 8; q++) { double v = D[colq[q] + r]; if(v != floor(v)) nonint++; acc += (long long)v * (1LL << sh[q]); }
				float I = (float)acc * B.scale;
				double S = 0.0;
				for(int t = W->off[j]; t < W->off[j + 1]; t++) { double pr = tab[img[(size_t)W->src[t] * cols + c]] * W->w[t]; S = S + pr; }
				float Iref = (float)S;
				double err = fabs((double)I - (double)Iref);
				double bound = B.e_abs * 1.01 + c1 * (fabs(I) + 2 * W->wsum_neg_max);
				maxerr = std::max(maxerr, err); worst = std::max(worst, err / bound);
				if(err > bound) bad++;
			}
		}
	}
	printf("max |I'-Iref| = %.3e  worst err/bound = %.3f  violations=%lld nonint=%lld over2^24=%lld\n", maxerr, worst, bad, nonint, big);
	return bad || nonint || big;
}
