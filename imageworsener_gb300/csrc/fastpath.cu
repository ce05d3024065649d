// fastpath.cu -- FP32 + guard-band form of the pixel pipeline.
//
// The vertical and horizontal resampling run in FP32.  Every output sample
// carries a rigorous bound E on |v_fp32 - v_ref|, where v_ref is the value the
// reference computes in double precision (with its float intermediate).  The
// quantisation tail then decides the output code for the whole interval
// [v - E, v + E]; if a decision boundary of the reference (a code bracket
// edge, a nearest-colour midpoint, an ordered-dither threshold) lies inside,
// the pixel is flagged and re-evaluated by the fix-up kernels (pipeline.cu:
// certified double-float, then FP64).  Output bytes therefore equal the plain form's.
//
// Error bound (u = 2^-24, per pass with n taps and weights w):
//   decode   |a' - a| <= e_dec + r_dec * a          (e_dec measured over every code)
//   vertical |I' - I_ref| <= e_dec*W1v + c1 * (|I'| + 2*Wneg_v)
//   horizontal |v' - v_ref| <= K0 + K1 * sum_k |I'_k||w_k|
// with c1 = (r_dec + 2u + gamma_nv + gamma_nv^(fp64)), the horizontal sum's
// c2 = (u + gamma_(b+nb+1) + gamma_nh^(fp64)) for blocks of b = min(nh, kHBlock)
// taps (nb = ceil(nh / kHBlock) partial sums), and K0, K1 assembled on
// the host below; unassociating alpha divides by the float alpha, whose own
// bound is propagated.
#include "iwg_internal.h"
#include "device.cuh"
#include "fastkern.cuh"
#include "fastpath.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

namespace iwg {

using namespace dev;

void launch_fix_flagged(cudaStream_t st, const Job &J, int *count, int *list, int cap);

namespace {

using namespace fp;

template<int NS, int NPL, int DEPTH>
__global__ void __launch_bounds__(kVThreads) k_vstream(FJob F)
{
	extern __shared__ __align__(16) float s_tab[];
	vstream_tile<NS, NPL, DEPTH>(F, s_tab, blockIdx.x, blockIdx.y);
}

template<int NS, int NCH, bool ALPHA, int DEPTH, int PX>
__global__ void __launch_bounds__(kBulkThreads, 2) k_vbulk(FJob F)
{
	extern __shared__ __align__(128) unsigned char s_bulk[];
	vbulk_tile<NS, NCH, ALPHA, DEPTH, PX>(F, s_bulk, blockIdx.x, blockIdx.y);
}

template<int NS, int NCH, bool ALPHA, int DEPTH, int PX>
__global__ void __launch_bounds__(kBulkThreads, 2) k_vhfuse(FJob F, const FuseTile *tiles)
{
	extern __shared__ __align__(128) unsigned char s_fuse[];
	vhfuse_tile<NS, NCH, ALPHA, DEPTH, PX>(F, tiles, s_fuse, blockIdx.x, blockIdx.y);
}

template<int NS, int NCH, bool ALPHA, int DEPTH, int PX>
__global__ void __launch_bounds__(kVPxThreads) k_vstream_px(FJob F)
{
	extern __shared__ __align__(16) float s_dyn[];
	vstream_px_tile<NS, NCH, ALPHA, DEPTH, PX>(F, s_dyn, blockIdx.x, blockIdx.y);
}

template<int NPL, int DEPTH>
__global__ void __launch_bounds__(kVThreads) k_vgather(FJob F)
{
	extern __shared__ __align__(16) float s_tab[];
	vgather_tile<NPL, DEPTH>(F, s_tab, blockIdx.x, blockIdx.y);
}

template<int NPL>
__global__ void __launch_bounds__(kHThreads) k_hpass_fast(FJob F)
{
	hpass_pixel<NPL>(F, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y);
}

// wide windows: a warp per output pixel, kHThreads / 32 pixels per block
template<int NPL>
__global__ void __launch_bounds__(kHThreads) k_hpass_warp(FJob F)
{
	hpass_pixel_warp<NPL>(F, blockIdx.x * (kHThreads / 32) + (threadIdx.x >> 5), blockIdx.y, threadIdx.x & 31);
}

constexpr int kHWarpTaps = 64;   // horizontal windows from this many taps: a warp per pixel

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

// Device copies of host tables.  The host tables are cached process-wide
// (tables.cpp), so keying by their address is stable; derived float versions
// are cached under (address, kind) together with a reference that keeps the
// source alive.
struct Cache {
	std::mutex mu;        // the per-image scratch and the band tuner
	std::mutex tab_mu;    // the device table cache 'dev' (and the decode-error record)
	struct Entry { std::shared_ptr<const void> keep; std::shared_ptr<const void> derived; void *dev; };
	std::map<std::pair<const void *, int>, Entry> dev;
	// each stream's per-image device block (grown stream-ordered on its own
	// stream, so a block is never reallocated under another stream's work)
	struct Scratch { void *p = nullptr; size_t cap = 0; };
	std::map<cudaStream_t, Scratch> scratch;
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
	std::lock_guard<std::mutex> lk(C.tab_mu);
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
	std::lock_guard<std::mutex> lk(C.tab_mu);
	auto key = std::make_pair((const void *)v.get(), kind);
	auto it = C.dev.find(key);
	if(it != C.dev.end()) return (const float *)it->second.dev;
	std::shared_ptr<std::vector<float>> f = make(*v);
	const float *d = upload_vec(*f);
	if(d) C.dev[key] = {std::static_pointer_cast<const void>(v), std::static_pointer_cast<const void>(f), (void *)d};
	return d;
}

// Double-float copy of a double table: (hi, lo) = (fl32(d), fl32(d - hi)),
// within 2^-48 |d| of d.
std::shared_ptr<std::vector<float>> as_dfloat(const std::vector<double> &v)
{
	auto f = std::make_shared<std::vector<float>>(2 * v.size());
	for(size_t i = 0; i < v.size(); i++) {
		const float hi = (float)v[i];
		(*f)[2 * i] = hi;
		(*f)[2 * i + 1] = std::isfinite(v[i]) ? (float)(v[i] - (double)hi) : 0.0f;
	}
	return f;
}

// Search start points for a float copy of an ascending table t[first ..
// first+n): cell i holds the number of entries <= i / kLutCells.
std::shared_ptr<std::vector<float>> make_lut(const std::vector<double> &t, int first, int n)
{
	auto f = std::make_shared<std::vector<float>>(kLutCells);
	int k = 0;
	for(int i = 0; i < kLutCells; i++) {
		const float c = (float)i / (float)kLutCells;
		while(k < n && (float)t[first + k] <= c) k++;
		(*f)[i] = (float)k;
	}
	return f;
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
		// Above 4096 output levels the FP32 bound (about taps * 2^-24 of the
		// value) spans a large share of a step: at 16-bit output most pixels
		// get flagged (measured: about 90 %), and re-evaluating each with its
		// own vertical sums costs more than the plain form, which shares them.
		if(P.out[oc].q.P > 4095) return false;
	}
	if(P.wsets[0][0]->edge_value != 0.0 || P.wsets[1][0]->edge_value != 0.0) return false;
	(void)J;
	fi.streaming = 0;
	fi.slots = 0;
	return true;
}



void fast_launch_impl(cudaStream_t st, void *state, void (*mark)(void *), void *markarg)
{
	FastState &S = *static_cast<FastState *>(state);
	cudaMemsetAsync(S.F.flag_count, 0, 4 * sizeof(int), st);
	void *fargs[] = {&S.F};
	void *targs[] = {&S.T};
	void *uargs[] = {&S.F, &S.fuse_tiles};
	if(S.fuse) {
		// one fused launch: its time is reported as the vertical group's, the
		// horizontal group's is empty
		cudaLaunchKernel(S.vkernel, S.vgrid, dim3(S.vthreads), uargs, S.vsmem, st);
		mark(markarg);
		mark(markarg);
	}
	else {
		cudaLaunchKernel(S.vkernel, S.vgrid, dim3(S.vthreads), S.tc ? targs : fargs, S.vsmem, st);
		mark(markarg);
		cudaLaunchKernel(S.hkernel, S.hgrid, dim3(kHThreads), fargs, 0, st);
		mark(markarg);
	}
	// exact re-evaluation of flagged pixels (recomputes the vertical pass too)
	launch_fix_flagged(st, S.J, S.F.flag_count, S.F.flag_list, (int)std::min<size_t>(S.flag_entries, 0x7fffffff));
	mark(markarg);
}

void fast_release(FastInfo &fi)
{
	delete static_cast<FastState *>(fi.state);
	fi.state = nullptr;
}

// Host preparation of one image: job layout, error model, per-image arrays
// (in FastState::blob, placed later) and kernel choice.  'batch' picks
// taller vertical tiles (many images fill the GPU).  Caller holds the cache lock.
static FastState *fast_build(const Plan &P, const Job &J, bool batch, int tc_mode, std::string &err,
	bool allow_fuse = false)
{
	FJob F;
	memset(&F, 0, sizeof(F));
	F.wait_polls = kWaitPolls;
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
		{
			std::lock_guard<std::mutex> lk(cache().tab_mu);
			e_dec = dec_err[std::make_pair((const void *)coltab.get(), P.in_depth)];
		}
		dec_floats = P.in_depth == 8 ? 256 : 8192;
		if(!dec_tab) { err = "Out of GPU memory (fast tables)"; return nullptr; }
	}
	e_dec = std::max(e_dec, 2.0 * u);   // code*inv: 1/maxcc rounded, product rounded
	F.dec_tab = dec_tab;
	F.dec_tab_floats = dec_floats;

	// ---- error model constants per plane
	const int nv = std::max(1, WV.max_taps), nh = std::max(1, WH.max_taps);
	const double W1v = WV.kind == RowKind::Copy ? 1.0 : WV.wsum_abs_max, W1h = WH.kind == RowKind::Copy ? 1.0 : WH.wsum_abs_max;
	const double Wnv = WV.kind == RowKind::Copy ? 0.0 : WV.wsum_neg_max;
	// roundings a horizontal product passes through: blocked sums per thread,
	// or a lane's strided sum plus a five-step butterfly (a warp per pixel)
	const bool hwarp = !batch && nh >= kHWarpTaps;
	const int h_rounds = hwarp ? (nh + 31) / 32 + 5 : std::min(nh, kHBlock) + (nh + kHBlock - 1) / kHBlock;
	for(int q = 0; q < nplanes; q++) {
		double r_dec = keys[q].premul ? 3.0 * u : 0.0;
		double c1 = (r_dec + 2.0 * u + gamma_n(nv + 1, u) + gamma_n(nv + 1, ud)) * 1.01;
		double c2 = (u + gamma_n(h_rounds + 1, u) + gamma_n(nh + 1, ud)) * 1.01;
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
	std::vector<float> wvdf = *as_dfloat(WV.w), whdf = *as_dfloat(WH.w);
	size_t o_wvdf = add(wvdf.data(), wvdf.size() * 4), o_whdf = add(whdf.data(), whdf.size() * 4);
	size_t o_fp = 0, o_lp = 0, o_src = 0, o_pi = 0, o_sw = 0;
	if(S.ok) {
		o_fp = add(S.first_pos.data(), S.first_pos.size() * 4);
		o_lp = add(S.last_pos.data(), S.last_pos.size() * 4);
		o_src = add(S.srcrow.data(), S.srcrow.size() * 4);
		o_pi = add(S.pinfo.data(), S.pinfo.size() * 4);
		o_sw = add(S.sw.data(), S.sw.size() * 4);
	}
	if(S.ok) {
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
		// start points for the table searches (counted with the same float compares)
		T.lut = q.use_nc ? dev_derived(q.nc, 401, [](const std::vector<double> &t) { return make_lut(t, 0, (int)t.size()); })
		                 : dev_derived(q.U, 400, [](const std::vector<double> &t) { return make_lut(t, 1, (int)t.size() - 2); });
		if(!T.U || !T.X || !T.code || !T.rev || (q.use_nc && !T.nc) || !T.lut) { err = "Out of GPU memory (fast tables)"; return nullptr; }
	}
	for(int k = 0; k < P.mid_n; k++) F.k_tail[k] = tails[F.k_out[k] >= 0 ? F.k_out[k] : 0];

	// ---- double-float tables for the re-evaluation tier (cached)
	const float2 *df_tab[dev::kMaxCh] = {nullptr, nullptr, nullptr, nullptr};
	const float2 *df_atab = nullptr;
	bool df_ok = true;
	{
		auto df_of_table = [&](const std::shared_ptr<const std::vector<double>> &t) {
			return (const float2 *)dev_derived(t, 300, as_dfloat);
		};
		const int ncodes = 1 << P.in_depth;
		for(int m = 0; m < P.mid_n; m++) {
			const MidChannel &mc = P.mid[m];
			if(mc.in_ch >= P.in_nphys) continue;   // virtual channel: value 1
			df_tab[m] = df_of_table(input_table(P.cs_in.cstype, P.cs_in.gamma, P.in_max, ncodes, mc.lin_cs));
			if(!df_tab[m]) df_ok = false;
		}
		if(IW_IMGTYPE_HAS_ALPHA(P.in_logtype) && P.in_alpha < P.in_nphys) {
			df_atab = df_of_table(input_table(P.cs_in.cstype, P.cs_in.gamma, P.in_max, ncodes, true));
			if(!df_atab) df_ok = false;
		}
	}

	// ---- kernel selection
	auto *FS = new FastState();
	for(int m = 0; m < dev::kMaxCh; m++) FS->df_tab[m] = df_tab[m];
	FS->df_atab = df_atab;
	FS->df = df_ok;
	const int gx = (F.mid_w + kVThreads - 1) / kVThreads;
	FS->vsmem = (size_t)dec_floats * sizeof(float);
	FS->vgrid = dim3(gx, F.mid_h);
#define IWG_VSTREAM(NS_, NPL_, D_) \
	if(!FS->vkernel && S.ns == NS_ && nplanes == NPL_ && P.in_depth == D_) { \
		int bands = std::max(1, std::min(F.mid_h, batch ? (F.mid_h + 47) / 48 : (4 * 152 + gx - 1) / gx)); \
		F.rows_per_band = (F.mid_h + bands - 1) / bands; \
		bands = (F.mid_h + F.rows_per_band - 1) / F.rows_per_band; \
		FS->vkernel = (const void *)k_vstream<NS_, NPL_, D_>; \
		FS->vgrid = dim3(gx, bands); \
		FS->vv.kind = 2; FS->vv.ns = NS_; FS->vv.nch = NPL_; FS->vv.depth = D_; \
	}
#define IWG_VGATHER(NPL_, D_) \
	if(!FS->vkernel && nplanes == NPL_ && P.in_depth == D_) { \
		FS->vkernel = (const void *)k_vgather<NPL_, D_>; \
		FS->vv.kind = 3; FS->vv.nch = NPL_; FS->vv.depth = D_; \
	}
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
			int bands = std::max(1, std::min(F.mid_h, batch ? (F.mid_h + 47) / 48 : (5 * 152 + gxp_ / 2) / gxp_)); \
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
				FS->vv.kind = 1; FS->vv.ns = NS_; FS->vv.nch = NCH_; FS->vv.alpha = A_; FS->vv.depth = D_; FS->vv.px = PX_; \
			} \
		} \
	}
	// rows staged by asynchronous bulk copies: input in device memory, rows
	// 16-byte aligned
	bool in_device = false;
	{
		cudaPointerAttributes pa{};
		if(cudaPointerGetAttributes(&pa, J.in) == cudaSuccess) in_device = pa.type == cudaMemoryTypeDevice;
		cudaGetLastError();
	}
#define IWG_VBULK(NS_, NCH_, A_, D_, PX_) \
	if(!FS->vkernel && in_device && ident && S.arith && S.ns == NS_ && nplanes == NCH_ && (F.alpha_src >= 0) == A_ && \
		P.in_depth == D_ && v_base % 16 == 0 && P.in_bpr % 16 == 0) { \
		const int gxb_ = (F.mid_w + kBulkConsumers * PX_ - 1) / (kBulkConsumers * PX_); \
		int bands = std::max(1, std::min(F.mid_h, batch ? (F.mid_h + 47) / 48 : (2 * 152 + gxb_ / 2) / gxb_)); \
		F.rows_per_band = (F.mid_h + bands - 1) / bands; \
		bands = (F.mid_h + F.rows_per_band - 1) / F.rows_per_band; \
		int nq_max = 0; \
		for(int b_ = 0; b_ < bands; b_++) { \
			const int jb_ = b_ * F.rows_per_band, je_ = std::min(jb_ + F.rows_per_band, F.mid_h); \
			nq_max = std::max(nq_max, S.last_pos[je_ - 1] - S.first_pos[jb_] + 1); \
		} \
		const size_t sm_ = (size_t)kBulkStages * kBulkConsumers * PX_ * NCH_ * (D_ / 8) + 256 + \
			(size_t)dec_floats * sizeof(float) + (size_t)nq_max * (NS_ * sizeof(float) + sizeof(int2)); \
		const void *k_ = (const void *)k_vbulk<NS_, NCH_, A_, D_, PX_>; \
		if(sm_ <= 200 * 1024 && \
			cudaFuncSetAttribute(k_, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_) == cudaSuccess) { \
			FS->vkernel = k_; \
			FS->vgrid = dim3(gxb_, bands); \
			FS->vthreads = kBulkThreads; \
			FS->vsmem = sm_; \
			FS->vv.kind = 4; FS->vv.ns = NS_; FS->vv.nch = NCH_; FS->vv.alpha = A_; FS->vv.depth = D_; FS->vv.px = PX_; \
		} \
		cudaGetLastError(); \
	}
	IWG_VBULK_VARIANTS(IWG_VBULK)
#undef IWG_VBULK
	IWG_VPX_VARIANTS(IWG_VPX)
#undef IWG_VPX
	if(S.ok) {
		IWG_VSTREAM_VARIANTS(IWG_VSTREAM)
	}
	IWG_VGATHER_VARIANTS(IWG_VGATHER)
#undef IWG_VSTREAM
#undef IWG_VGATHER
	// Vertical pass on the tensor cores (tcvert.cu): 8-bit channels decoded
	// through the input table, no alpha, rows in device memory.  Its bound is
	// far tighter than an FP32 sum over a wide window (fixed-point quantisation
	// only), which is what pays for wide windows: fewer flagged pixels.
	// tc_mode: 0 never, 1 windows of kTcAutoTaps rows or more, 2 whenever eligible.
	constexpr int kTcAutoTaps = 48;
	if(!batch && tc_mode != 0 && (tc_mode == 2 || nv >= kTcAutoTaps) && in_device && ident && F.alpha_src < 0 &&
		P.in_depth == 8 && v_bpp == P.in_nphys && coltab && P.crop_h > 0) {
		bool all_tab = true;
		for(int q = 0; q < nplanes; q++)
			if(!F.pl[q].table || F.pl[q].premul) all_tab = false;
		std::vector<const std::vector<double> *> tabs(nplanes, coltab.get());
		tc::TcBuild TB;
		if(all_tab && tc::tc_build(WV, P.crop_h, nplanes, tabs, TB)) {
			int dev = 0, sms = 152;
			if(cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
				sms = 152;
			cudaGetLastError();
			const size_t tsm = tc::tc_smem_bytes(nplanes);
			const bool tvec = v_base % 2 == 0 && P.in_bpr % 2 == 0;
			const void *tk = tc::tc_kernel(tvec);
			int strips = 0, bands = 0, bpb = 0;
			tc::tc_geometry(TB, J.mid_w * nplanes, sms, strips, bands, bpb);
			if(cudaFuncSetAttribute(tk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsm) == cudaSuccess) {
				FS->tc = true;
				FS->vkernel = tk;
				FS->vgrid = dim3(strips, bands);
				FS->vthreads = tc::kThreads;
				FS->vsmem = tsm;
				FS->vv.kind = 5;
				tc::TcJob &T = FS->T;
				memset(&T, 0, sizeof(T));
				T.in_rows = P.crop_h;
				T.cols = J.mid_w * nplanes;
				T.nphys = nplanes;
				T.mid_w = J.mid_w;
				T.mid_h = J.mid_h;
				T.plane = J.interm_plane;
				T.nblk = TB.nblk;
				T.blocks_per_band = bpb;
				T.scale = TB.scale;
				FS->o_tct = add(TB.tiles.data(), TB.tiles.size());
				FS->o_tcb = add(TB.blk.data(), TB.blk.size() * sizeof(int4));
				FS->o_tcl = add(TB.lut.data(), TB.lut.size() * sizeof(uint2));
				// error model of the exact-integer pass: |I' - I_ref| <= e_abs*1.01 + (2u + gamma_nv^(fp64))*(|I'| + 2*Wneg_v)
				const double ed_tc = TB.e_abs * 1.01 / std::max(W1v, 1e-300);
				for(int q = 0; q < nplanes; q++) {
					double c1 = (2.0 * u + gamma_n(nv + 1, ud)) * 1.01;
					double c2 = (u + gamma_n(h_rounds + 1, u) + gamma_n(nh + 1, ud)) * 1.01;
					F.K0[q] = (float)((ed_tc * W1v * W1h + 2.02 * c1 * Wnv * W1h) * 1.05);
					F.K1[q] = (float)((1.01 * c1 + c2) * 1.05);
				}
			}
			cudaGetLastError();
		}
	}
	if(!FS->vkernel) { delete FS; err = "fast form: no kernel for this layout"; return nullptr; }
	FS->in_device = in_device;
	// Fused vertical + horizontal pass: where the bulk-copy vertical pass runs
	// (rows in device memory, 16-byte aligned) and the horizontal windows are
	// narrow (a thread per pixel).  Column tiles are chosen so that each
	// tile's input columns, widened to 16-byte boundaries, fit one strip.
	std::vector<FuseTile> ftiles;
	if(allow_fuse && !batch && FS->vv.kind == 4 && FS->vv.nch == 4 && FS->vv.px == 2 && FS->vv.ns == 4 && !hwarp &&
		WH.kind == RowKind::Sum && F.mid_h == F.out_h) {
		const int al = 16 / v_bpp;   // columns per 16 bytes
		const int maxc = kBulkConsumers * FS->vv.px;
		const long long row_cols = (long long)P.in_bpr / v_bpp - P.crop_x;   // columns a row's bytes hold from the crop
		bool ok = 16 % v_bpp == 0;
		auto plan_tiles = [&](int ntiles) {
			std::vector<FuseTile> t;
			const int tw = (F.out_w + ntiles - 1) / ntiles;
			for(int i0 = 0; i0 < F.out_w; i0 += tw) {
				const int i1 = std::min(F.out_w, i0 + tw);
				int lo = INT32_MAX, hi = -1;
				for(int t2 = WH.off[i0]; t2 < WH.off[i1]; t2++)
					if(WH.src[t2] >= 0) { lo = std::min(lo, WH.src[t2]); hi = std::max(hi, WH.src[t2]); }
				if(hi < 0) return std::vector<FuseTile>();
				const int xa = lo / al * al, xb = (hi + 1 + al - 1) / al * al;
				if(xb - xa > maxc || xb > row_cols) return std::vector<FuseTile>();
				t.push_back(FuseTile{xa, xb - xa, i0, i1});
			}
			return t;
		};
		for(int ntiles = std::max(1, F.out_w * 4 / maxc); ok && ntiles <= F.out_w && ftiles.empty(); ntiles++)
			ftiles = plan_tiles(ntiles);
	}
	if(getenv("IWG_TRACE"))
		fprintf(stderr, "iwg fast_build: vertical kind %d ns %d nch %d alpha %d depth %d px %d in_device %d arith %d "
			"stream %d hwarp %d allow_fuse %d tiles %d mid %dx%d out %dx%d\n", FS->vv.kind, FS->vv.ns, FS->vv.nch,
			FS->vv.alpha, FS->vv.depth, FS->vv.px, (int)in_device, (int)S.arith, (int)S.ok, (int)hwarp, (int)allow_fuse,
			(int)ftiles.size(), F.mid_w, F.mid_h, F.out_w, F.out_h);
	if(!ftiles.empty()) {
		const void *k_ = nullptr;
		if(FS->vv.alpha && FS->vv.depth == 16) k_ = (const void *)k_vhfuse<4, 4, true, 16, 2>;
		const size_t fixed = (size_t)kBulkStages * kBulkConsumers * FS->vv.px * FS->vv.nch * (FS->vv.depth / 8) +
			(size_t)kFuseRows * kBulkConsumers * FS->vv.px * sizeof(float4) + 256 + (size_t)dec_floats * sizeof(float);
		const size_t per_pos = (size_t)FS->vv.ns * sizeof(float) + sizeof(int2);
		const int ntiles = (int)ftiles.size();
		int bands = std::max(1, std::min(F.mid_h, (2 * 152) / ntiles));
		int rows = (F.mid_h + bands - 1) / bands;
		bands = (F.mid_h + rows - 1) / rows;
		int nq_max = 0;
		for(int b = 0; b < bands; b++) {
			const int jb = b * rows, je = std::min(jb + rows, F.mid_h);
			nq_max = std::max(nq_max, S.last_pos[je - 1] - S.first_pos[jb] + 1);
		}
		const size_t sm = fixed + (size_t)nq_max * per_pos;
		if(k_ && sm <= 200 * 1024 &&
			cudaFuncSetAttribute(k_, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) == cudaSuccess) {
			FS->fuse = true;
			FS->vkernel = k_;
			FS->vgrid = dim3(ntiles, bands);
			FS->vthreads = kBulkThreads;
			FS->vsmem = sm;
			F.rows_per_band = rows;
			FS->vv.kind = 6;
			FS->o_fuse = add(ftiles.data(), ftiles.size() * sizeof(FuseTile));
		}
		cudaGetLastError();
	}
	if(S.ok) {
		FS->first_pos = S.first_pos;
		FS->last_pos = S.last_pos;
	}
	if(FS->vv.kind == 1) {
		FS->vsmem_per_pos = (size_t)FS->vv.ns * sizeof(float) + sizeof(int2);
		FS->vsmem_fixed = (size_t)dec_floats * sizeof(float);
	}
	else if(FS->vv.kind == 4) {
		FS->vsmem_per_pos = (size_t)FS->vv.ns * sizeof(float) + sizeof(int2);
		FS->vsmem_fixed = (size_t)kBulkStages * kBulkConsumers * FS->vv.px * FS->vv.nch * (FS->vv.depth / 8) + 256 +
			(size_t)dec_floats * sizeof(float);
	}
	else if(FS->vv.kind == 6) {
		FS->vsmem_per_pos = (size_t)FS->vv.ns * sizeof(float) + sizeof(int2);
		FS->vsmem_fixed = (size_t)kBulkStages * kBulkConsumers * FS->vv.px * FS->vv.nch * (FS->vv.depth / 8) +
			(size_t)kFuseRows * kBulkConsumers * FS->vv.px * sizeof(float4) + 256 + (size_t)dec_floats * sizeof(float);
	}
	else FS->vsmem_fixed = FS->vsmem;
	if(hwarp) {
		switch(nplanes) {
		case 1: FS->hkernel = (const void *)k_hpass_warp<1>; break;
		case 2: FS->hkernel = (const void *)k_hpass_warp<2>; break;
		case 3: FS->hkernel = (const void *)k_hpass_warp<3>; break;
		default: FS->hkernel = (const void *)k_hpass_warp<4>; break;
		}
		FS->hgrid = dim3((F.out_w + kHThreads / 32 - 1) / (kHThreads / 32), F.out_h);
	}
	else {
		switch(nplanes) {
		case 1: FS->hkernel = (const void *)k_hpass_fast<1>; break;
		case 2: FS->hkernel = (const void *)k_hpass_fast<2>; break;
		case 3: FS->hkernel = (const void *)k_hpass_fast<3>; break;
		default: FS->hkernel = (const void *)k_hpass_fast<4>; break;
		}
		FS->hgrid = dim3((F.out_w + kHThreads - 1) / kHThreads, F.out_h);
	}
	F.vgx = (int)FS->vgrid.x;
	F.vgy = (int)FS->vgrid.y;
	F.hgx = (int)FS->hgrid.x;
	FS->F = F;
	FS->J = J;
	// start points of the re-evaluation's bracket searches: the tail's tables
	static_assert(kLutCells == dev::kBracketLutCells, "one cell count for both searches");
	for(int oc = 0; oc < P.out_n; oc++) FS->J.outc[oc].q.lut = tails[oc].use_nc ? nullptr : tails[oc].lut;
	FS->blob = std::move(blob);
	FS->o_hoff = o_hoff; FS->o_hsrc = o_hsrc; FS->o_hw = o_hw;
	FS->o_voff = o_voff; FS->o_vsrc = o_vsrc; FS->o_vw = o_vw;
	FS->o_fp = o_fp; FS->o_lp = o_lp; FS->o_src = o_src; FS->o_pi = o_pi; FS->o_sw = o_sw;
	FS->o_wvdf = o_wvdf; FS->o_whdf = o_whdf;
	FS->streaming = S.ok;
	FS->flag_entries = (size_t)F.out_w * F.out_h;
	return FS;
}

// Points the image's per-image arrays at 'base' (a device copy of its blob)
// and its flags at the given counter and list.
static void fast_place(FastState *FS, const uint8_t *base, int *flag_count, int *flag_list, int img, size_t flag_cap)
{
	FJob &F = FS->F;
	F.flag_count = flag_count;
	F.flag_list = flag_list;
	F.flag_cap = (int)std::min<size_t>(flag_cap, 0x7fffffff);
	F.err_flag = flag_count + 2;
	F.img = img;
	F.hoff = (const int *)(base + FS->o_hoff);
	F.hsrc = (const int *)(base + FS->o_hsrc);
	F.hw = (const float *)(base + FS->o_hw);
	F.voff = (const int *)(base + FS->o_voff);
	F.vsrc = (const int *)(base + FS->o_vsrc);
	F.vw = (const float *)(base + FS->o_vw);
	if(FS->tc) {
		tc::TcJob &T = FS->T;
		T.in = F.in + (size_t)F.crop_x * F.nphys + (unsigned long long)F.crop_y * F.in_bpr;
		T.in_bpr = F.in_bpr;
		T.interm = F.interm;
		T.err_flag = F.err_flag;
		T.tiles = (const uint4 *)(base + FS->o_tct);
		T.blk = (const int4 *)(base + FS->o_tcb);
		T.lut = (const uint2 *)(base + FS->o_tcl);
	}
	FS->fuse_tiles = FS->fuse ? (const FuseTile *)(base + FS->o_fuse) : nullptr;
	Job &J = FS->J;
	for(int m = 0; m < dev::kMaxCh; m++) J.df_tab[m] = FS->df ? FS->df_tab[m] : nullptr;
	J.df_atab = FS->df ? FS->df_atab : nullptr;
	J.df_wv = FS->df ? (const float2 *)(base + FS->o_wvdf) : nullptr;
	J.df_wh = FS->df ? (const float2 *)(base + FS->o_whdf) : nullptr;
	if(FS->streaming) {
		F.first_pos = (const int *)(base + FS->o_fp);
		F.last_pos = (const int *)(base + FS->o_lp);
		F.srcrow = (const int *)(base + FS->o_src);
		F.pinfo = (const int2 *)(base + FS->o_pi);
		F.sw = (const float *)(base + FS->o_sw);
	}
}

// ---- the autotuner: band heights of the vertical pass ----
//
// The vertical kernels split the output rows into bands (one block per strip
// and band; for the tensor-core pass, bands of 16-row blocks).  Taller bands
// read fewer overlapping input rows, shorter ones give the GPU more blocks;
// the best count depends on the geometry, the kernel and the machine.  The
// first image of a geometry times a few candidate counts on its own data
// (CUDA events, best of two launches each after a warm launch) and keeps the
// fastest; later images of that geometry reuse it.  Every output row is summed
// by one block in the same order whatever the count, so the bytes never
// depend on the choice.

// Current band count of the prepared vertical pass (0: not banded).
static int vbands(const FastState &FS)
{
	if(FS.tc) return (FS.T.nblk + FS.T.blocks_per_band - 1) / FS.T.blocks_per_band;
	if(FS.vv.kind == 1 || FS.vv.kind == 2 || FS.vv.kind == 4 || FS.vv.kind == 6) return (int)FS.vgrid.y;
	return 0;
}

// Re-targets the prepared vertical pass to about 'bands' bands; false if that
// count is not possible (shared memory).
static bool set_vbands(FastState &FS, int bands)
{
	if(FS.tc) {
		const int nblk = FS.T.nblk;
		bands = std::max(1, std::min(bands, nblk));
		const int bpb = (nblk + bands - 1) / bands;
		FS.T.blocks_per_band = bpb;
		FS.vgrid.y = (nblk + bpb - 1) / bpb;
		FS.F.vgy = (int)FS.vgrid.y;
		return true;
	}
	FJob &F = FS.F;
	const int mid_h = F.mid_h;
	bands = std::max(1, std::min(bands, mid_h));
	const int rows = (mid_h + bands - 1) / bands;
	bands = (mid_h + rows - 1) / rows;
	size_t sm = FS.vsmem_fixed;
	if(FS.vsmem_per_pos) {
		if(FS.first_pos.size() < (size_t)mid_h || FS.last_pos.size() < (size_t)mid_h) return false;
		int nq_max = 0;
		for(int b = 0; b < bands; b++) {
			const int jb = b * rows, je = std::min(jb + rows, mid_h);
			nq_max = std::max(nq_max, FS.last_pos[je - 1] - FS.first_pos[jb] + 1);
		}
		sm = FS.vsmem_fixed + (size_t)nq_max * FS.vsmem_per_pos;
		if(sm > 200 * 1024) return false;
		if(sm > 48 * 1024 && cudaFuncSetAttribute(FS.vkernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess) {
			cudaGetLastError();
			return false;
		}
	}
	F.rows_per_band = rows;
	FS.vgrid.y = bands;
	F.vgy = bands;
	FS.vsmem = sm;
	return true;
}

static bool launch_vertical(cudaStream_t st, FastState &FS)
{
	void *fargs[] = {&FS.F};
	void *uargs[] = {&FS.F, &FS.fuse_tiles};
	void *targs[] = {&FS.T};
	// The fused pass also lists flagged pixels: its counters start at zero
	// for every trial launch (the scratch holding them is reused between
	// jobs, and trials must not pile entries past the list's capacity).
	if(FS.fuse) cudaMemsetAsync(FS.F.flag_count, 0, 4 * sizeof(int), st);
	return cudaLaunchKernel(FS.vkernel, FS.vgrid, dim3(FS.vthreads), FS.tc ? targs : (FS.fuse ? uargs : fargs), FS.vsmem,
		st) == cudaSuccess;
}

// Chooses the band count of FS's vertical pass (cached per geometry).  Runs
// on 'st' after the input upload; the vertical pass's output is rewritten by
// the real run.  Caller holds the cache lock.
static void tune_vertical(cudaStream_t st, FastState &FS)
{
	const int b0 = vbands(FS);
	if(b0 <= 0 || !FS.in_device) return;
	static std::map<std::vector<long long>, int> tuned;
	const std::vector<long long> key = {(long long)(uintptr_t)FS.vkernel, FS.F.mid_w, FS.F.mid_h, FS.F.in_rows,
		FS.J.wv[0].max_taps, FS.tc ? FS.T.nblk : 0};
	auto it = tuned.find(key);
	if(it != tuned.end()) {
		if(!set_vbands(FS, it->second)) set_vbands(FS, b0);
		return;
	}
	cudaEvent_t e0, e1;
	if(cudaEventCreate(&e0) != cudaSuccess) { cudaGetLastError(); return; }
	if(cudaEventCreate(&e1) != cudaSuccess) { cudaEventDestroy(e0); cudaGetLastError(); return; }
	int best = b0;
	float best_ms = 1e30f;
	std::vector<int> cands = {b0, std::max(1, b0 / 2), 2 * b0, 3 * b0, 4 * b0};
	std::vector<int> tried;
	for(int c : cands) {
		if(!set_vbands(FS, c)) continue;
		const int actual = vbands(FS);
		if(std::find(tried.begin(), tried.end(), actual) != tried.end()) continue;
		tried.push_back(actual);
		if(!launch_vertical(st, FS)) { cudaGetLastError(); continue; }   // warm
		float ms_min = 1e30f;
		for(int rep = 0; rep < 2; rep++) {
			cudaEventRecord(e0, st);
			launch_vertical(st, FS);
			cudaEventRecord(e1, st);
			float ms = 0.0f;
			if(cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess)
				ms_min = std::min(ms_min, ms);
		}
		cudaGetLastError();
		if(ms_min < best_ms) { best_ms = ms_min; best = actual; }
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	if(!set_vbands(FS, best)) set_vbands(FS, b0);
	tuned[key] = vbands(FS);
}

bool fast_prepare(cudaStream_t st, const Plan &P, Job &J, FastInfo &fi, std::string &err)
{
	Cache &C = cache();
	std::lock_guard<std::mutex> lk(C.mu);
	FastState *FS = fast_build(P, J, false, fi.tc_mode, err, fi.fuse_mode != 0 && !fi.dbg);
	if(!FS) return false;
	const size_t flag_off = (FS->blob.size() + 255) & ~(size_t)255;
	const size_t need = flag_off + 256 + FS->flag_entries * 16;
	Cache::Scratch &SC = C.scratch[st];
	if(need > SC.cap) {
		if(SC.p) cudaFreeAsync(SC.p, st);
		SC.p = nullptr;
		SC.cap = 0;
		if(cudaMallocAsync(&SC.p, need + need / 8, st) != cudaSuccess) {
			cudaGetLastError();
			delete FS;
			err = "Out of GPU memory (fast form)";
			return false;
		}
		SC.cap = need + need / 8;
	}
	uint8_t *base = (uint8_t *)SC.p;
	cudaMemcpyAsync(base, FS->blob.data(), FS->blob.size(), cudaMemcpyHostToDevice, st);
	fast_place(FS, base, (int *)(base + flag_off), (int *)(base + flag_off + 256), 0, FS->flag_entries);
	FS->F.dbg = fi.dbg;
	for(int k = 0; k < P.mid_n && k < 4; k++) fi.plane_of[J.order[k]] = FS->F.k_plane[k];
	if(fi.wait_polls > 0) FS->F.wait_polls = fi.wait_polls;
	FS->F.starve = fi.starve;
	if(fi.autotune && fi.wait_polls <= 0 && !fi.starve) tune_vertical(st, *FS);
	fi.state = FS;
	fi.launches = FS->fuse ? 2 : 3;
	fi.fused = FS->fuse ? 1 : 0;
	fi.launch_fn = fast_launch_impl;
	fi.streaming = FS->streaming;
	fi.slots = FS->F.ns;
	fi.tc = FS->tc ? 1 : 0;
	fi.flag_count_dev = FS->F.flag_count;
	return true;
}

// ---- batch support (see fastpath.cuh) ----

// Safe to call from several host threads at once: fast_build's shared state
// (the device table cache) is guarded by its own lock.
void *fast_batch_item(const Plan &P, const Job &J, std::string &err)
{
	return fast_build(P, J, true, 0, err);
}

size_t fast_item_blob_bytes(const void *item) { return static_cast<const FastState *>(item)->blob.size(); }
const void *fast_item_blob(const void *item) { return static_cast<const FastState *>(item)->blob.data(); }
size_t fast_item_flag_entries(const void *item) { return static_cast<const FastState *>(item)->flag_entries; }
int fast_item_htaps(const void *item) { return static_cast<const FastState *>(item)->J.wh[0].max_taps; }
int fast_item_vtaps(const void *item) { return static_cast<const FastState *>(item)->J.wv[0].max_taps; }

void fast_item_place(void *item, const uint8_t *dev_blob, int *flag_count, int *flag_list, int img, size_t flag_cap)
{
	fast_place(static_cast<FastState *>(item), dev_blob, flag_count, flag_list, img, flag_cap);
}

void fast_item_job_df(const void *item, Job &J)
{
	const Job &K = static_cast<const FastState *>(item)->J;
	for(int m = 0; m < dev::kMaxCh; m++) J.df_tab[m] = K.df_tab[m];
	J.df_atab = K.df_atab;
	J.df_wv = K.df_wv;
	J.df_wh = K.df_wh;
	for(int oc = 0; oc < dev::kMaxCh; oc++) J.outc[oc].q.lut = K.outc[oc].q.lut;
}

void fast_item_free(void *item) { delete static_cast<FastState *>(item); }

void preload_fast_kernels()
{
	cudaFuncAttributes a;
#define IWG_PRE_BU(NS_, NCH_, A_, D_, PX_) cudaFuncGetAttributes(&a, (const void *)k_vbulk<NS_, NCH_, A_, D_, PX_>);
#define IWG_PRE_PX(NS_, NCH_, A_, D_, PX_) cudaFuncGetAttributes(&a, (const void *)k_vstream_px<NS_, NCH_, A_, D_, PX_>);
#define IWG_PRE_ST(NS_, NPL_, D_) cudaFuncGetAttributes(&a, (const void *)k_vstream<NS_, NPL_, D_>);
#define IWG_PRE_GA(NPL_, D_) cudaFuncGetAttributes(&a, (const void *)k_vgather<NPL_, D_>);
	IWG_VBULK_VARIANTS(IWG_PRE_BU)
	IWG_VPX_VARIANTS(IWG_PRE_PX)
	IWG_VSTREAM_VARIANTS(IWG_PRE_ST)
	IWG_VGATHER_VARIANTS(IWG_PRE_GA)
#undef IWG_PRE_BU
#undef IWG_PRE_PX
#undef IWG_PRE_ST
#undef IWG_PRE_GA
	cudaFuncGetAttributes(&a, (const void *)k_vhfuse<4, 4, true, 16, 2>);
	cudaFuncGetAttributes(&a, tc::tc_kernel(true));
	cudaFuncGetAttributes(&a, tc::tc_kernel(false));
	cudaFuncGetAttributes(&a, (const void *)k_hpass_fast<1>);
	cudaFuncGetAttributes(&a, (const void *)k_hpass_fast<2>);
	cudaFuncGetAttributes(&a, (const void *)k_hpass_fast<3>);
	cudaFuncGetAttributes(&a, (const void *)k_hpass_fast<4>);
	cudaFuncGetAttributes(&a, (const void *)k_hpass_warp<1>);
	cudaFuncGetAttributes(&a, (const void *)k_hpass_warp<2>);
	cudaFuncGetAttributes(&a, (const void *)k_hpass_warp<3>);
	cudaFuncGetAttributes(&a, (const void *)k_hpass_warp<4>);
	cudaGetLastError();
}

}  // namespace iwg
