// noalloc.cu -- a resampling entry point that allocates no memory.
//
// iwg_resize_u8_noalloc() runs the plain (FP64) form of the pixel pipeline
// for one 8-bit image whose input and output buffers the caller owns.  Every
// buffer it needs besides those lives in fixed, file-scope storage:
//
//   * device scratch: g_scratch, a static __device__ array of kScratchBytes.
//     Its head holds the decode and quantisation tables and the two weight
//     lists (copied from the host staging area below); the rest holds the
//     float intermediate image of the vertical pass;
//   * host staging: g_stage, a static array of kStageBytes where the tables
//     and weight lists are built before one copy to the device.
//
// Who needs this: a caller that must not allocate while it runs -- a
// real-time or serving loop that reserves all its memory up front, a
// process whose device memory pool is owned by another allocator, or code
// that runs where an allocation would stall on the device-wide
// synchronisation that cudaMalloc/cudaFree imply.  iw_process_image()
// allocates its context, plan and device buffers per call, so it cannot
// serve those callers.
//
// The arithmetic is the reference's, sample for sample, as in pipeline.cu:
// decode through an exact table, premultiply by alpha, vertical weighted sum
// into a float intermediate (src/imagew-main.c:831-927), horizontal weighted
// sum, divide by the float-rounded alpha, quantise to the nearest code
// (src/imagew-main.c:929-1155) and blacken colour samples of fully
// transparent pixels (src/imagew-main.c:1139-1146).
#include "iwg_internal.h"
#include "device.cuh"
#include "imagew_gb300.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

namespace iwg {
namespace {

using namespace dev;

constexpr size_t kScratchBytes = (size_t)32 << 20;   // device scratch: 32 MiB
constexpr size_t kStageBytes = (size_t)4 << 20;      // tables + weight lists: 4 MiB
constexpr int kMaxDim = 16384;
constexpr int kMaxDevices = 64;

// Shared by every call on every stream.  Nothing in it needs to start at zero:
// each call writes every byte it reads.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

alignas(256) static unsigned char g_stage[kStageBytes];

std::mutex g_mu;
void *g_scratch_ptr[kMaxDevices];
int g_pageable[kMaxDevices];   // 0: not queried, 1: no pageable access, 2: pageable access

// ---- 8-bit tables, rebuilt only when the colour space changes ----
struct Tables8 {
	double tab_c[256], tab_a[256];            // code -> linear value
	double Uc[257], Xc[256], revc[256], nc[255];
	double Ua[257], Xa[256], reva[256];
	int codec[257], codea[257];
};
static_assert(sizeof(Tables8) % 16 == 0, "table block keeps 16-byte alignment");

int g_tab_cstype = -1;
double g_tab_gamma = 0.0;

void fill_tables(Tables8 &T, int cstype, double gamma)
{
	struct iw_csdescr cs{};
	cs.cstype = cstype;
	cs.gamma = gamma;
	for(int v = 0; v < 256; v++) {
		T.tab_c[v] = to_linear(((double)v) / 255.0, cs);
		T.tab_a[v] = ((double)v) / 255.0;
	}
	quant_fill(cstype, gamma, 255, 0, T.Uc, T.Xc, T.codec, T.revc);
	quant_fill(IW_CSTYPE_LINEAR, 0.0, 255, 0, T.Ua, T.Xa, T.codea, T.reva);
	if(cstype != IW_CSTYPE_LINEAR) nc_fill(cstype, gamma, T.nc);
	else memset(T.nc, 0, sizeof(T.nc));
}

struct NAJob {
	const uint8_t *in;
	long long in_bpr;
	int in_w, in_h, nch, alpha;   // alpha: index of the alpha sample, -1 if none
	uint8_t *out;
	long long out_bpr;
	int out_w, out_h;
	const double *tab_c, *tab_a;
	DQuant qc, qa;
	DWeights wh, wv;
	float *interm;                // [nch][out_h][in_w]
};

// Linear (premultiplied) value of sample c at input (x, y).
__device__ __forceinline__ double na_decode(const NAJob &J, int c, int x, int y)
{
	const uint8_t *p = J.in + (unsigned long long)y * (unsigned long long)J.in_bpr + (size_t)x * J.nch;
	if(c == J.alpha) return J.tab_a[p[c]];
	double s = J.tab_c[p[c]];
	if(J.alpha >= 0) s = dmul(s, J.tab_a[p[J.alpha]]);
	return s;
}

// Vertical pass: one thread per (input column x, output row j), all samples.
__global__ void k_na_vpass(NAJob J)
{
	const int x = blockIdx.x * blockDim.x + threadIdx.x;
	const int j = blockIdx.y;
	if(x >= J.in_w || j >= J.out_h) return;
	const DWeights &W = J.wv;
	for(int c = 0; c < J.nch; c++) {
		double s = 0.0;
		if(W.kind == 1) {
			int src = W.src[j];
			s = src < 0 ? 0.0 : na_decode(J, c, x, src);
		}
		else {
			for(int t = W.off[j]; t < W.off[j + 1]; t++) {
				int src = W.src[t];
				double v = src >= 0 ? na_decode(J, c, x, src) : W.edge_value;
				s = dadd(s, dmul(v, W.w[t]));
			}
		}
		J.interm[((unsigned long long)c * J.out_h + j) * J.in_w + x] = __double2float_rn(s);
	}
}

__device__ __forceinline__ double na_hsum(const NAJob &J, int c, int i, int j)
{
	const DWeights &W = J.wh;
	const float *row = J.interm + ((unsigned long long)c * J.out_h + j) * J.in_w;
	double s = 0.0;
	if(W.kind == 1) {
		int src = W.src[i];
		s = src < 0 ? 0.0 : (double)row[src];
	}
	else {
		for(int t = W.off[i]; t < W.off[i + 1]; t++) {
			int src = W.src[t];
			double v = src >= 0 ? (double)row[src] : W.edge_value;
			s = dadd(s, dmul(v, W.w[t]));
		}
	}
	return s;
}

// Horizontal pass fused with the output tail: one thread per output pixel.
__global__ void k_na_hpass(NAJob J)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	const int j = blockIdx.y;
	if(i >= J.out_w || j >= J.out_h) return;
	uint8_t *px = J.out + (unsigned long long)j * (unsigned long long)J.out_bpr + (size_t)i * J.nch;
	double a = 0.0;
	int acode = -1;
	if(J.alpha >= 0) {
		double s = na_hsum(J, J.alpha, i, j);
		a = (double)__double2float_rn(s);
		acode = quantize_exact(J.qa, s, i, j);
		px[J.alpha] = (uint8_t)acode;
	}
	for(int c = 0; c < J.nch; c++) {
		if(c == J.alpha) continue;
		double v = na_hsum(J, c, i, j);
		if(J.alpha >= 0 && a != 0.0) v = ddiv(v, a);
		int code = quantize_exact(J.qc, v, i, j);
		if(acode == 0) code = 0;
		px[c] = (uint8_t)code;
	}
}

void set_msg(char *msg, int len, const char *text)
{
	if(!msg || len <= 0) return;
	snprintf(msg, (size_t)len, "%s", text);
}

// Bump allocator over the staging area; offsets are 256-byte aligned so the
// same offsets are valid in the device scratch.
struct Bump {
	size_t used = 0;
	size_t take(size_t bytes, size_t limit)
	{
		size_t at = (used + 255) & ~(size_t)255;
		if(at > limit || bytes > limit - at) return (size_t)-1;
		used = at + bytes;
		return at;
	}
};

// Device-side view of a quantisation table set placed at 'base'.
DQuant make_dquant(const unsigned char *base, const Tables8 *T, bool colour, bool use_nc)
{
	DQuant q{};
	auto dev_of = [&](const void *host) { return (const void *)(base + ((const unsigned char *)host - g_stage)); };
	q.float_out = 0;
	q.use_nc = use_nc ? 1 : 0;
	q.dfam = IW_DITHERFAMILY_NONE;
	q.dsub = 0;
	q.maxcc = 255;
	q.P = 255;
	q.U = (const double *)dev_of(colour ? T->Uc : T->Ua);
	q.X = (const double *)dev_of(colour ? T->Xc : T->Xa);
	q.code = (const int *)dev_of(colour ? T->codec : T->codea);
	q.rev = (const double *)dev_of(colour ? T->revc : T->reva);
	q.nc = colour ? (const double *)dev_of(T->nc) : nullptr;
	return q;
}

// True if the current device can dereference 'p' from a kernel.
bool device_can_access(const void *p, int dev, bool pageable)
{
	cudaPointerAttributes at{};
	if(cudaPointerGetAttributes(&at, p) != cudaSuccess) {
		cudaGetLastError();
		return false;
	}
	switch(at.type) {
	case cudaMemoryTypeDevice: return at.device == dev;
	case cudaMemoryTypeManaged: return true;
	case cudaMemoryTypeHost: return at.devicePointer == p;
	default: return pageable;   // ordinary host memory
	}
}

}  // namespace

void preload_noalloc_kernels()
{
	cudaFuncAttributes a;
	cudaFuncGetAttributes(&a, (const void *)k_na_vpass);
	cudaFuncGetAttributes(&a, (const void *)k_na_hpass);
	cudaGetLastError();
}

}  // namespace iwg

using namespace iwg;

extern "C" int iwg_resize_u8_noalloc(const unsigned char *src, int src_w, int src_h, long long src_bpr,
	unsigned char *dst, int dst_w, int dst_h, long long dst_bpr, int imgtype, int resize_type,
	double param1, double param2, int cstype, double gamma, void *stream, char *errmsg, int errmsg_len)
{
	char buf[200];
	int nch;
	switch(imgtype) {
	case IW_IMGTYPE_GRAY: nch = 1; break;
	case IW_IMGTYPE_GRAYA: nch = 2; break;
	case IW_IMGTYPE_RGB: nch = 3; break;
	case IW_IMGTYPE_RGBA: nch = 4; break;
	default:
		set_msg(errmsg, errmsg_len, "noalloc: image type must be gray, gray+alpha, RGB or RGBA");
		return 0;
	}
	if(!src || !dst) {
		set_msg(errmsg, errmsg_len, "noalloc: null image buffer");
		return 0;
	}
	if(src_w < 1 || src_h < 1 || dst_w < 1 || dst_h < 1 || src_w > kMaxDim || src_h > kMaxDim ||
		dst_w > kMaxDim || dst_h > kMaxDim) {
		snprintf(buf, sizeof(buf), "noalloc: image dimensions must be 1..%d", kMaxDim);
		set_msg(errmsg, errmsg_len, buf);
		return 0;
	}
	if(src_bpr < (long long)src_w * nch || dst_bpr < (long long)dst_w * nch) {
		set_msg(errmsg, errmsg_len, "noalloc: bytes per row smaller than a row of samples");
		return 0;
	}
	if(cstype == IW_CSTYPE_GAMMA) {
		if(!(gamma >= 0.1 && gamma <= 10.0)) {
			set_msg(errmsg, errmsg_len, "noalloc: gamma must be 0.1..10");
			return 0;
		}
		if(gamma >= 0.999995 && gamma <= 1.000005) cstype = IW_CSTYPE_LINEAR;   // as the API's colour spaces
	}
	else if(cstype == IW_CSTYPE_SRGB || cstype == IW_CSTYPE_LINEAR || cstype == IW_CSTYPE_REC709) gamma = 0.0;
	else {
		set_msg(errmsg, errmsg_len, "noalloc: unknown colour space type");
		return 0;
	}

	// Per-dimension filter requests; AUTO resolves like iw_process_image.
	DimRequest d[2];
	for(int k = 0; k < 2; k++) {
		int n_in = k == 0 ? src_w : src_h, n_out = k == 0 ? dst_w : dst_h;
		d[k].edge = IW_EDGE_POLICY_STANDARD;
		d[k].blur = 1.0;
		d[k].true_size = (double)n_out;
		if(resize_type == IW_RESIZETYPE_AUTO) {
			if(n_in == n_out) d[k].family = IW_RESIZETYPE_NULL;
			else { d[k].family = IW_RESIZETYPE_CUBIC; d[k].p1 = 0.0; d[k].p2 = 0.5; }
		}
		else { d[k].family = resize_type; d[k].p1 = param1; d[k].p2 = param2; }
		if(weights_max_taps(d[k], n_in, n_out) < 0) {
			set_msg(errmsg, errmsg_len, "noalloc: unknown resize algorithm");
			return 0;
		}
	}

	std::lock_guard<std::mutex> lk(g_mu);

	int dev = -1;
	if(cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
		cudaGetLastError();
		set_msg(errmsg, errmsg_len, "noalloc: no usable CUDA device");
		return 0;
	}
	// Once per device: resolve the scratch array's device address (this may
	// load the module on that device).
	if(!g_scratch_ptr[dev]) {
		void *p = nullptr;
		cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
		if(e != cudaSuccess || !p) {
			snprintf(buf, sizeof(buf), "noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
			cudaGetLastError();
			set_msg(errmsg, errmsg_len, buf);
			return 0;
		}
		int v = 0;
		if(cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) {
			cudaGetLastError();
			v = 0;
		}
		g_pageable[dev] = v ? 2 : 1;
		g_scratch_ptr[dev] = p;
	}
	unsigned char *scratch = (unsigned char *)g_scratch_ptr[dev];
	const bool pageable = g_pageable[dev] == 2;
	if(!device_can_access(src, dev, pageable) || !device_can_access(dst, dev, pageable)) {
		set_msg(errmsg, errmsg_len, "noalloc: an image buffer is not accessible from the current device");
		return 0;
	}

	// ---- stage tables and weight lists ----
	Bump bump;
	size_t t_off = bump.take(sizeof(Tables8), kStageBytes);
	Tables8 *T = (Tables8 *)(g_stage + t_off);
	if(g_tab_cstype != cstype || memcmp(&g_tab_gamma, &gamma, sizeof(double)) != 0) {
		fill_tables(*T, cstype, gamma);
		g_tab_cstype = cstype;
		g_tab_gamma = gamma;
	}
	DWeights dw[2];
	for(int k = 0; k < 2; k++) {
		int n_in = k == 0 ? src_w : src_h, n_out = k == 0 ? dst_w : dst_h;
		size_t off_at = bump.take(sizeof(int) * (size_t)(n_out + 1), kStageBytes);
		size_t room = off_at == (size_t)-1 ? 0 : kStageBytes - bump.used;
		// taps that fit in what is left: 4 bytes of source index + 8 of weight each, plus alignment
		long long cap = room > 1024 ? (long long)((room - 1024) / 12) : 0;
		if(cap > 0x7fffffff) cap = 0x7fffffff;
		int *off = (int *)(g_stage + off_at);
		size_t src_at = bump.take(0, kStageBytes);   // placeholder: sizes known after the fill
		size_t w_at = ((src_at + sizeof(int) * (size_t)cap) + 255) & ~(size_t)255;
		if(off_at == (size_t)-1 || src_at == (size_t)-1 || cap <= 0 || w_at + sizeof(double) * (size_t)cap > kStageBytes) {
			set_msg(errmsg, errmsg_len, "noalloc: weight lists exceed the 4 MiB staging limit");
			return 0;
		}
		int kind = 0;
		double edge = 0.0;
		int n = weights_into(d[k], 0, n_in, n_out, 0.0, off, (int *)(g_stage + src_at),
			(double *)(g_stage + w_at), nullptr, (int)cap, &kind, &edge);
		if(n < 0) {
			set_msg(errmsg, errmsg_len, "noalloc: weight lists exceed the 4 MiB staging limit");
			return 0;
		}
		// pack the weights right after the used part of the source list
		size_t w_final = ((src_at + sizeof(int) * (size_t)n) + 255) & ~(size_t)255;
		memmove(g_stage + w_final, g_stage + w_at, sizeof(double) * (size_t)n);
		bump.used = w_final + sizeof(double) * (size_t)n;
		DWeights &W = dw[k];
		W = DWeights{};
		W.kind = kind;
		W.n_in = n_in;
		W.n_out = n_out;
		W.edge_value = edge;
		W.off = (const int *)(scratch + off_at);
		W.src = (const int *)(scratch + src_at);
		W.w = (const double *)(scratch + w_final);
	}
	const size_t stage_used = bump.used;

	// ---- the intermediate image ----
	const size_t interm_bytes = sizeof(float) * (size_t)nch * (size_t)dst_h * (size_t)src_w;
	const size_t interm_at = (stage_used + 255) & ~(size_t)255;
	if(interm_at > kScratchBytes || interm_bytes > kScratchBytes - interm_at) {
		snprintf(buf, sizeof(buf), "noalloc: job needs %llu bytes of device scratch; the limit is %llu (32 MiB)",
			(unsigned long long)(interm_at + interm_bytes), (unsigned long long)kScratchBytes);
		set_msg(errmsg, errmsg_len, buf);
		return 0;
	}

	NAJob J{};
	J.in = src;
	J.in_bpr = src_bpr;
	J.in_w = src_w;
	J.in_h = src_h;
	J.nch = nch;
	J.alpha = (imgtype == IW_IMGTYPE_GRAYA || imgtype == IW_IMGTYPE_RGBA) ? nch - 1 : -1;
	J.out = dst;
	J.out_bpr = dst_bpr;
	J.out_w = dst_w;
	J.out_h = dst_h;
	J.tab_c = (const double *)(scratch + ((unsigned char *)T->tab_c - g_stage));
	J.tab_a = (const double *)(scratch + ((unsigned char *)T->tab_a - g_stage));
	// nearest-colour table: 8-bit non-linear output of more than 512 pixels
	// (src/imagew-main.c:1197-1236)
	const bool use_nc = cstype != IW_CSTYPE_LINEAR && (size_t)dst_w * (size_t)dst_h > 512;
	J.qc = make_dquant(scratch, T, true, use_nc);
	J.qa = make_dquant(scratch, T, false, false);
	J.wh = dw[0];
	J.wv = dw[1];
	J.interm = (float *)(scratch + interm_at);

	cudaStream_t st = (cudaStream_t)stream;
	// A copy from pageable memory returns once the bytes are staged, so the
	// next call may rebuild g_stage right away.
	cudaError_t e = cudaMemcpyAsync(scratch, g_stage, stage_used, cudaMemcpyHostToDevice, st);
	if(e == cudaSuccess) {
		dim3 blk(128);
		k_na_vpass<<<dim3((unsigned)((src_w + 127) / 128), (unsigned)dst_h), blk, 0, st>>>(J);
		e = cudaGetLastError();
	}
	if(e == cudaSuccess) {
		k_na_hpass<<<dim3((unsigned)((dst_w + 127) / 128), (unsigned)dst_h), dim3(128), 0, st>>>(J);
		e = cudaGetLastError();
	}
	if(e != cudaSuccess) {
		snprintf(buf, sizeof(buf), "noalloc: launch failed: %s", cudaGetErrorString(e));
		set_msg(errmsg, errmsg_len, buf);
		return 0;
	}
	return 1;
}
