// fastbatch.cu -- the FP32 + guard-band form for a batch of images.
//
// A batch runs each pass as one launch per kernel variant (template instance)
// instead of one launch per image: every block finds its image with a binary
// search over a prefix table of per-image block counts, copies that image's
// FJob into shared memory and runs the same tile body as the per-image kernel
// (fastkern.cuh).  Images keep their own weight lists, tables and buffers, so
// each result is byte-identical to processing the image alone.
#include "fastkern.cuh"
#include "fastpath.cuh"
#include "iwg_internal.h"

#include <algorithm>
#include <chrono>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

namespace iwg {
namespace {

using namespace fp;

// Position g of the largest start[g] <= b (start ascending, start[0] == 0).
__device__ __forceinline__ int find_image(const int *start, int n, int b)
{
	int lo = 0, hi = n - 1;
	while(lo < hi) {
		const int mid = (lo + hi + 1) >> 1;
		if(__ldg(start + mid) <= b) lo = mid; else hi = mid - 1;
	}
	return lo;
}

// Copies an image's job description into shared memory (whole block).
__device__ __forceinline__ void load_job(FJob &dst, const FJob *src)
{
	const int *s = reinterpret_cast<const int *>(src);
	int *d = reinterpret_cast<int *>(&dst);
	for(int k = threadIdx.x; k < (int)(sizeof(FJob) / sizeof(int)); k += blockDim.x) d[k] = __ldg(s + k);
	__syncthreads();
}

template<int NS, int NCH, bool ALPHA, int DEPTH, int PX>
__global__ void __launch_bounds__(kVPxThreads) kb_vstream_px(const FJob *jobs, const int *idx, const int *start, int n)
{
	extern __shared__ __align__(16) float s_dyn[];
	__shared__ FJob sF;
	const int g = find_image(start, n, blockIdx.x);
	load_job(sF, jobs + idx[g]);
	const int local = blockIdx.x - start[g];
	vstream_px_tile<NS, NCH, ALPHA, DEPTH, PX>(sF, s_dyn, local % sF.vgx, local / sF.vgx);
}

template<int NS, int NCH, bool ALPHA, int DEPTH, int PX>
__global__ void __launch_bounds__(kBulkThreads, 2) kb_vbulk(const FJob *jobs, const int *idx, const int *start, int n)
{
	extern __shared__ __align__(128) unsigned char s_bulk[];
	__shared__ FJob sF;
	const int g = find_image(start, n, blockIdx.x);
	load_job(sF, jobs + idx[g]);
	const int local = blockIdx.x - start[g];
	vbulk_tile<NS, NCH, ALPHA, DEPTH, PX>(sF, s_bulk, local % sF.vgx, local / sF.vgx);
}

template<int NS, int NPL, int DEPTH>
__global__ void __launch_bounds__(kVThreads) kb_vstream(const FJob *jobs, const int *idx, const int *start, int n)
{
	extern __shared__ __align__(16) float s_dyn[];
	__shared__ FJob sF;
	const int g = find_image(start, n, blockIdx.x);
	load_job(sF, jobs + idx[g]);
	const int local = blockIdx.x - start[g];
	vstream_tile<NS, NPL, DEPTH>(sF, s_dyn, local % sF.vgx, local / sF.vgx);
}

template<int NPL, int DEPTH>
__global__ void __launch_bounds__(kVThreads) kb_vgather(const FJob *jobs, const int *idx, const int *start, int n)
{
	extern __shared__ __align__(16) float s_dyn[];
	__shared__ FJob sF;
	const int g = find_image(start, n, blockIdx.x);
	load_job(sF, jobs + idx[g]);
	const int local = blockIdx.x - start[g];
	vgather_tile<NPL, DEPTH>(sF, s_dyn, local % sF.vgx, local / sF.vgx);
}

template<int NPL>
__global__ void __launch_bounds__(kHThreads) kb_hpass(const FJob *jobs, const int *idx, const int *start, int n)
{
	__shared__ FJob sF;
	const int g = find_image(start, n, blockIdx.x);
	load_job(sF, jobs + idx[g]);
	const int local = blockIdx.x - start[g];
	hpass_pixel<NPL>(sF, (local % sF.hgx) * blockDim.x + threadIdx.x, local / sF.hgx);
}

const void *batch_vkernel(const VVariant &v)
{
#define IWG_BPX(NS_, NCH_, A_, D_, PX_) \
	if(v.kind == 1 && v.ns == NS_ && v.nch == NCH_ && v.alpha == (int)A_ && v.depth == D_ && v.px == PX_) \
		return (const void *)kb_vstream_px<NS_, NCH_, A_, D_, PX_>;
#define IWG_BST(NS_, NPL_, D_) \
	if(v.kind == 2 && v.ns == NS_ && v.nch == NPL_ && v.depth == D_) return (const void *)kb_vstream<NS_, NPL_, D_>;
#define IWG_BGA(NPL_, D_) \
	if(v.kind == 3 && v.nch == NPL_ && v.depth == D_) return (const void *)kb_vgather<NPL_, D_>;
#define IWG_BBU(NS_, NCH_, A_, D_, PX_) \
	if(v.kind == 4 && v.ns == NS_ && v.nch == NCH_ && v.alpha == (int)A_ && v.depth == D_ && v.px == PX_) \
		return (const void *)kb_vbulk<NS_, NCH_, A_, D_, PX_>;
	IWG_VBULK_VARIANTS(IWG_BBU)
#undef IWG_BBU
	IWG_VPX_VARIANTS(IWG_BPX)
	IWG_VSTREAM_VARIANTS(IWG_BST)
	IWG_VGATHER_VARIANTS(IWG_BGA)
#undef IWG_BPX
#undef IWG_BST
#undef IWG_BGA
	return nullptr;
}

const void *batch_hkernel(int npl)
{
	switch(npl) {
	case 1: return (const void *)kb_hpass<1>;
	case 2: return (const void *)kb_hpass<2>;
	case 3: return (const void *)kb_hpass<3>;
	default: return (const void *)kb_hpass<4>;
	}
}

struct Group {
	const void *kernel = nullptr;
	int threads = 0;
	size_t smem = 0;
	std::vector<int> idx, start;
	long long blocks = 0;
	size_t off_idx = 0, off_start = 0;
};

// Grow-only device buffer for the batch's job array and block tables, one
// per stream: a batch writes its tables and launches its kernels on its own
// stream, so the next batch's writes into the same buffer are ordered after
// them, and batches on other streams (lanes) never share it.
struct BatchArena {
	void *p = nullptr;
	size_t cap = 0;
	bool ensure(size_t n, cudaStream_t st)   // stream-ordered: never waits for other streams
	{
		if(n <= cap) return true;
		if(p) cudaFreeAsync(p, st);
		p = nullptr;
		cap = 0;
		if(cudaMallocAsync(&p, n + n / 4, st) != cudaSuccess) {
			cudaGetLastError();
			return false;
		}
		cap = n + n / 4;
		return true;
	}
};

BatchArena &arena(cudaStream_t st)
{
	static std::mutex mu;
	static auto *m = new std::map<cudaStream_t, BatchArena>();
	std::lock_guard<std::mutex> lk(mu);
	return (*m)[st];   // std::map: references stay valid as entries are added
}

}  // namespace

void preload_batch_kernels()
{
	cudaFuncAttributes a;
#define IWG_PRE_BU(NS_, NCH_, A_, D_, PX_) cudaFuncGetAttributes(&a, (const void *)kb_vbulk<NS_, NCH_, A_, D_, PX_>);
#define IWG_PRE_PX(NS_, NCH_, A_, D_, PX_) cudaFuncGetAttributes(&a, (const void *)kb_vstream_px<NS_, NCH_, A_, D_, PX_>);
#define IWG_PRE_ST(NS_, NPL_, D_) cudaFuncGetAttributes(&a, (const void *)kb_vstream<NS_, NPL_, D_>);
#define IWG_PRE_GA(NPL_, D_) cudaFuncGetAttributes(&a, (const void *)kb_vgather<NPL_, D_>);
	IWG_VBULK_VARIANTS(IWG_PRE_BU)
	IWG_VPX_VARIANTS(IWG_PRE_PX)
	IWG_VSTREAM_VARIANTS(IWG_PRE_ST)
	IWG_VGATHER_VARIANTS(IWG_PRE_GA)
#undef IWG_PRE_BU
#undef IWG_PRE_PX
#undef IWG_PRE_ST
#undef IWG_PRE_GA
	for(int npl = 1; npl <= 4; npl++) cudaFuncGetAttributes(&a, batch_hkernel(npl));
	cudaGetLastError();
}

int fast_launch_batch(cudaStream_t st, void *const *items, int n, std::string &err, cudaEvent_t after_vertical,
	cudaEvent_t after_horizontal, const std::function<int()> &tail, bool *graphed)
{
	if(graphed) *graphed = false;
	if(n <= 0) return 0;
	std::vector<Group> vg, hg;
	auto group_of = [](std::vector<Group> &gs, const void *k) -> Group & {
		for(Group &g : gs) if(g.kernel == k) return g;
		gs.emplace_back();
		gs.back().kernel = k;
		return gs.back();
	};
	for(int i = 0; i < n; i++) {
		const FastState &S = *static_cast<const FastState *>(items[i]);
		const void *vk = batch_vkernel(S.vv);
		if(!vk) {
			err = "batch: no batched kernel for an image's layout";
			return -1;
		}
		Group &v = group_of(vg, vk);
		v.threads = S.vthreads;
		v.smem = std::max(v.smem, S.vsmem);
		v.idx.push_back(i);
		v.start.push_back((int)v.blocks);
		v.blocks += (long long)S.F.vgx * S.F.vgy;
		Group &h = group_of(hg, batch_hkernel(S.F.npl));
		h.threads = kHThreads;
		h.idx.push_back(i);
		h.start.push_back((int)h.blocks);
		h.blocks += (long long)S.F.hgx * S.F.out_h;
	}
	// layout: FJob array, then each group's image list and block starts
	std::vector<uint8_t> host;
	auto add = [&](const void *p, size_t bytes) {
		size_t off = (host.size() + 255) & ~(size_t)255;
		host.resize(off + bytes);
		memcpy(host.data() + off, p, bytes);
		return off;
	};
	std::vector<FJob> jobs(n);
	for(int i = 0; i < n; i++) jobs[i] = static_cast<const FastState *>(items[i])->F;
	const size_t off_jobs = add(jobs.data(), jobs.size() * sizeof(FJob));
	for(std::vector<Group> *gs : {&vg, &hg}) {
		for(Group &g : *gs) {
			if(g.blocks > 0x7fffffffLL) {
				err = "batch: too many blocks in one launch";
				return -1;
			}
			g.off_idx = add(g.idx.data(), g.idx.size() * sizeof(int));
			g.off_start = add(g.start.data(), g.start.size() * sizeof(int));
		}
	}
	const auto t_tab = std::chrono::steady_clock::now();
	BatchArena &A = arena(st);
	if(!A.ensure(host.size(), st)) {
		err = "Out of GPU memory (batch tables)";
		return -1;
	}
	uint8_t *base = (uint8_t *)A.p;
	cudaMemcpyAsync(base, host.data(), host.size(), cudaMemcpyHostToDevice, st);
	batch_phase_add(6, std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_tab).count());
	const FJob *djobs = (const FJob *)(base + off_jobs);
	int launches = 0;
	auto launch = [&](Group &g) -> bool {
		if(g.blocks == 0) return true;
		const auto t_attr = std::chrono::steady_clock::now();
		if(g.smem > 48 * 1024 &&
			cudaFuncSetAttribute(g.kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem) != cudaSuccess) {
			err = "batch: shared memory request refused";
			return false;
		}
		batch_phase_add(7, std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_attr).count());
		const int *didx = (const int *)(base + g.off_idx);
		const int *dstart = (const int *)(base + g.off_start);
		int ng = (int)g.idx.size();
		void *args[] = {(void *)&djobs, (void *)&didx, (void *)&dstart, (void *)&ng};
		cudaError_t e = cudaLaunchKernel(g.kernel, dim3((unsigned)g.blocks), dim3(g.threads), args, g.smem, st);
		if(e != cudaSuccess) {
			err = std::string("batch launch: ") + cudaGetErrorString(e);
			return false;
		}
		launches++;
		return true;
	};
	// shared-memory attributes before the capture (host-side calls)
	for(std::vector<Group> *gs : {&vg, &hg})
		for(Group &g : *gs)
			if(g.blocks > 0 && g.smem > 48 * 1024 &&
				cudaFuncSetAttribute(g.kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem) != cudaSuccess) {
				err = "batch: shared memory request refused";
				return -1;
			}
	auto issue = [&]() -> int {
		launches = 0;
		for(Group &g : vg) if(!launch(g)) return -1;
		if(after_vertical) cudaEventRecord(after_vertical, st);
		for(Group &g : hg) if(!launch(g)) return -1;
		if(after_horizontal) cudaEventRecord(after_horizontal, st);
		if(tail) {
			const int t = tail();
			if(t < 0) return -1;
			launches += t;
		}
		return launches;
	};
	if(!graphed) return issue();
	return run_as_graph(st, issue, graphed);
}

}  // namespace iwg
