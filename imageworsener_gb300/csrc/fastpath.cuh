// fastpath.cuh -- interface of the FP32 + guard-band form (fastpath.cu).
#pragma once

#include <functional>
#include <string>
#include <cuda_runtime.h>

#include "device.cuh"

namespace iwg {

struct Plan;

struct FastInfo {
	int streaming = 0;   // vertical pass streams input rows into register slots
	int slots = 0;       // register slots per column (streaming)
	int tc_mode = 1;     // in: vertical pass on the tensor cores: 0 never, 1 wide windows, 2 whenever eligible
	int tc = 0;          // out: the vertical pass runs on the tensor cores
	int autotune = 1;    // in: choose the vertical pass's band count by measurement (cached per geometry)
	int fuse_mode = 0;   // in: 1 fuse the vertical and horizontal passes where possible, 0 never
	int fused = 0;       // out: the passes run as one fused launch
	int wait_polls = 0;  // in: >0 shortens the vertical pipeline's bounded waits (failure tests)
	int starve = 0;      // in: 1: the pipeline's producer issues nothing, so its waits run out (failure tests)
	int *flag_count_dev = nullptr;   // device counter of pixels re-evaluated exactly
	float *dbg = nullptr;            // in: debug readback buffer of the tail's values and bounds (FJob::dbg)
	int plane_of[4] = {0, 0, 0, 0};  // out: intermediate plane of each intermediate channel
	void *state = nullptr;            // prepared launch state (fastpath.cu)
	int launches = 0;
	void (*launch_fn)(cudaStream_t, void *, void (*)(void *), void *) = nullptr;
};

// Whether the plan can run in the fast form (and how).
bool fast_eligible(const Plan &P, const dev::Job &J, FastInfo &fi);

// Uploads the fast form's per-call tables on 'st' and prepares its launches.
bool fast_prepare(cudaStream_t st, const Plan &P, dev::Job &J, FastInfo &fi, std::string &err);

// Launches the prepared fast form: vertical pass, horizontal pass with the
// guarded tail, exact re-evaluation of flagged pixels.  'mark' is called after
// each launch group.  Returns the number of kernel launches.
template<class Mark>
int fast_launch(cudaStream_t st, FastInfo &fi, Mark mark)
{
	fi.launch_fn(st, fi.state, [](void *m) { (*static_cast<Mark *>(m))(); }, &mark);
	return fi.launches;
}

// Frees the prepared state.
void fast_release(FastInfo &fi);

// Queues what 'issue' launches on 'st' as one CUDA graph: captured,
// instantiated, launched (and freed once it has run).  Returns issue's value;
// *graphed tells whether the graph ran.  If the stream cannot be captured or
// the graph not launched, the same launches are issued directly.
template<class F>
int run_as_graph(cudaStream_t st, F &&issue, bool *graphed)
{
	*graphed = false;
	if(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed) == cudaSuccess) {
		const int r = issue();
		cudaGraph_t g = nullptr;
		const cudaError_t e = cudaStreamEndCapture(st, &g);
		cudaGraphExec_t x = nullptr;
		if(e == cudaSuccess && g && r >= 0 && cudaGraphInstantiate(&x, g, 0) == cudaSuccess &&
			cudaGraphLaunch(x, st) == cudaSuccess) {
			cudaGraphExecDestroy(x);
			cudaGraphDestroy(g);
			*graphed = true;
			return r;
		}
		if(x) cudaGraphExecDestroy(x);
		if(g) cudaGraphDestroy(g);
	}
	cudaGetLastError();
	return issue();
}

// ---- batch: many images in a few launches ----
// Host preparation of one image (no device work); null with 'err' if the
// image cannot run in the fast form.  J's device pointers (input, output,
// intermediate) must already be final.
void *fast_batch_item(const Plan &P, const dev::Job &J, std::string &err);
size_t fast_item_blob_bytes(const void *item);     // per-image arrays, to copy to the device as one block
const void *fast_item_blob(const void *item);
size_t fast_item_flag_entries(const void *item);   // flag list capacity the image needs
int fast_item_htaps(const void *item);             // widest horizontal window
int fast_item_vtaps(const void *item);             // widest vertical window
// Points the image at its device copy of the blob and the shared flag list.
void fast_item_place(void *item, const uint8_t *dev_blob, int *flag_count, int *flag_list, int img, size_t flag_cap);
// Launches the vertical and horizontal passes of n placed images, one launch
// per kernel variant (fastbatch.cu).  Returns the number of launches, -1 on error.
// Load every kernel of the fast form (per image / batched) now: with lazy
// module loading a kernel's first launch loads it, which can wait for work
// running on other streams.
void preload_fast_kernels();
void preload_batch_kernels();
void preload_noalloc_kernels();   // noalloc.cu

// The launches of a batch: vertical groups, 'after_vertical' recorded,
// horizontal groups, 'after_horizontal' recorded, then 'tail()' (the
// re-evaluation launches, returning their count); the job tables are uploaded
// before them.  With graphed != nullptr they are captured and run as one CUDA
// graph (*graphed: whether it ran); nullptr: launched directly.  Returns the
// kernel launches, -1 on error.
int fast_launch_batch(cudaStream_t st, void *const *items, int n, std::string &err,
	cudaEvent_t after_vertical, cudaEvent_t after_horizontal, const std::function<int()> &tail, bool *graphed);
// Copies the image's double-float re-evaluation pointers (set by placement)
// into the caller's job record.
void fast_item_job_df(const void *item, dev::Job &J);
void fast_item_free(void *item);

}  // namespace iwg
