// iwg_internal.h -- private state of libimagew_gb300.
//
// The library keeps the reference's settings model (a context collects
// settings, then iw_process_image() runs once), but splits the work into
//   1. host planning (plan.cpp): every decision the reference makes in
//      iw_prepare_processing (src/imagew-main.c:1899-2248), resolved into a
//      Plan that describes the pixel work as data;
//   2. host tables (weights.cpp, tables.cpp): resampling weights, input
//      transfer tables and quantisation tables, built with the host libm so
//      that every transcendental value equals the reference's;
//   3. device work (pipeline.cu): the pixel passes as CUDA kernels;
//   4. the host post-pass (optimize.cpp, src/imagew-opt.c).
#pragma once

#define IW_INCLUDE_UTIL_FUNCTIONS
#include "imagew.h"

#include <cstddef>
#include <cstdint>
#include <functional>
#include <memory>
#include <string>
#include <vector>

namespace iwg {

constexpr int kNCTypes = 5;   // R, G, B, A, Gray
constexpr int kMaxCh = 4;
constexpr int kMsgMax = 200;

// ---------------------------------------------------------------------------
// Resampling weights for one dimension (one channel class).
// ---------------------------------------------------------------------------
enum class RowKind : int { Sum = 0, Copy = 1 };

struct Weights {
	RowKind kind = RowKind::Sum;
	int n_in = 0, n_out = 0;
	double edge_value = 0.0;          // value of a virtual (transparent-edge) pixel
	// CSR, one list per output pixel in the reference's accumulation order.
	// src == -1: virtual pixel (Sum) / "no source, value 0" (Copy).
	std::vector<int> off;              // n_out + 1
	std::vector<int> src;
	std::vector<double> w;
	int max_taps = 0;
	// Window in "virtual input position" space used by the streaming kernels:
	// pos_first[o] .. pos_last[o] covers every tap of output o.
	std::vector<int> pos;              // per tap: virtual position (may be <0 or >=n_in)
	double wsum_abs_max = 0.0;         // max over outputs of sum |w|
	double wsum_neg_max = 0.0;         // max over outputs of sum of |negative w|
	bool same_as(const Weights &o) const;
};

// ---------------------------------------------------------------------------
// Quantisation of one output channel (src/imagew-main.c:570-765).
// ---------------------------------------------------------------------------
struct Quant {
	int float_out = 0;        // write (float)v, no quantisation
	int use_nc = 0;           // nearest-colour table path
	int dfam = 0, dsub = 0;   // dither family / subtype
	int maxcc = 255;          // M
	int cc = 0;               // colour count (0 = all codes)
	int P = 255;              // number of brackets - 1 (M, or cc-1)
	int cstype = 0;
	double gamma = 0.0;
	// shared, cached tables
	std::shared_ptr<const std::vector<double>> U;    // P+2: U[0]=-inf, U[k] = min v with g(v)>=k, U[P+1]=+inf
	std::shared_ptr<const std::vector<double>> X;    // P+1: min v with g(v) > k  (X[P] = +inf)
	std::shared_ptr<const std::vector<int>> code;    // P+2: bracket -> output code (code[P+1] = code[P])
	std::shared_ptr<const std::vector<double>> rev;  // M+1: code -> linear value
	std::shared_ptr<const std::vector<double>> nc;   // 255 midpoints (use_nc only)
	// error diffusion only: per bracket k, 8 words {U[k], U[k+1], X[k], C[k]
	// (bit patterns), rev[code[k]], rev[code[k+1]] (bit patterns),
	// code[k] | code[k+1] << 32, 0}, where C[k] is the least v whose ceiling
	// is at least as near as its floor (rev_hi - v <= v - rev_lo, each rounded)
	std::shared_ptr<const std::vector<long long>> rec;
};

// ---------------------------------------------------------------------------
// The resolved plan for one iw_process_image call.
// ---------------------------------------------------------------------------
struct MidChannel {
	int ctype = 0;
	int in_ch = 0;          // first input channel read
	int to_gray = 0;        // combine in_ch..in_ch+2 to gray
	int out_ch = 0;         // output channel, -1 if dropped
	int unassoc = 0;        // colour channel of an image with alpha
	double bk_early = 0.0;  // early background colour (linear)
	int wset_h = 0, wset_v = 0;  // indices of its weight sets (horizontal, vertical)
	int lin_cs = 0;         // 1: decode with the linear transfer (alpha / no-gamma)
};

struct OutChannel {
	int ctype = 0;
	int dfam = 0, dsub = 0, cc = 0, maxcc = 0;
	double bk1 = 0.0, bk2 = 0.0;
	Quant q;
};

enum { BK_EARLY = 1, BK_LATE = 2 };
enum { BKSRC_NONE = 0, BKSRC_FILE = 1, BKSRC_REQ = 2 };

struct Plan {
	// input
	int in_type = 0, in_depth = 8, in_sampletype = 0, in_nphys = 1, in_nlog = 1, in_logtype = 0;
	int in_alpha = 0;              // logical alpha channel index
	int orient = 0;
	int img1_w = 0, img1_h = 0;
	size_t in_bpr = 0;
	int crop_x = 0, crop_y = 0, crop_w = 0, crop_h = 0;
	int in_slow[kMaxCh] = {0, 0, 0, 0};
	int in_max = 0;
	double in_maxcc_d[kMaxCh] = {0, 0, 0, 0};
	int reduced_in = 0;
	struct iw_csdescr cs_in{}, cs_out{};
	int no_gamma = 0;
	int gsf = 0;
	double gsw[3] = {0, 0, 0};

	// intermediate
	int mid_type = 0, mid_n = 0, mid_alpha = -1;
	MidChannel mid[kMaxCh];

	// output
	int out_w = 0, out_h = 0, out_type = 0, out_n = 0, out_depth = 8, out_sampletype = 0;
	size_t out_bpr = 0;
	OutChannel out[kMaxCh];
	int reduced_out = 0;
	int no_out_tables = 0;
	int errdiff = 0;

	// background
	int apply_bk = 0, bk_strategy = 0, bk_checker = 0, bk_source = 0, bk_trns = 0;
	double bk1_alpha = 0.0, bk2_alpha = 0.0;
	int check_size = 1, check_origin[2] = {0, 0};
	struct iw_color inlabel_lin{};

	int intclamp = 0, negate = 0, blacken = 0;

	// resampling: weight sets per dimension (index 0 = H, 1 = V)
	std::vector<std::shared_ptr<const Weights>> wsets[2];

	// 32-bit float input in a non-linear colour space: the stored image with
	// every colour sample converted to linear light on the host (glibc pow,
	// the reference's formulas; alpha samples as they are), one double per
	// sample, lin_bpr bytes per stored row.  The device reads these instead
	// of the caller's floats.
	std::shared_ptr<const std::vector<double>> lin_in;
	size_t lin_bpr = 0;
};

// The input bytes the device passes read and their row stride: the caller's
// image, or its linearised copy (Plan::lin_in).
inline const void *plan_input(const iw_context *ctx, const Plan &P);
inline size_t plan_in_bpr(const Plan &P) { return P.lin_in ? P.lin_bpr : P.in_bpr; }

struct OptState {
	int width = 0, height = 0, imgtype = 0, bit_depth = 0;
	size_t bpr = 0;
	const iw_byte *pix = nullptr;
	iw_byte *tmp = nullptr;
	int has_trns = 0, has_partial_trns = 0, has_16bit = 0, has_color = 0;
	int pal_is_gray = 0;
	struct iw_palette *pal = nullptr;
	int has_ckey = 0;
	unsigned int ckey[3] = {0, 0, 0};
	int has_label = 0;
	unsigned int label[4] = {0, 0, 0, 0};
};

struct DimRequest {
	int family = IW_RESIZETYPE_AUTO;
	int edge = IW_EDGE_POLICY_STANDARD;
	double blur = 1.0, p1 = 0.0, p2 = 0.0;
	double translate = 0.0;
	double chan_offset[3] = {0, 0, 0};
	int use_offset = 0;    // derived
	int no_cache = 0;      // derived
	double true_size = 0;  // derived
};

// Debug readback of one call (option gpu:debug_values): the intermediate
// image [mid_n][mid_h][mid_w] and, per output sample [out_n][out_h][out_w],
// the value the quantisation starts from and its error bound (fast form;
// 0 in the plain form, whose values are the reference's).  NaN: no value.
struct DebugValues {
	std::vector<double> interm, value, bound;
	int dims[6] = {0, 0, 0, 0, 0, 0};   // mid_n, mid_h, mid_w, out_n, out_h, out_w
	void clear() { interm.clear(); value.clear(); bound.clear(); for(int &d : dims) d = 0; }
};

struct Stats {   // per call, readable through the iwg_* extension API
	double ms_total = 0, ms_device = 0;
	double ms_part[4] = {0, 0, 0, 0};   // per launch group: vertical, horizontal, fix-up / scan
	long long flagged = 0;       // pixels re-evaluated (fast form)
	long long flagged_exact = 0; // of them, pixels the double-float tier left to FP64
	int form = 0;                // 0 = plain FP64, 1 = FP32 + guard band
	int kernels = 0;             // kernel launches issued
	int zero_copy = 0;           // kernels read/wrote the host image buffers directly
	int vertical_tensor = 0;     // the vertical pass ran on the tensor cores
	int graph = 0;               // the timed passes were replayed as a CUDA graph
	int fused = 0;               // the fp32 form's passes ran as one fused launch
	double ms_phase[6] = {0, 0, 0, 0, 0, 0};   // plan, upload, device, download, post-pass, device part's wall
};

}  // namespace iwg

struct iw_context {
	// allocation and messages
	iw_mallocfn_type mallocfn = nullptr;
	iw_freefn_type freefn = nullptr;
	void *userdata = nullptr;
	size_t max_malloc = 2000000000;
	int max_w = 40000, max_h = 40000;
	int api_version = 0;
	int error_flag = 0;
	char *error_msg = nullptr;
	iw_translatefn_type xlate = nullptr;
	iw_warningfn_type warn = nullptr;

	// input
	struct iw_image img1{};
	struct iw_csdescr cs_in{};
	int in_maxcc[iwg::kMaxCh] = {0, 0, 0, 0};

	// request
	unsigned int profile = 0;
	int canvas_w = 0, canvas_h = 0;
	int crop_x = 0, crop_y = 0, crop_w = -1, crop_h = -1;
	int req_depth = 0, req_sampletype = 0;
	int req_maxcc[iwg::kNCTypes] = {0, 0, 0, 0, 0};
	int req_cc[iwg::kNCTypes] = {0, 0, 0, 0, 0};
	int dfam[iwg::kNCTypes] = {0, 0, 0, 0, 0};
	int dsub[iwg::kNCTypes] = {0, 0, 0, 0, 0};
	int true_valid = 0;
	double true_w = 0, true_h = 0;
	int req_intent = 0;
	int cs_out_valid = 0;
	struct iw_csdescr cs_out_req{};
	int no_cslabel = 0, negate = 0;
	int bkgd_valid = 0, bkgd_checker = 0;
	struct iw_color bkgd{}, bkgd2{};
	int check_size = 0, check_origin[2] = {0, 0};
	int outlabel_valid = 0;
	struct iw_color outlabel{};
	int use_file_label = 0, no_outlabel = 0;
	int inlabel_set = 0;
	struct iw_color inlabel{};
	int to_gray = 0, gsf = IW_GSF_STANDARD;
	double gsw[3] = {0, 0, 0};
	int no_gamma = 0, intclamp = 0, pref_units = 0;
	int randomize = 0, seed = 0;
	iw_byte opt_gray = 1, opt_pal = 1, opt_16to8 = 1, opt_strip = 1, opt_bintrns = 1;
	// the post-pass's property scan done on the device (pipeline.cu
	// k_out_props): bits 0-3 as OptState's has_16bit, has_trns,
	// has_partial_trns, has_color; 0x100 = valid
	int opt_dev_props = 0;
	iwg::DimRequest dim[2];
	int compression = 0, page = 0, include_screen = 1, interlaced = 0, bmp_nofh = 0, out_fmt = 0;
	struct Option { char *name; char *val; };
	Option *opts = nullptr;
	int nopts = 0;

	// results
	int use_count = 0;
	struct iw_image img2{};
	struct iw_csdescr cs_out{};
	int reduced_out = 0;
	int out_maxcc[iwg::kMaxCh] = {0, 0, 0, 0};
	iwg::OptState opt;
	iwg::Stats stats;
	iwg::DebugValues dbg;
};

namespace iwg {

inline const void *plan_input(const iw_context *ctx, const Plan &P)
{
	return P.lin_in ? (const void *)P.lin_in->data() : (const void *)ctx->img1.pixels;
}

// plan.cpp
bool build_plan(iw_context *ctx, Plan &P);
void bkgd_label(iw_context *ctx, const Plan &P);
double to_linear(double v, const struct iw_csdescr &cs);
double from_linear(double v, const struct iw_csdescr &cs);
double gray_of(const Plan &P, double r, double g, double b);

// weights.cpp
std::shared_ptr<const Weights> build_weights(iw_context *ctx, const DimRequest &d, int ctype,
	int n_in, int n_out, double edge_bkgd_value);
// Fills caller arrays without allocating: off (n_out+1), src/w/pos (cap; pos may
// be null).  Returns the tap count, -1 if cap is too small, -2 for an unknown
// filter family.
int weights_into(const DimRequest &d, int ctype, int n_in, int n_out, double edge_bkgd_value,
	int *off, int *src, double *w, int *pos, int cap, int *kind, double *edge_value);
// Upper bound on the taps of one output (-1: unknown family).
int weights_max_taps(const DimRequest &d, int n_in, int n_out);

// tables.cpp
std::shared_ptr<const std::vector<double>> input_table(int cstype, double gamma, int maxcc, int ncodes, bool linear);
void build_quant(Quant &q);
// Non-allocating fills of the quantisation tables for one output channel:
// U (P+2), X (P+1), code (P+2), rev (maxcc+1), with P = cc ? cc-1 : maxcc.
void quant_fill(int cstype, double gamma, int maxcc, int cc, double *U, double *X, int *code, double *rev);
// The 255 nearest-colour midpoints of an 8-bit channel.
void nc_fill(int cstype, double gamma, double *nc);

// optimize.cpp
void optimize(iw_context *ctx);

// pipeline.cu
// Device lanes (independent streams, buffers and table caches): lane 0 serves
// the public entry points; a request server runs its serial dither scans on
// lanes 1 .. kLanes-1 (kSmallScanLanes of them for small outputs).  Every
// lane is one stream (plus a download stream used only with staged copies):
// with CUDA_DEVICE_MAX_CONNECTIONS at 32 (set when the library loads, if the
// process has not set it), each lane's stream has a hardware queue of its
// own, so a long scan on one lane never holds up work queued on another.
constexpr int kLanes = 32;
constexpr int kSmallScanLanes = 4;
bool run_pipeline(iw_context *ctx, Plan &P, int warmup = 0, int iters = 1, int lane = 0);
// Host wall time of the batched calls' phases, summed (ms): preparation,
// uploads, the passes' launches, the fix-up's launch, device wait with
// downloads, the rest; then, inside the passes' launches, the table upload and
// the attribute calls; within the downloads (lane 0, staged), the wait for
// the device and the host copies.
constexpr int kBatchPhases = 10;
void batch_phase_ms(double *out);
void batch_phase_add(int phase, double ms);
// Whether an output channel is quantised by a serial scan (api.cpp).
bool plan_needs_scan(const Plan &P);
// Device bytes an image holds while it runs in a batch (api.cpp).
size_t batch_device_bytes(const Plan &P);
// Runs the fast-form images of a batch together (pipeline.cu); see there.
bool run_batch(const std::vector<iw_context *> &ctxs, const std::vector<Plan *> &plans, std::vector<int> &status,
	double &dev_ms, int lane = 0);
// The same in the plain (FP64) form for any image, scans in parallel
// (pipeline.cu).  On a lane other than 0, on_done(i) is called for each image
// as soon as its output is in the caller's buffer (status[i] is then 1 and
// the context is not touched again); images not reported that way follow the
// return as usual.
bool run_batch_plain(const std::vector<iw_context *> &ctxs, const std::vector<Plan *> &plans, std::vector<int> &status,
	double &dev_ms, int lane = 0, const std::function<void(int)> &on_done = nullptr);

// api.cpp
const char *get_option(iw_context *ctx, const char *name);

}  // namespace iwg
