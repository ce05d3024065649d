// server.cpp -- a request loop over the batch machinery (iwg_server_*).
//
// Requests are configured contexts.  Three stages run concurrently:
//   * planning: a pool of host threads plans requests as they arrive
//     (weight lists, tables: the host part of iw_process_image);
//   * device: one dispatcher takes every planned request that fits the
//     device-memory budget and runs them as one batch (run_batch: one launch
//     per kernel variant for all of them; requests the batched form does not
//     take run alone right after).  Requests that arrive while a batch is on
//     the GPU are planned meanwhile and join the next batch, so the GPU goes
//     from one batch to the next without waiting for the host.  Requests
//     with error-diffusion or random dither end in a serial scan that can take
//     far longer than a batch; they go to scan workers, each with a device
//     lane of its own (stream and buffers), running concurrently with the
//     batches and with each other.  Small and large scans queue apart and have
//     workers of their own, so a small request never waits behind a long scan;
//     a worker runs everything of its class that is queued as one batch (one
//     block per image, all scans at once);
//   * finishing: the output post-pass, then the request is reported done;
//     large outputs have finishing threads of their own, so that the
//     post-pass of a large image never delays a small one.
// Each request's bytes equal what iw_process_image() gives it alone.
#include "iwg_internal.h"
#include "imagew_gb300.h"

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

namespace iwg {

using SrvClock = std::chrono::steady_clock;

struct Request {
	iw_context *ctx = nullptr;
	unsigned long long tag = 0;
	Plan plan;
	size_t bytes = 0;
	int ok = 0;
	SrvClock::time_point t_submit;
	double latency_ms = 0;
	double planned_ms = 0, started_ms = 0, ran_ms = 0;   // phase ends, from submit
	double since_submit() const { return std::chrono::duration<double, std::milli>(SrvClock::now() - t_submit).count(); }
};

}  // namespace iwg

struct iwg_server {
	size_t budget = 0;
	int max_batch = 0;
	std::mutex mu;
	std::condition_variable cv_intake, cv_planned, cv_done, cv_finish;
	std::condition_variable cv_slow;
	std::deque<iwg::Request *> intake, planned, done;
	std::deque<iwg::Request *> finishing[2];   // post-pass: small, large outputs
	std::deque<iwg::Request *> slow[2];   // serial-scan requests: small, large
	bool stopping = false;
	int in_flight = 0;                 // submitted, not yet polled out
	std::vector<std::thread> planners, finishers, scan_workers;
	std::thread dispatcher;
	size_t slow_bytes = 0;             // device bytes held by the scan workers' requests
	// statistics
	long long batches = 0, batched_requests = 0;
	double device_ms = 0;
	long long slow_batches = 0, slow_requests = 0;   // scan lanes (serial dither scans)
	double slow_device_ms = 0;
	double batch_wall_ms = 0, rest_wall_ms = 0, plan_ms = 0;
};

namespace {

// Output samples from which a request counts as large (scan workers, post-pass).
constexpr long long kLargeScan = 1LL << 20;

int size_class(const iwg::Request *r)
{
	return (long long)r->plan.out_w * r->plan.out_h * r->plan.out_n >= kLargeScan ? 1 : 0;
}

void planner_loop(iwg_server *S)
{
	for(;;) {
		iwg::Request *r;
		{
			std::unique_lock<std::mutex> lk(S->mu);
			S->cv_intake.wait(lk, [&] { return S->stopping || !S->intake.empty(); });
			if(S->intake.empty()) return;
			r = S->intake.front();
			S->intake.pop_front();
		}
		iw_context *ctx = r->ctx;
		const auto t0 = iwg::SrvClock::now();
		if(ctx->use_count > 0) iw_set_error(ctx, "Internal: Incorrect attempt to reprocess image");
		else {
			ctx->use_count++;
			r->ok = iwg::build_plan(ctx, r->plan) ? 1 : 0;
		}
		if(r->ok) r->bytes = iwg::batch_device_bytes(r->plan);
		const double ms = std::chrono::duration<double, std::milli>(iwg::SrvClock::now() - t0).count();
		r->planned_ms = r->since_submit();
		std::lock_guard<std::mutex> lk(S->mu);
		S->plan_ms += ms;
		if(r->ok && iwg::plan_needs_scan(r->plan)) {
			S->slow[size_class(r)].push_back(r);
			S->cv_slow.notify_all();
		}
		else if(r->ok) {
			S->planned.push_back(r);
			S->cv_planned.notify_one();
		}
		else {
			r->latency_ms = std::chrono::duration<double, std::milli>(iwg::SrvClock::now() - r->t_submit).count();
			S->done.push_back(r);
			S->cv_done.notify_all();
		}
	}
}

// Runs requests as one plain-form batch on 'lane' (alone if that fails to
// take one), then hands them to the finishing stage.
void run_plain(iwg_server *S, std::vector<iwg::Request *> &batch, int lane)
{
	for(iwg::Request *r : batch) r->started_ms = r->since_submit();
	std::vector<char> handed(batch.size(), 0);
	if(!batch.empty()) {
		std::vector<iw_context *> cc;
		std::vector<iwg::Plan *> pp;
		for(iwg::Request *r : batch) {
			cc.push_back(r->ctx);
			pp.push_back(&r->plan);
		}
		std::vector<int> status;
		double dev_ms = 0;
		// on a scan lane each request goes on to its post-pass as soon as its
		// own scan is done, not when the batch's longest one is
		auto on_done = [&](int k) {
			iwg::Request *r = batch[k];
			r->ok = 1;
			r->ran_ms = r->since_submit();
			handed[k] = 1;
			std::lock_guard<std::mutex> lk(S->mu);
			S->finishing[size_class(r)].push_back(r);
			S->cv_finish.notify_all();
		};
		iwg::run_batch_plain(cc, pp, status, dev_ms, lane, lane != 0 ? std::function<void(int)>(on_done) : nullptr);
		for(size_t k = 0; k < batch.size(); k++) {
			if(handed[k]) continue;
			if(status[k] == 1) batch[k]->ok = 1;
			else if(status[k] == 0) batch[k]->ok = iwg::run_pipeline(batch[k]->ctx, batch[k]->plan, 0, 1, lane) ? 1 : 0;
			else batch[k]->ok = 0;
		}
		std::lock_guard<std::mutex> lk(S->mu);
		S->device_ms += dev_ms;
		if(lane >= 1) {
			S->slow_batches++;
			S->slow_requests += (long long)batch.size();
			S->slow_device_ms += dev_ms;
		}
	}
	for(size_t k = 0; k < batch.size(); k++) if(!handed[k]) batch[k]->ran_ms = batch[k]->since_submit();
	std::lock_guard<std::mutex> lk(S->mu);
	for(size_t k = 0; k < batch.size(); k++) if(!handed[k]) S->finishing[size_class(batch[k])].push_back(batch[k]);
	S->cv_finish.notify_all();
}

void dispatcher_loop(iwg_server *S)
{
	for(;;) {
		std::vector<iwg::Request *> batch;
		{
			std::unique_lock<std::mutex> lk(S->mu);
			S->cv_planned.wait(lk, [&] { return S->stopping || !S->planned.empty(); });
			if(S->planned.empty()) {
				if(S->stopping && S->intake.empty()) return;
				continue;
			}
			// admission: everything planned that fits the budget (at least one)
			size_t bytes = 0;
			while(!S->planned.empty() && (int)batch.size() < S->max_batch) {
				iwg::Request *r = S->planned.front();
				if(!batch.empty() && bytes + r->bytes > S->budget) break;
				bytes += r->bytes;
				batch.push_back(r);
				S->planned.pop_front();
			}
		}
		std::vector<iw_context *> cc;
		std::vector<iwg::Plan *> pp;
		for(iwg::Request *r : batch) {
			cc.push_back(r->ctx);
			pp.push_back(&r->plan);
		}
		std::vector<int> status;
		double dev_ms = 0;
		const auto t0 = iwg::SrvClock::now();
		for(iwg::Request *r : batch) r->started_ms = r->since_submit();
		iwg::run_batch(cc, pp, status, dev_ms);
		const auto t1 = iwg::SrvClock::now();
		std::vector<iwg::Request *> rest, finished;
		for(size_t k = 0; k < batch.size(); k++) {
			if(status[k] == 0) rest.push_back(batch[k]);
			else {
				batch[k]->ok = status[k] == 1;
				batch[k]->ran_ms = batch[k]->since_submit();
				finished.push_back(batch[k]);
			}
		}
		{
			std::lock_guard<std::mutex> lk(S->mu);
			S->batches++;
			S->batched_requests += (long long)batch.size();
			S->device_ms += dev_ms;
			S->batch_wall_ms += std::chrono::duration<double, std::milli>(t1 - t0).count();
			for(iwg::Request *r : finished) S->finishing[size_class(r)].push_back(r);
			S->cv_finish.notify_all();
		}
		run_plain(S, rest, 0);
		const double rest_ms = std::chrono::duration<double, std::milli>(iwg::SrvClock::now() - t1).count();
		std::lock_guard<std::mutex> lk(S->mu);
		S->rest_wall_ms += rest_ms;
	}
}

// A scan worker of class 'cls' (0 small, 1 large): takes queued requests of
// its class that fit the device budget the workers share (a worker may take
// one request whatever the budget when no other scan holds memory), at most
// kScanBatch[cls] of them, and runs them as one batch on its own lane (their
// scans concurrently, each request handed on as its own scan ends).  Large
// scans take seconds and a worker holds its lane until its batch ends, so a
// request that arrives while lanes are idle gets one alone; only a backlog
// fills batches, up to four per lane, of similar sizes.  (Measured with two
// in arrival order: the serving configuration's error-diffused upscales need
// about 30 lane-seconds per second against 27 large lanes, and their queue
// still grew.)
constexpr int kScanBatch[2] = {16, 4};
constexpr size_t kMatchWindow = 64;

long long out_samples(const iwg::Request *r)
{
	return (long long)r->plan.out_w * r->plan.out_h * r->plan.out_n;
}

void slow_loop(iwg_server *S, int lane, int cls)
{
	std::deque<iwg::Request *> &q = S->slow[cls];
	const int max_batch = std::min(S->max_batch, kScanBatch[cls]);
	for(;;) {
		std::vector<iwg::Request *> batch;
		size_t bytes = 0;
		{
			std::unique_lock<std::mutex> lk(S->mu);
			S->cv_slow.wait(lk, [&] {
				return (S->stopping && q.empty()) ||
					(!q.empty() && (S->slow_bytes == 0 || S->slow_bytes + q.front()->bytes <= S->budget));
			});
			if(q.empty()) return;
			// the oldest request, then queued ones of a similar size (output
			// within a factor of two of its own, among the next kMatchWindow):
			// the batch holds the lane until its largest scan ends, so
			// similar sizes keep every scan of it busy that long
			const long long s0 = out_samples(q.front());
			for(size_t i = 0; i < q.size() && i < kMatchWindow && (int)batch.size() < max_batch;) {
				iwg::Request *r = q[i];
				const long long sr = out_samples(r);
				if(!batch.empty() && (2 * sr < s0 || sr > 2 * s0)) {
					i++;
					continue;
				}
				if((!batch.empty() || S->slow_bytes > 0) && S->slow_bytes + bytes + r->bytes > S->budget) break;
				bytes += r->bytes;
				batch.push_back(r);
				q.erase(q.begin() + (std::ptrdiff_t)i);
			}
			S->slow_bytes += bytes;
		}
		run_plain(S, batch, lane);
		std::lock_guard<std::mutex> lk(S->mu);
		S->slow_bytes -= bytes;
		S->cv_slow.notify_all();
	}
}

void finisher_loop(iwg_server *S, int cls)
{
	std::deque<iwg::Request *> &q = S->finishing[cls];
	for(;;) {
		iwg::Request *r;
		{
			std::unique_lock<std::mutex> lk(S->mu);
			S->cv_finish.wait(lk, [&] { return S->stopping || !q.empty(); });
			if(q.empty()) {
				if(S->stopping && S->intake.empty() && S->planned.empty() && S->slow[0].empty() && S->slow[1].empty()) return;
				continue;
			}
			r = q.front();
			q.pop_front();
		}
		if(r->ok) {
			iwg::bkgd_label(r->ctx, r->plan);
			iwg::optimize(r->ctx);
		}
		r->latency_ms = std::chrono::duration<double, std::milli>(iwg::SrvClock::now() - r->t_submit).count();
		r->ctx->stats.ms_total = r->latency_ms;
		std::lock_guard<std::mutex> lk(S->mu);
		S->done.push_back(r);
		S->cv_done.notify_all();
	}
}

}  // namespace

extern "C" struct iwg_server *iwg_server_create(size_t device_budget, int max_batch, int host_threads)
{
	iwg_server *S = new iwg_server();
	S->budget = device_budget ? device_budget : ((size_t)8 << 30);
	S->max_batch = max_batch > 0 ? max_batch : 4096;
	int T = host_threads > 0 ? host_threads : (int)std::thread::hardware_concurrency();
	T = std::max(2, T);
	const int nplan = std::max(1, T - T / 4), nfin = std::max(1, T / 4);
	for(int k = 0; k < nplan; k++) S->planners.emplace_back(planner_loop, S);
	for(int k = 0; k < 2 * nfin; k++) S->finishers.emplace_back(finisher_loop, S, k & 1);
	S->dispatcher = std::thread(dispatcher_loop, S);
	for(int lane = 1; lane < iwg::kLanes; lane++)
		S->scan_workers.emplace_back(slow_loop, S, lane, lane <= iwg::kSmallScanLanes ? 0 : 1);
	return S;
}

extern "C" int iwg_server_submit(struct iwg_server *S, struct iw_context *ctx, unsigned long long tag)
{
	if(!S || !ctx) return 0;
	iwg::Request *r = new iwg::Request();
	r->ctx = ctx;
	r->tag = tag;
	r->t_submit = iwg::SrvClock::now();
	std::lock_guard<std::mutex> lk(S->mu);
	if(S->stopping) {
		delete r;
		return 0;
	}
	S->intake.push_back(r);
	S->in_flight++;
	S->cv_intake.notify_one();
	return 1;
}

extern "C" int iwg_server_poll(struct iwg_server *S, struct iwg_completion *out, int max, int wait_ms)
{
	if(!S || !out || max <= 0) return 0;
	std::unique_lock<std::mutex> lk(S->mu);
	if(S->done.empty() && wait_ms != 0) {
		auto pred = [&] { return !S->done.empty(); };
		if(wait_ms < 0) S->cv_done.wait(lk, pred);
		else S->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), pred);
	}
	int n = 0;
	while(n < max && !S->done.empty()) {
		iwg::Request *r = S->done.front();
		S->done.pop_front();
		out[n].tag = r->tag;
		out[n].ok = r->ok;
		out[n].latency_ms = r->latency_ms;
		out[n].planned_ms = r->planned_ms;
		out[n].started_ms = r->started_ms;
		out[n].ran_ms = r->ran_ms;
		S->in_flight--;
		delete r;
		n++;
	}
	return n;
}

extern "C" int iwg_server_info(struct iwg_server *S, struct iwg_server_stats *out)
{
	if(!S || !out) return 0;
	std::lock_guard<std::mutex> lk(S->mu);
	out->in_flight = S->in_flight;
	out->queued = (int)(S->intake.size() + S->planned.size() + S->slow[0].size() + S->slow[1].size());
	out->batches = S->batches;
	out->batched_requests = S->batched_requests;
	out->device_ms = S->device_ms;
	out->slow_batches = S->slow_batches;
	out->slow_requests = S->slow_requests;
	out->slow_device_ms = S->slow_device_ms;
	out->batch_wall_ms = S->batch_wall_ms;
	out->rest_wall_ms = S->rest_wall_ms;
	out->plan_ms = S->plan_ms;
	iwg::batch_phase_ms(out->batch_phase_ms);
	return 1;
}

extern "C" void iwg_server_destroy(struct iwg_server *S)
{
	if(!S) return;
	{
		// finish everything submitted, then stop the stages
		std::unique_lock<std::mutex> lk(S->mu);
		S->cv_done.wait(lk, [&] { return S->intake.empty() && S->planned.empty() && S->slow[0].empty() && S->slow[1].empty() &&
			S->finishing[0].empty() && S->finishing[1].empty() && (int)S->done.size() >= S->in_flight; });
		S->stopping = true;
		S->cv_intake.notify_all();
		S->cv_planned.notify_all();
		S->cv_slow.notify_all();
		S->cv_finish.notify_all();
	}
	for(std::thread &t : S->planners) t.join();
	S->dispatcher.join();
	for(std::thread &t : S->scan_workers) t.join();
	for(std::thread &t : S->finishers) t.join();
	for(iwg::Request *r : S->done) delete r;
	delete S;
}
