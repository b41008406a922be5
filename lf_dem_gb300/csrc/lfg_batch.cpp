// lfg_batch.cpp -- many independent suspensions on one GPU.
//
//  lfg_batch_*  : a rheology sweep (many suspensions of uneven N, each with
//                 its own parameters) advanced together.  Each suspension is
//                 an lfg_sim with its own CUDA stream; a pool of host worker
//                 threads steps them in round-robin slices, so kernels of
//                 different suspensions overlap on the device.  The factor
//                 and solve launch sequences of each suspension are CUDA
//                 graphs (captured once per symbolic analysis).  An autotuner
//                 picks the nested-dissection leaf size (the supernode size at
//                 the bottom of the assembly tree) per size class by timing
//                 steps.
//  lfg_server_* : a request loop.  Requests (one suspension each, run to a
//                 strain) are admitted while a slot is free and their
//                 estimated device footprint (dominated by the factor's front
//                 arena) fits in the HBM budget; admitted requests run
//                 concurrently, each on its own stream and worker thread, and
//                 new ones are admitted as others finish (continuous
//                 batching).  Each result records submit / admit / done times
//                 for time-to-strain percentiles.
//
// Suspensions never exchange data, so every suspension's result is the same
// whether it runs alone or among others: the engine's kernels are
// deterministic (no floating-point atomics on the data path) and each
// suspension's work is ordered on its own stream.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "lfg_internal.h"

namespace lfg {
int fail(lfg_status *st, int code, int info, const char *msg);
int ok(lfg_status *st);
int check_device(int device, lfg_status *st);
}
using namespace lfg;

namespace {

class WorkerPool {
public:
	explicit WorkerPool(int n)
	{
		for (int i = 0; i < n; i++) th_.emplace_back([this] { loop(); });
	}
	~WorkerPool()
	{
		{
			std::lock_guard<std::mutex> lk(mu_);
			stop_ = true;
		}
		cv_.notify_all();
		for (auto &t : th_) t.join();
	}
	void submit(std::function<void()> f)
	{
		{
			std::lock_guard<std::mutex> lk(mu_);
			q_.push_back(std::move(f));
			pending_++;
		}
		cv_.notify_one();
	}
	void wait()
	{
		std::unique_lock<std::mutex> lk(mu_);
		done_.wait(lk, [this] { return pending_ == 0; });
	}

private:
	void loop()
	{
		for (;;) {
			std::function<void()> f;
			{
				std::unique_lock<std::mutex> lk(mu_);
				cv_.wait(lk, [this] { return stop_ || !q_.empty(); });
				if (stop_ && q_.empty()) return;
				f = std::move(q_.front());
				q_.pop_front();
			}
			f();
			{
				std::lock_guard<std::mutex> lk(mu_);
				pending_--;
			}
			done_.notify_all();
		}
	}
	std::vector<std::thread> th_;
	std::mutex mu_;
	std::condition_variable cv_, done_;
	std::deque<std::function<void()>> q_;
	int pending_ = 0;
	bool stop_ = false;
};

double now_s(std::chrono::steady_clock::time_point t0)
{
	return std::chrono::duration<double>(std::chrono::steady_clock::now()-t0).count();
}

// size class of a suspension for the autotuner: half-octaves of N, precision
int size_class(int n, int precision) { return 2*(int)std::lround(2*std::log2((double)std::max(n, 1)))+precision; }

} // namespace

// ---------------------------------------------------------------------------
// batch
// ---------------------------------------------------------------------------
struct lfg_batch {
	int device = 0;
	int nthreads = 1;
	FusedGroup *fused = nullptr;     // lockstep through one joint solver (lfg_batch_create_fused)
	int fused_precision = 0;
	std::vector<lfg_sim *> sims;
	std::vector<int> n, precision;
	std::map<int, int> tuned_leaf;   // size class -> leaf size
	WorkerPool *pool = nullptr;
};

extern "C" {

int64_t lfg_footprint_estimate(int n, int precision)
{
	// front arena of the geometric nested dissection at phi ~ 0.5-0.58,
	// measured 1.6 GB (FP64) at N = 4096 and growing as N^1.55, with 25%
	// margin, plus ~30 kB per particle of pair records, scratch and vectors
	if (n <= 0) return 0;
	double fp64 = 1.6e9*std::pow((double)n/4096.0, 1.55);
	double arena = precision == LFG_PREC_FP64 ? fp64 : 0.5*fp64;
	return (int64_t)(1.25*arena+3.0e4*n);
}

int lfg_batch_create(int device, int nthreads, lfg_batch **out, lfg_status *st)
{
	if (!out) return fail(st, LFG_ERR_BAD_ARG, 0, "null output");
	int rc = check_device(device, st);
	if (rc) return rc;
	try {
		lfg_batch *b = new lfg_batch();
		b->device = device;
		b->nthreads = nthreads > 0 ? nthreads
		                           : std::max(1, std::min(16, (int)std::thread::hardware_concurrency()));
		b->pool = new WorkerPool(b->nthreads);
		*out = b;
		return ok(st);
	} catch (...) {
		return fail(st, LFG_ERR_OOM, 0, "host allocation failed");
	}
}

int lfg_batch_create_fused(int device, int precision, lfg_batch **out, lfg_status *st)
{
	if (!out) return fail(st, LFG_ERR_BAD_ARG, 0, "null output");
	if (precision != LFG_PREC_FP64 && precision != LFG_PREC_FP32_REFINE)
		return fail(st, LFG_ERR_BAD_ARG, precision, "unknown precision");
	int rc = check_device(device, st);
	if (rc) return rc;
	lfg_batch *b = nullptr;
	try {
		b = new lfg_batch();
		b->device = device;
		b->fused_precision = precision;
		b->fused = fused_create(device, precision);
		*out = b;
		return ok(st);
	} catch (const Error &e) {
		delete b;
		return fail(st, e.code, e.info, e.msg.c_str());
	} catch (...) {
		delete b;
		return fail(st, LFG_ERR_OOM, 0, "allocation failed");
	}
}

int lfg_batch_add(lfg_batch *b, const lfg_params *p, const lfg_options *opt, int n, const double *pos,
                  const double *radius, double lx, double ly, double lz, const double *le_disp, int *slot,
                  lfg_status *st)
{
	if (!b) return fail(st, LFG_ERR_BAD_ARG, 0, "null batch");
	lfg_options o;
	if (opt) o = *opt; else lfg_default_options(&o);
	o.device = b->device;
	if (b->fused) o.precision = b->fused_precision;
	auto it = b->tuned_leaf.find(size_class(n, o.precision));
	if (it != b->tuned_leaf.end()) o.leaf_size = it->second;
	lfg_sim *s = nullptr;
	int rc = b->fused ? fused_add(b->fused, p, &o, n, pos, radius, lx, ly, lz, le_disp, &s, st)
	                  : lfg_sim_create(p, &o, n, pos, radius, lx, ly, lz, le_disp, 0, nullptr, nullptr, nullptr, &s, st);
	if (rc) return rc;
	b->sims.push_back(s);
	b->n.push_back(n);
	b->precision.push_back(o.precision);
	if (slot) *slot = (int)b->sims.size()-1;
	return ok(st);
}

int lfg_batch_size(const lfg_batch *b) { return b ? (int)b->sims.size() : 0; }

lfg_sim *lfg_batch_sim(lfg_batch *b, int slot)
{
	if (!b || slot < 0 || slot >= (int)b->sims.size()) return nullptr;
	return b->sims[slot];
}

// Runs fn(slot) for every slot on the worker pool in slices: each task runs
// one slice of a slot and re-queues the slot until fn reports it is done, so
// suspensions of different sizes progress together.  First error wins.
static int batch_drive(lfg_batch *b, const std::function<int(int, bool *, lfg_status *)> &fn, lfg_status *st)
{
	std::mutex emu;
	int first_rc = LFG_OK;
	lfg_status first_st;
	std::memset(&first_st, 0, sizeof first_st);
	std::function<void(int)> task = [&](int slot) {
		cudaSetDevice(b->device);
		lfg_status s;
		std::memset(&s, 0, sizeof s);
		bool done = false;
		int rc = fn(slot, &done, &s);
		if (rc) {
			std::lock_guard<std::mutex> lk(emu);
			if (first_rc == LFG_OK) { first_rc = rc; first_st = s; first_st.info = slot; }
			return;
		}
		if (!done) b->pool->submit([&task, slot] { task(slot); });
	};
	for (int i = 0; i < (int)b->sims.size(); i++) b->pool->submit([&task, i] { task(i); });
	b->pool->wait();
	if (first_rc) {
		if (st) *st = first_st;
		return first_rc;
	}
	return ok(st);
}

// the fused group's calls, errors as status codes
static int fused_call(lfg_batch *b, const std::function<void()> &f, lfg_status *st)
{
	try {
		cudaSetDevice(b->device);
		f();
		return ok(st);
	} catch (const Error &e) {
		return fail(st, e.code, e.info, e.msg.c_str());
	} catch (const std::bad_alloc &) {
		return fail(st, LFG_ERR_OOM, 0, "host allocation failed");
	}
}

int lfg_batch_run(lfg_batch *b, int nsteps, lfg_status *st)
{
	if (!b || nsteps < 0) return fail(st, LFG_ERR_BAD_ARG, 0, "bad arguments");
	if (b->fused) return fused_call(b, [&] { fused_run(b->fused, nsteps); }, st);
	std::vector<int> left(b->sims.size(), nsteps);
	const int slice = 2;
	return batch_drive(b, [&](int slot, bool *done, lfg_status *s) {
		int k = std::min(slice, left[slot]);
		int rc = k > 0 ? lfg_sim_run(b->sims[slot], k, -1.0, 1e300, s) : LFG_OK;
		left[slot] -= k;
		*done = left[slot] <= 0;
		return rc;
	}, st);
}

int lfg_batch_advance(lfg_batch *b, const double *strain_end, lfg_status *st)
{
	if (!b || !strain_end) return fail(st, LFG_ERR_BAD_ARG, 0, "bad arguments");
	if (b->fused) return fused_call(b, [&] { fused_advance(b->fused, strain_end); }, st);
	const int slice = 2;
	return batch_drive(b, [&](int slot, bool *done, lfg_status *s) {
		int d = 0;
		int rc = lfg_sim_advance_partial(b->sims[slot], -1.0, strain_end[slot], slice, &d, s);
		*done = d != 0;
		return rc;
	}, st);
}

// For each size class present, time `steps` steps of its first suspension
// with every candidate leaf size (sequentially, nothing else running), keep
// the fastest for every suspension of that class and for later additions.
int lfg_batch_autotune(lfg_batch *b, const int *leaf_sizes, int count, int steps, lfg_status *st)
{
	if (!b || !leaf_sizes || count <= 0 || steps <= 0) return fail(st, LFG_ERR_BAD_ARG, 0, "bad arguments");
	if (b->fused) {
		// one leaf size for the joint system: time the fused step with each
		// (after a step that captures its graphs), keep the fastest
		double best = 1e300;
		int best_leaf = leaf_sizes[0];
		for (int c = 0; c < count; c++) {
			int rc = fused_call(b, [&] {
				fused_set_leaf_size(b->fused, leaf_sizes[c]);
				fused_run(b->fused, 1);
				cudaDeviceSynchronize();
				auto t0 = std::chrono::steady_clock::now();
				fused_run(b->fused, steps);
				double t = now_s(t0);
				if (t < best) { best = t; best_leaf = leaf_sizes[c]; }
			}, st);
			if (rc) return rc;
		}
		for (size_t i = 0; i < b->sims.size(); i++) b->tuned_leaf[size_class(b->n[i], b->precision[i])] = best_leaf;
		return fused_call(b, [&] { fused_set_leaf_size(b->fused, best_leaf); }, st);
	}
	std::map<int, std::vector<int>> classes;
	for (int i = 0; i < (int)b->sims.size(); i++) classes[size_class(b->n[i], b->precision[i])].push_back(i);
	for (auto &kv : classes) {
		lfg_sim *s = b->sims[kv.second[0]];
		double best = 1e300;
		int best_leaf = leaf_sizes[0];
		for (int c = 0; c < count; c++) {
			int rc = lfg_sim_set_leaf_size(s, leaf_sizes[c], st);
			if (rc) return rc;
			rc = lfg_sim_run(s, 1, -1.0, 1e300, st);   // capture the graphs of this analysis
			if (rc) return rc;
			lfg_sim_clear_step_times(s);
			rc = lfg_sim_run(s, steps, -1.0, 1e300, st);
			if (rc) return rc;
			std::vector<double> ms(steps+4);
			int64_t kern = 0;
			int got = lfg_sim_get_step_times(s, ms.data(), (int)ms.size(), &kern);
			double t = 0;
			for (int i = 0; i < got; i++) t += ms[i];
			if (got > 0 && t/got < best) { best = t/got; best_leaf = leaf_sizes[c]; }
		}
		b->tuned_leaf[kv.first] = best_leaf;
		for (int i : kv.second) {
			int rc = lfg_sim_set_leaf_size(b->sims[i], best_leaf, st);
			if (rc) return rc;
		}
	}
	return ok(st);
}

int lfg_batch_tuned_leaf(const lfg_batch *b, int n, int precision)
{
	if (!b) return 0;
	auto it = b->tuned_leaf.find(size_class(n, precision));
	return it == b->tuned_leaf.end() ? 0 : it->second;
}

int lfg_batch_get_stats(const lfg_batch *b, lfg_batch_stats *out)
{
	if (!b || !out) return LFG_ERR_BAD_ARG;
	std::memset(out, 0, sizeof *out);
	out->fused = b->fused != nullptr;
	if (b->fused) {
		fused_stats(b->fused, &out->kernels, &out->joint_analyses, &out->factor_flops, &out->last_refine_iters);
	} else {
		for (lfg_sim *s : b->sims) {
			lfg_sim_timing t;
			if (lfg_sim_get_timing(s, &t) == LFG_OK) out->factor_flops += t.factor_flops;
			double ms;
			int64_t k = 0;
			lfg_sim_get_step_times(s, &ms, 0, &k);
			out->kernels += k;
		}
	}
	return LFG_OK;
}

void lfg_batch_destroy(lfg_batch *b)
{
	if (!b) return;
	delete b->pool;
	if (b->fused) fused_destroy(b->fused);   // before its members: it refers to them
	for (lfg_sim *s : b->sims) lfg_sim_destroy(s);
	delete b;
}

} // extern "C"

// ---------------------------------------------------------------------------
// server
// ---------------------------------------------------------------------------
namespace {
struct Req {
	int64_t id;
	lfg_params p;
	lfg_options o;
	int n;
	std::vector<double> pos, radius;
	double lx, ly, lz;
	double strain_end;
	int64_t est;
	double t_submit;
};
}

struct lfg_server {
	int device = 0;
	int max_active = 1;
	int64_t budget = 0;
	std::chrono::steady_clock::time_point t0;
	std::mutex mu;
	std::condition_variable cv;
	std::deque<Req> queue;
	int active = 0;
	int64_t reserved = 0;
	int64_t submitted = 0, finished = 0;
	bool stop = false;
	std::vector<lfg_result> results;     // not yet polled
	std::map<int64_t, std::vector<double>> final_pos;
	lfg_server_stats stats{};
	std::thread dispatcher;
	std::vector<std::thread> workers;
	std::deque<Req> admitted;
	std::condition_variable wcv;
};

static void server_run_one(lfg_server *S, Req &r)
{
	lfg_result res;
	std::memset(&res, 0, sizeof res);
	res.id = r.id;
	res.n = r.n;
	res.t_submit = r.t_submit;
	res.t_admit = now_s(S->t0);
	res.footprint_est = r.est;
	lfg_status st;
	std::memset(&st, 0, sizeof st);
	lfg_sim *sim = nullptr;
	std::vector<double> pos;
	int rc = lfg_sim_create(&r.p, &r.o, r.n, r.pos.data(), r.radius.data(), r.lx, r.ly, r.lz, nullptr, 0, nullptr,
	                        nullptr, nullptr, &sim, &st);
	if (!rc) {
		int64_t actual = lfg_sim_device_bytes(sim);
		res.footprint_bytes = actual;
		{
			std::lock_guard<std::mutex> lk(S->mu);
			S->reserved += actual-r.est;   // replace the estimate by the actual size
			r.est = actual;
			S->stats.peak_reserved_bytes = std::max(S->stats.peak_reserved_bytes, S->reserved);
		}
		rc = lfg_sim_advance(sim, -1.0, r.strain_end, &st);
	}
	if (!rc) {
		lfg_sim_scalars sc;
		lfg_sim_get_scalars(sim, &sc);
		res.steps = sc.total_num_timesteps;
		res.strain = sc.strain;
		res.shear_rate = sc.shear_rate;
		res.viscosity = sc.viscosity;
		res.N1 = sc.N1;
		res.N2 = sc.N2;
		pos.resize(3*(size_t)r.n);
		lfg_sim_get_particles(sim, pos.data(), nullptr, nullptr, nullptr, nullptr);
	}
	if (sim) lfg_sim_destroy(sim);
	res.status = rc;
	if (rc) snprintf(res.msg, sizeof res.msg, "%s", st.msg);
	res.t_done = now_s(S->t0);
	{
		std::lock_guard<std::mutex> lk(S->mu);
		S->active--;
		S->reserved -= r.est;
		S->finished++;
		S->results.push_back(res);
		if (!rc) S->final_pos[r.id] = std::move(pos);
	}
	S->cv.notify_all();
}

static void server_worker(lfg_server *S)
{
	cudaSetDevice(S->device);
	for (;;) {
		Req r;
		{
			std::unique_lock<std::mutex> lk(S->mu);
			S->wcv.wait(lk, [S] { return S->stop || !S->admitted.empty(); });
			if (S->admitted.empty()) return;
			r = std::move(S->admitted.front());
			S->admitted.pop_front();
		}
		server_run_one(S, r);
	}
}

// Admission: first fit in arrival order over the queue, by estimated device
// footprint against the budget, while a slot is free.  A request that has
// waited longer than 5 s blocks later ones until it fits (no starvation).
// One request is always admitted when nothing runs, whatever its size.
static void server_dispatch(lfg_server *S)
{
	std::unique_lock<std::mutex> lk(S->mu);
	for (;;) {
		S->cv.wait(lk, [S] { return S->stop || (!S->queue.empty() && S->active < S->max_active); });
		if (S->stop) return;
		bool admitted_any = false;
		double t = now_s(S->t0);
		for (auto it = S->queue.begin(); it != S->queue.end() && S->active < S->max_active;) {
			bool fits = S->reserved+it->est <= S->budget || S->active == 0;
			if (fits) {
				S->reserved += it->est;
				S->active++;
				S->stats.admitted++;
				S->stats.peak_active = std::max(S->stats.peak_active, S->active);
				S->stats.peak_reserved_bytes = std::max(S->stats.peak_reserved_bytes, S->reserved);
				S->admitted.push_back(std::move(*it));
				it = S->queue.erase(it);
				admitted_any = true;
				S->wcv.notify_one();
				continue;
			}
			if (t-it->t_submit > 5.0) break;   // the oldest waiting request keeps its turn
			++it;
		}
		if (!admitted_any) S->cv.wait(lk);   // wait for a completion (or a new request)
	}
}

extern "C" {

int lfg_server_create(int device, int max_active, int64_t hbm_budget_bytes, lfg_server **out, lfg_status *st)
{
	if (!out || max_active <= 0 || hbm_budget_bytes <= 0) return fail(st, LFG_ERR_BAD_ARG, 0, "bad arguments");
	int rc = check_device(device, st);
	if (rc) return rc;
	try {
		lfg_server *S = new lfg_server();
		S->device = device;
		S->max_active = max_active;
		S->budget = hbm_budget_bytes;
		S->t0 = std::chrono::steady_clock::now();
		for (int i = 0; i < max_active; i++) S->workers.emplace_back(server_worker, S);
		S->dispatcher = std::thread(server_dispatch, S);
		*out = S;
		return ok(st);
	} catch (...) {
		return fail(st, LFG_ERR_OOM, 0, "host allocation failed");
	}
}

int lfg_server_submit(lfg_server *S, const lfg_request *r, lfg_status *st)
{
	if (!S || !r || !r->params || !r->pos || !r->radius || r->n <= 0)
		return fail(st, LFG_ERR_BAD_ARG, 0, "bad request");
	try {
		Req q;
		q.id = r->id;
		q.p = *r->params;
		if (r->options) q.o = *r->options; else lfg_default_options(&q.o);
		q.o.device = S->device;
		q.n = r->n;
		q.pos.assign(r->pos, r->pos+3*(size_t)r->n);
		q.radius.assign(r->radius, r->radius+(size_t)r->n);
		q.lx = r->lx; q.ly = r->ly; q.lz = r->lz;
		q.strain_end = r->strain_end;
		q.est = lfg_footprint_estimate(r->n, q.o.precision);
		{
			std::lock_guard<std::mutex> lk(S->mu);
			q.t_submit = now_s(S->t0);
			S->queue.push_back(std::move(q));
			S->submitted++;
			S->stats.submitted++;
		}
		S->cv.notify_all();
		return ok(st);
	} catch (...) {
		return fail(st, LFG_ERR_OOM, 0, "host allocation failed");
	}
}

int lfg_server_poll(lfg_server *S, lfg_result *out, int cap)
{
	if (!S || cap < 0) return 0;
	std::lock_guard<std::mutex> lk(S->mu);
	int k = std::min(cap, (int)S->results.size());
	for (int i = 0; i < k; i++) out[i] = S->results[i];
	S->results.erase(S->results.begin(), S->results.begin()+k);
	return k;
}

int lfg_server_wait(lfg_server *S, double timeout_s, lfg_status *st)
{
	if (!S) return fail(st, LFG_ERR_BAD_ARG, 0, "null server");
	std::unique_lock<std::mutex> lk(S->mu);
	bool done = S->cv.wait_for(lk, std::chrono::duration<double>(timeout_s > 0 ? timeout_s : 1e9),
	                           [S] { return S->finished == S->submitted; });
	if (!done) return fail(st, LFG_ERR_TIMEOUT, (int)(S->submitted-S->finished), "requests still running");
	return ok(st);
}

int lfg_server_final_positions(lfg_server *S, int64_t id, double *pos, int n)
{
	if (!S || !pos) return LFG_ERR_BAD_ARG;
	std::lock_guard<std::mutex> lk(S->mu);
	auto it = S->final_pos.find(id);
	if (it == S->final_pos.end() || (int)it->second.size() != 3*n) return LFG_ERR_BAD_ARG;
	std::copy(it->second.begin(), it->second.end(), pos);
	return LFG_OK;
}

int lfg_server_get_stats(lfg_server *S, lfg_server_stats *o)
{
	if (!S || !o) return LFG_ERR_BAD_ARG;
	std::lock_guard<std::mutex> lk(S->mu);
	*o = S->stats;
	o->active = S->active;
	o->queued = (int)S->queue.size();
	o->reserved_bytes = S->reserved;
	o->budget_bytes = S->budget;
	return LFG_OK;
}

void lfg_server_destroy(lfg_server *S)
{
	if (!S) return;
	{
		std::lock_guard<std::mutex> lk(S->mu);
		S->stop = true;
		S->queue.clear();
	}
	S->cv.notify_all();
	S->wcv.notify_all();
	if (S->dispatcher.joinable()) S->dispatcher.join();
	for (auto &t : S->workers) t.join();
	delete S;
}

} // extern "C"
