// Request loop over pools of every degree: continuous batching by size class
// with admission by device-memory footprint.
//
// Threads: the caller submits requests; a preparation thread computes each
// request's exponent and Gerbicz-Li block sum on the host; the worker thread
// owns the CUDA work.  Each worker iteration admits prepared requests into
// free slots of the pool of their class (allocating a new pool only while
// the pools' bytes stay within the budget, and releasing idle pools when a
// request is blocked by the budget), keeps at most two graph launches queued
// per pool, and retires finished tests.  Pools run on their own streams, so
// ticks of different degrees overlap on the device.  A class is a degree and,
// where the degree has a two-prime kernel, whether b lies within the two-prime
// bound: tests above it get pools of their own, so that they never hold the
// others' launches at three primes.
//
// Grid lanes: a test of degree >= grid_min (2^16 by default) runs instead on a
// one-lane engine, i.e. on the cooperative grid kernel that spreads one test
// over 64-128 SMs, each lane a thread of its own running one test at a time
// (one lane by default, up to GRID_LANES).  A cooperative grid needs all of
// its CTAs resident at once, so the lanes and the pools take turns on the
// device: the worker hands the device to the waiting lanes whose CTAs fit on
// the SMs together (two tests of 64 CTAs, one of 128); at every Gerbicz-Li
// checkpoint a lane hands it back; once all have, the worker keeps busy pools
// running for as long as the lanes held it (an even share while both have
// work), waits for the pools' streams and hands it over again.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/ctwin_gb300.h"
#include "bignum.h"
#include "prp_host.h"
#include "prp_pool.h"
#include "prp_tables.h"

using namespace ctw;

namespace {

constexpr int GRID_LANES = 2;

struct Request {
	int ln = 0;
	uint32_t b = 0;
	uint64_t tag = 0;
	double t_submit = 0;
};

struct Prepared {
	Request r;
	PreparedTest t;
};

}  // namespace

struct ctw_server {
	size_t budget = 0;
	int max_slots = 256, tpl = 2, autotune = 0, device = 0;
	uint32_t base = 2;
	double t0 = 0;

	std::mutex mu;
	std::condition_variable cv_in, cv_ready, cv_done;
	std::deque<Request> incoming;
	std::deque<Prepared> ready;
	std::deque<ctw_result> done;
	std::deque<std::pair<int, int>> prepare_req;   // (class, slots) pools to create ahead
	bool stop = false;
	std::string error;
	long long submitted = 0, finished = 0, active = 0, pending = 0;
	size_t bytes = 0;

	std::thread prep, worker, grid[GRID_LANES];
	// grid lanes (guarded by mu): queue, per-lane turn flags and CTA counts
	int grid_min = 16, grid_lanes = 1, sms = 0, grid_next = 0;
	std::deque<Request> grid_q;
	std::condition_variable cv_grid, cv_turn;
	struct Lane {
		bool wants = false, has = false;
		int ctas = 0, running = 0;
	} lane[GRID_LANES];
	bool lanes_want() const
	{
		for (const Lane &l : lane)
			if (l.wants && !l.has) return true;
		return false;
	}
	bool lanes_have() const
	{
		for (const Lane &l : lane)
			if (l.has) return true;
		return false;
	}
	int lanes_running() const
	{
		int n = 0;
		for (const Lane &l : lane) n += l.running;
		return n;
	}
	// worker-owned
	std::map<int, std::vector<ctw_pool *>> pools;   // class -> pools
	std::map<int, std::pair<int, int>> split;      // class -> (log2 CTAs, csize)
	std::vector<Prepared> waiting;
};

namespace {

// Class key 2 ln + w: w = 1 for b above the two-prime bound of a degree that has
// a two-prime kernel.
int class_of(int ln, uint32_t b)
{
	const int lg = prp_lg_for(ln);        // the pools' default split
	const bool capable = prp_two_prime_split(ln - lg, lg);
	return 2 * ln + ((capable && !prp_two_primes_exact(1.5 * (double)((size_t)1 << ln), b)) ? 1 : 0);
}

int pool_slots_for(ctw_server *s, int ln)
{
	const size_t sb = pool_slot_bytes(ln, default_gl_block(ln));
	const size_t cap = std::max<size_t>(1, (s->budget / 4) / sb);
	return (int)std::min<size_t>((size_t)s->max_slots, cap);
}

// Split and carry chunk of a class: tuned once on first use, else the defaults.
std::pair<int, int> split_for(ctw_server *s, int cls, int slots)
{
	auto it = s->split.find(cls);
	if (it != s->split.end()) return it->second;
	const int ln = cls / 2;
	int lg = prp_lg_for(ln), cs = 8;
	if (s->autotune)
	{
		double us = 0;
		int tlg = 0, tcs = 0;
		if (ctw_prp_autotune_primes(ln, slots, (cls & 1) ? 3 : 2, &tlg, &tcs, &us) == CTW_OK) { lg = tlg; cs = tcs; }
	}
	return s->split[cls] = std::make_pair(lg, cs);
}

size_t new_pool_bytes(ctw_server *s, int cls, int slots)
{
	return pool_bytes_estimate(cls / 2, split_for(s, cls, slots).first, slots, default_gl_block(cls / 2));
}

int new_pool(ctw_server *s, int cls, int slots, ctw_pool **out)
{
	const std::pair<int, int> sp = split_for(s, cls, slots);
	return ctw_pool_create(cls / 2, slots, sp.first, sp.second, s->base, 0, out);
}

void prep_loop(ctw_server *s)
{
	for (;;)
	{
		Request r;
		{
			std::unique_lock<std::mutex> lk(s->mu);
			s->cv_in.wait(lk, [&] { return s->stop || !s->incoming.empty(); });
			if (s->stop) return;
			r = s->incoming.front();
			s->incoming.pop_front();
		}
		Prepared p;
		p.r = r;
		p.t.b = r.b;
		slot_prepare(p.t, r.ln, default_gl_block(r.ln));
		{
			std::lock_guard<std::mutex> lk(s->mu);
			s->ready.push_back(std::move(p));
		}
		s->cv_ready.notify_one();
	}
}

void set_error(ctw_server *s, const char *where)
{
	std::lock_guard<std::mutex> lk(s->mu);
	if (s->error.empty()) s->error = std::string(where) + ": " + ctw_last_error();
}

void worker_loop(ctw_server *s)
{
	cudaSetDevice(s->device);
	std::vector<ctw_result> buf(256);
	// device-time share with the grid lane: after the lane held the device for
	// a time t, busy pools get the device for at least t before the next turn
	double granted_at = -1.0, pools_until = 0.0;
	for (;;)
	{
		std::vector<std::pair<int, int>> ahead;
		{
			std::unique_lock<std::mutex> lk(s->mu);
			bool busy = !s->waiting.empty();
			for (auto &kv : s->pools)
				for (ctw_pool *p : kv.second)
					if (pool_active(p) > 0 || pool_in_flight(p) > 0) busy = true;
			if (!busy)
				s->cv_ready.wait_for(lk, std::chrono::milliseconds(2), [&] {
					return s->stop || !s->ready.empty() || !s->prepare_req.empty() || s->lanes_want();
				});
			// no pool work is issued while a grid lane holds the device
			s->cv_turn.wait(lk, [&] { return s->stop || !s->lanes_have(); });
			if (s->stop) break;
			if (granted_at >= 0)
			{
				const double now = mono_seconds();
				pools_until = now + (now - granted_at);
				granted_at = -1.0;
			}
			while (!s->ready.empty())
			{
				s->waiting.push_back(std::move(s->ready.front()));
				s->ready.pop_front();
			}
			while (!s->prepare_req.empty())
			{
				ahead.push_back(s->prepare_req.front());
				s->prepare_req.pop_front();
			}
		}
		for (auto &pr : ahead)
		{
			if (!s->pools[pr.first].empty()) continue;
			ctw_pool *p = nullptr;
			const int slots = pr.second > 0 ? std::min(pr.second, s->max_slots) : pool_slots_for(s, pr.first / 2);
			if (new_pool(s, pr.first, slots, &p) == CTW_OK)
			{
				s->pools[pr.first].push_back(p);
				std::lock_guard<std::mutex> lk(s->mu);
				s->bytes += pool_bytes(p);
			}
			else
				set_error(s, "prepare");
		}

		// admission, first come first served within each class
		long long admitted = 0;
		bool blocked_by_budget = false;
		std::vector<Prepared> still;
		std::vector<ctw_result> out;
		for (Prepared &w : s->waiting)
		{
			const int cls = class_of(w.r.ln, w.r.b);
			if (new_pool_bytes(s, cls, 1) > s->budget)
			{
				// not even a one-slot pool fits: the request fails instead of waiting forever
				ctw_result r{};
				r.tag = w.r.tag;
				r.b = w.r.b;
				r.log2_degree = w.r.ln;
				r.status = (int8_t)CTW_E_NOMEM;
				r.slot = -1;
				r.t_submit = w.r.t_submit;
				r.t_admit = r.t_done = mono_seconds();
				out.push_back(r);
				continue;
			}
			auto &vec = s->pools[cls];
			ctw_pool *target = nullptr;
			for (ctw_pool *p : vec)
				if (pool_free_slots(p) > 0) { target = p; break; }
			if (!target)
			{
				const int slots = pool_slots_for(s, w.r.ln);
				if (s->bytes + new_pool_bytes(s, cls, slots) <= s->budget)
				{
					ctw_pool *p = nullptr;
					if (new_pool(s, cls, slots, &p) == CTW_OK)
					{
						vec.push_back(p);
						std::lock_guard<std::mutex> lk(s->mu);
						s->bytes += pool_bytes(p);
						target = p;
					}
					else
						set_error(s, "pool");
				}
				else
					blocked_by_budget = true;
			}
			if (target && pool_admit_prepared(target, std::move(w.t), w.r.tag, w.r.t_submit) >= 0)
				++admitted;
			else
				still.push_back(std::move(w));
		}
		s->waiting.swap(still);
		if (blocked_by_budget)
		{
			// give back pools with nothing to do
			for (auto &kv : s->pools)
				for (auto it = kv.second.begin(); it != kv.second.end();)
				{
					ctw_pool *p = *it;
					if (pool_active(p) == 0 && pool_in_flight(p) == 0 && ctw_pool_collect(p, 0) == 0)
					{
						const size_t pb = pool_bytes(p);
						ctw_pool_destroy(p);
						it = kv.second.erase(it);
						std::lock_guard<std::mutex> lk(s->mu);
						s->bytes -= pb;
					}
					else
						++it;
				}
		}

		// keep two launches queued per busy pool; retire finished tests
		long long act = 0;
		for (auto &kv : s->pools)
			for (ctw_pool *p : kv.second)
			{
				if (pool_active(p) > 0 && pool_in_flight(p) < 2)
					if (ctw_pool_run(p, s->tpl) != CTW_OK) set_error(s, "run");
				const int n = ctw_pool_collect(p, 0);
				if (n < 0) set_error(s, "collect");
				for (int got; n > 0 && (got = ctw_pool_results(p, buf.data(), (int)buf.size())) > 0;)
					for (int i = 0; i < got; ++i) out.push_back(buf[(size_t)i]);
				act += pool_active(p);
			}
		{
			std::lock_guard<std::mutex> lk(s->mu);
			for (ctw_result &r : out)
			{
				r.t_submit -= s->t0;
				r.t_admit -= s->t0;
				r.t_done -= s->t0;
				s->done.push_back(r);
			}
			s->finished += (long long)out.size();
			s->active = act + s->lanes_running();
			s->pending = (long long)s->waiting.size() + (long long)s->ready.size() + (long long)s->incoming.size() +
			             (long long)s->grid_q.size();
		}
		if (!out.empty()) s->cv_done.notify_all();
		// grid lanes ask for the device: once the pools have had their share (or
		// have nothing to do), let the queued pool launches finish and hand the
		// device over
		bool grant;
		{
			std::lock_guard<std::mutex> lk(s->mu);
			bool pools_busy = !s->waiting.empty();
			for (auto &kv : s->pools)
				for (ctw_pool *p : kv.second)
					if (pool_active(p) > 0 || pool_in_flight(p) > 0) pools_busy = true;
			grant = s->lanes_want() && !s->lanes_have() && (!pools_busy || mono_seconds() >= pools_until);
		}
		if (grant)
		{
			for (auto &kv : s->pools)
				for (ctw_pool *p : kv.second)
					if (cudaStreamSynchronize((cudaStream_t)ctw_pool_stream(p)) != cudaSuccess) set_error(s, "sync");
			{
				// the waiting lanes whose CTAs fit on the SMs together, taken in
				// turn from the one after the lane served first last time
				std::lock_guard<std::mutex> lk(s->mu);
				int used = 0, granted = 0;
				for (int k = 0; k < GRID_LANES && granted < s->grid_lanes; ++k)
				{
					const int i = (s->grid_next + k) % GRID_LANES;
					ctw_server::Lane &l = s->lane[i];
					if (!l.wants || (granted > 0 && used + l.ctas > s->sms)) continue;
					if (granted == 0) s->grid_next = (i + 1) % GRID_LANES;
					l.has = true;
					used += l.ctas;
					++granted;
				}
			}
			granted_at = mono_seconds();
			s->cv_turn.notify_all();
			continue;
		}
		if (admitted == 0 && out.empty()) std::this_thread::sleep_for(std::chrono::microseconds(100));
	}
	for (auto &kv : s->pools)
		for (ctw_pool *p : kv.second) ctw_pool_destroy(p);
	s->pools.clear();
}

// A lane's turn: ask the worker for the device for `ctas` CTAs and wait until
// it is handed over (false when the server stops).
bool grid_take(ctw_server *s, int i, int ctas)
{
	std::unique_lock<std::mutex> lk(s->mu);
	s->lane[i].wants = true;
	s->lane[i].ctas = ctas;
	s->cv_ready.notify_all();
	s->cv_turn.wait(lk, [&] { return s->stop || s->lane[i].has; });
	s->lane[i].wants = false;
	return !s->stop;
}
void grid_give(ctw_server *s, int i)
{
	{
		std::lock_guard<std::mutex> lk(s->mu);
		s->lane[i].has = false;
	}
	s->cv_turn.notify_all();
}
struct LaneCtx {
	ctw_server *s;
	int i, ctas;
};
int grid_checkpoint(void *user, long long)
{
	LaneCtx *c = static_cast<LaneCtx *>(user);
	grid_give(c->s, c->i);
	return grid_take(c->s, c->i, c->ctas) ? 0 : 1;
}

// Squarings and multiplies of ctw_prp_run_ex for one test of b at degree 2^ln.
long long grid_squarings(uint32_t b, int ln)
{
	const Big E = prp_exponent(b, ln);
	const long long i0 = (long long)big_bitlen(E) - 1;
	const int L = 2 << ((31 - __builtin_clz((uint32_t)i0)) / 2);
	const long long B = (i0 - 1) / L + 1;
	const long long j0 = (long long)big_bitlen(big_block_sum(E, (int)B)) - 1;
	return (i0 + 1) + (i0 / B) + (j0 >= B ? j0 - B + 1 : 0) + B + 2;
}

void grid_loop(ctw_server *s, int lane)
{
	cudaSetDevice(s->device);
	std::map<int, ctw_prp *> eng;
	for (;;)
	{
		Request r;
		{
			std::unique_lock<std::mutex> lk(s->mu);
			// lanes beyond grid_lanes take no requests: with one lane the large
			// tests run first come, first served
			s->cv_grid.wait(lk, [&] { return s->stop || (lane < s->grid_lanes && !s->grid_q.empty()); });
			if (s->stop) break;
			r = s->grid_q.front();
			s->grid_q.pop_front();
		}
		ctw_result res{};
		res.tag = r.tag;
		res.b = r.b;
		res.log2_degree = r.ln;
		res.slot = -2;
		res.t_submit = r.t_submit;
		ctw_prp *&h = eng[r.ln];
		int rc = CTW_OK;
		if (!h && (rc = ctw_prp_create(r.ln, 1, &h)) == CTW_OK) rc = ctw_prp_set_base(h, s->base);
		if (rc != CTW_OK && h)
		{
			ctw_prp_destroy(h);
			h = nullptr;
		}
		bool stopped = false;
		int ctas = 0;
		if (rc == CTW_OK) rc = ctw_prp_geometry(h, &ctas, nullptr, nullptr);
		if (rc == CTW_OK)
		{
			LaneCtx ctx{ s, lane, ctas };
			if (!grid_take(s, lane, ctas)) break;
			res.t_admit = mono_seconds();
			{
				std::lock_guard<std::mutex> lk(s->mu);
				s->lane[lane].running = 1;           // counted as active from its first turn on
			}
			uint8_t prp = 0, gl = 0;
			uint64_t r64 = 0;
			rc = ctw_prp_run_ex(h, &r.b, 1, -1, grid_checkpoint, &ctx, &prp, &r64, &gl);
			stopped = rc == CTW_STOPPED;
			{
				std::lock_guard<std::mutex> lk(s->mu);
				s->lane[lane].has = false;
			}
			s->cv_turn.notify_all();
			res.is_prp = prp;
			res.res64 = r64;
			res.gl_ok = gl;
			res.squarings = grid_squarings(r.b, r.ln);
		}
		else
			res.t_admit = mono_seconds();
		if (stopped) break;
		res.t_done = mono_seconds();
		res.status = (int8_t)rc;
		if (rc == CTW_E_CUDA) set_error(s, "grid lane");
		{
			std::lock_guard<std::mutex> lk(s->mu);
			res.t_submit -= s->t0;
			res.t_admit -= s->t0;
			res.t_done -= s->t0;
			s->done.push_back(res);
			++s->finished;
			s->lane[lane].running = 0;
		}
		s->cv_done.notify_all();
	}
	for (auto &kv : eng)
		if (kv.second) ctw_prp_destroy(kv.second);
}

}  // namespace

extern "C" {

int ctw_server_create(size_t hbm_budget_bytes, int max_slots, uint32_t base, int ticks_per_launch, int autotune,
                      ctw_server **out)
{
	if (!out) return fail(CTW_E_ARG, "null output pointer");
	*out = nullptr;
	if (base != 2 && base != 3) return fail(CTW_E_ARG, "base %u not in {2,3}", base);
	if (max_slots < 1 || max_slots > 65535) return fail(CTW_E_ARG, "max_slots %d outside [1, 65535]", max_slots);
	if (ticks_per_launch < 1 || ticks_per_launch > POOL_TMAX)
		return fail(CTW_E_ARG, "ticks_per_launch %d outside [1, %d]", ticks_per_launch, POOL_TMAX);
	if (ctw_device_count() == 0) return fail(CTW_E_CUDA, "no CUDA device");
	ctw_server *s = new ctw_server();
	cudaGetDevice(&s->device);
	if (hbm_budget_bytes == 0)
	{
		size_t fr = 0, tot = 0;
		if (cudaMemGetInfo(&fr, &tot) != cudaSuccess)
		{
			delete s;
			return fail(CTW_E_CUDA, "cudaMemGetInfo failed");
		}
		hbm_budget_bytes = fr / 10 * 8;
	}
	s->budget = hbm_budget_bytes;
	s->max_slots = max_slots;
	s->base = base;
	s->tpl = ticks_per_launch;
	s->autotune = autotune;
	s->t0 = mono_seconds();
	s->prep = std::thread(prep_loop, s);
	s->worker = std::thread(worker_loop, s);
	cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->device);
	for (int i = 0; i < GRID_LANES; ++i) s->grid[i] = std::thread(grid_loop, s, i);
	*out = s;
	return CTW_OK;
}

int ctw_server_submit(ctw_server *s, int log2_degree, uint32_t b, uint64_t tag)
{
	if (!s) return fail(CTW_E_ARG, "null server");
	if (log2_degree < 8 || log2_degree > 18) return fail(CTW_E_ARG, "log2_degree %d outside [8, 18]", log2_degree);
	if (b < 64 || b >= 0x80000000u) return fail(CTW_E_ARG, "b = %u outside [64, 2^31)", b);
	{
		std::lock_guard<std::mutex> lk(s->mu);
		if (!s->error.empty()) return fail(CTW_E_CUDA, "server failed: %s", s->error.c_str());
		Request r;
		r.ln = log2_degree;
		r.b = b;
		r.tag = tag;
		r.t_submit = mono_seconds();
		++s->submitted;
		++s->pending;
		if (s->grid_min > 0 && log2_degree >= s->grid_min)
		{
			s->grid_q.push_back(r);
			s->cv_grid.notify_one();
			return CTW_OK;
		}
		s->incoming.push_back(r);
	}
	s->cv_in.notify_one();
	return CTW_OK;
}

int ctw_server_set_grid_lane(ctw_server *s, int min_log2_degree)
{
	if (!s) return fail(CTW_E_ARG, "null server");
	if (min_log2_degree != 0 && (min_log2_degree < 8 || min_log2_degree > 18))
		return fail(CTW_E_ARG, "grid lane degree %d not 0 or in [8, 18]", min_log2_degree);
	std::lock_guard<std::mutex> lk(s->mu);
	s->grid_min = min_log2_degree;
	return CTW_OK;
}

int ctw_server_set_grid_lanes(ctw_server *s, int lanes)
{
	if (!s) return fail(CTW_E_ARG, "null server");
	if (lanes < 1 || lanes > GRID_LANES) return fail(CTW_E_ARG, "grid lanes %d outside [1, %d]", lanes, GRID_LANES);
	{
		std::lock_guard<std::mutex> lk(s->mu);
		s->grid_lanes = lanes;
	}
	s->cv_grid.notify_all();
	return CTW_OK;
}

int ctw_server_prepare(ctw_server *s, int log2_degree, int slots)
{
	if (!s) return fail(CTW_E_ARG, "null server");
	if (log2_degree < 8 || log2_degree > 18) return fail(CTW_E_ARG, "log2_degree %d outside [8, 18]", log2_degree);
	{
		std::lock_guard<std::mutex> lk(s->mu);
		s->prepare_req.emplace_back(2 * log2_degree, slots);
		if (prp_two_prime_split(log2_degree - prp_lg_for(log2_degree), prp_lg_for(log2_degree)))
			s->prepare_req.emplace_back(2 * log2_degree + 1, slots);
	}
	s->cv_ready.notify_one();
	return CTW_OK;
}

int ctw_server_poll(ctw_server *s, ctw_result *out, int max, int timeout_ms)
{
	if (!s || (!out && max > 0)) return fail(CTW_E_ARG, "bad arguments");
	std::unique_lock<std::mutex> lk(s->mu);
	if (s->done.empty() && timeout_ms > 0)
		s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms),
		                    [&] { return !s->done.empty() || !s->error.empty(); });
	if (!s->error.empty() && s->done.empty()) return fail(CTW_E_CUDA, "server failed: %s", s->error.c_str());
	int n = 0;
	while (n < max && !s->done.empty())
	{
		out[n++] = s->done.front();
		s->done.pop_front();
	}
	return n;
}

int ctw_server_stats(ctw_server *s, long long *submitted, long long *pending, long long *active, long long *finished,
                     size_t *pool_bytes_out)
{
	if (!s) return fail(CTW_E_ARG, "null server");
	std::lock_guard<std::mutex> lk(s->mu);
	if (submitted) *submitted = s->submitted;
	if (pending) *pending = s->pending;
	if (active) *active = s->active;
	if (finished) *finished = s->finished;
	if (pool_bytes_out) *pool_bytes_out = s->bytes;
	return CTW_OK;
}

double ctw_server_clock(ctw_server *s) { return s ? mono_seconds() - s->t0 : 0.0; }

int ctw_server_destroy(ctw_server *s)
{
	if (!s) return CTW_OK;
	{
		std::lock_guard<std::mutex> lk(s->mu);
		s->stop = true;
	}
	s->cv_in.notify_all();
	s->cv_ready.notify_all();
	s->cv_grid.notify_all();
	s->cv_turn.notify_all();
	if (s->prep.joinable()) s->prep.join();
	if (s->worker.joinable()) s->worker.join();
	for (std::thread &t : s->grid)
		if (t.joinable()) t.join();
	delete s;
	return CTW_OK;
}

}  // extern "C"
