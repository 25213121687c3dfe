// Pools of resident PRP tests of one degree (continuous batching) and the
// autotuner of the cluster split and carry chunk.
//
// A pool keeps six registers and the multiply's scratch per slot in HBM.  Each
// slot runs the program of cyclo::check (cyclo/src/cyclo.h:252-377) as ticks
// of B squarings (B = the Gerbicz-Li block):
//
//   main      nb ticks over E padded with leading zero bits to nb * B bits
//             (x stays 1 over the padding, so every checkpoint is where the
//             reference puts it); after each, d <- d * x; before the last,
//             d(t) is saved, so the last multiply leaves d(t+1);
//   verify    kh ticks over the bits of the block sum above B (zero-padded),
//             from y = 1, then y <- y * d(t); one tick over its low B bits.
//
// Every launch of a tick is uniform over the pool's lanes (the engine's own
// squaring and multiply launches): the B exponent bits of each slot's tick are
// cut on the host into a per-tick staging row, and the per-slot register
// moves run in a small kernel before the squarings and after the multiply.
// Idle and finished slots square and multiply values nobody reads.  Ticks are
// replayed from CUDA graphs; the host uploads each launch's staging rows and
// register moves with the graph.
#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <thread>
#include <tuple>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/ctwin_gb300.h"
#include "bignum.h"
#include "prp_arith.cuh"
#include "prp_batch.h"
#include "prp_host.h"
#include "prp_kernels.cuh"
#include "prp_pool.h"
#include "prp_tables.h"

namespace ctw {

double mono_seconds()
{
	return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Gerbicz-Li block length for an exponent whose top bit is i0
// (cyclo/src/cyclo.h:272: L = 2 << (ilog2(i0) / 2), B_GL = (i0 - 1) / L + 1).
int gl_block_for(long long i0)
{
	if (i0 < 2) return 1;
	const int lg = 63 - __builtin_clzll((unsigned long long)i0);
	const long long L = 2LL << (lg / 2);
	return (int)((i0 - 1) / L + 1);
}

int default_gl_block(int ln) { return gl_block_for(((long long)20 << ln) - 1); }

static int stage_words(int B) { return (B + 31) / 32; }

size_t pool_slot_bytes(int ln, int B)
{
	const size_t D = (size_t)1 << ln;
	return (size_t)POOL_REGS * D * 4 + 3 * D * 4 + 16 +
	       2 * (size_t)POOL_TMAX * ((size_t)stage_words(B) * 4 + 2 * sizeof(PrpLaneAux));
}

size_t pool_bytes_estimate(int ln, int lg, int slots, int B)
{
	const size_t D = (size_t)1 << ln, G = (size_t)1 << lg;
	const size_t shoup = (ln - lg == 12) ? 2 * G * 3 * 256 * 2 * 4 : 0;
	return (size_t)slots * pool_slot_bytes(ln, B) + 2 * 3 * D * 4 + shoup + 4;
}

void slot_prepare(PreparedTest &t, int ln, int B, bool minus)
{
	t.E = prp_exponent(t.b, ln);
	if (minus) big_sub_inplace(t.E, big_from_u64(2));
	t.res = big_block_sum(t.E, B);
	t.B = B;
}

void slot_start(PoolSlot &s, PreparedTest &&t, uint64_t tag)
{
	const int B = t.B;
	const long long L = std::max<long long>(1, (long long)big_bitlen(t.E));
	const long long rl = (long long)big_bitlen(t.res);
	s.state = SLOT_ACTIVE;
	s.tk = 0;
	s.nb = (int)((L + B - 1) / B);
	s.P = (long long)s.nb * B;
	s.kh = (int)std::max<long long>(1, (rl - B + B - 1) / B);
	s.tag = tag;
	s.b = t.b;
	s.squarings = 0;
	s.done_seq = -1;
	s.t = std::move(t);
}

SlotTick slot_tick(PoolSlot &s, int B)
{
	SlotTick k;
	const int t = s.tk++;
	if (t < s.nb)
	{
		k.source = 0;
		k.lo = s.P - (long long)(t + 1) * B;
		if (t == 0) k.before |= AUX_INIT;
		if (t == s.nb - 1) k.before |= AUX_SAVE_D;
	}
	else if (t < s.nb + s.kh)
	{
		const int j = t - s.nb;
		k.source = 1;
		k.lo = (long long)(s.kh - j) * B;
		if (j == 0) k.before |= AUX_SAVE_X | AUX_SAVE_D1 | AUX_SET_Y;
		if (j == s.kh - 1)
		{
			k.before |= AUX_LOAD_D;
			k.after |= AUX_TAKE_PRODUCT;
		}
	}
	else
	{
		k.source = 1;
		k.lo = 0;
		k.after |= AUX_SAVE_Y;
		k.last = true;
		s.state = SLOT_FINISHED;
	}
	s.squarings += B + 1;
	return k;
}

// Bits [lo, lo + B) of v into nw words (bit 0 of word 0 = bit lo).
static void bit_slice(const Big &v, long long lo, int B, uint32_t *out, int nw)
{
	memset(out, 0, (size_t)nw * 4);
	for (int k = 0; k < B; ++k)
		if (big_bit(v, lo + k)) out[k >> 5] |= 1u << (k & 31);
}

}  // namespace ctw

using namespace ctw;

struct ctw_pool {
	int ln = 0, lg = 0, lm = 0, slots = 0, csize = 8, B = 0, nws = 0;
	uint32_t base = 2;
	size_t D = 0, M = 0, G = 1;
	int tw_smem = 0;
	cudaStream_t stream = nullptr, cap_stream = nullptr, rb_stream = nullptr;
	int32_t *d_regs = nullptr;                 // [POOL_REGS][slots][D]
	uint32_t *d_scratch = nullptr, *d_tf = nullptr, *d_ti = nullptr, *d_tfs = nullptr, *d_tis = nullptr;
	uint32_t *d_laneb = nullptr, *d_status = nullptr;
	uint32_t *d_stage[2] = { nullptr, nullptr };    // [POOL_TMAX][slots][nws] exponent bits per tick
	PrpLaneAux *d_aux[2] = { nullptr, nullptr };    // [POOL_TMAX][2][slots] moves before / after
	uint32_t *h_stage[2] = { nullptr, nullptr };    // pinned mirrors
	PrpLaneAux *h_aux[2] = { nullptr, nullptr };
	uint32_t *h_laneb = nullptr;                    // pinned [slots][4]
	int32_t *h_read = nullptr;                      // pinned [3][D]
	cudaEvent_t ev[2] = { nullptr, nullptr };
	bool ev_pending[2] = { false, false };
	long long ev_seq[2] = { -1, -1 };
	long long seq_issued = 0, seq_complete = 0;
	std::map<std::tuple<int, int, int, int>, cudaGraphExec_t> graphs;   // (buffer, ticks, lanes, primes)
	std::vector<PoolSlot> slot;
	std::vector<double> t_admit, t_submit;
	std::vector<ctw_result> results;
	PrpKernelArgs proto{};
	int active = 0;
	long long squarings = 0;
	size_t bytes = 0;
	bool direct = false;     // CTW_POOL_DIRECT=1: direct launches, each checked (diagnostics)
	int minus = 0;           // N- = b^Dn - b^{Dn/2} - 1 on the transform of degree D = 2 Dn
	int ln_test = 0;         // log2 of the tested degree (ln, or ln - 1 for N-)
	size_t Dn = 0;           // digits of the tested numbers
	int prime_mode = 0;      // 0: two NTT primes whenever the launch's lanes allow it; 3: always three
};

namespace {

#define POOL_CUDA(call)                                                                                      \
	do {                                                                                                     \
		cudaError_t e_ = (call);                                                                             \
		if (e_ != cudaSuccess) return fail(CTW_E_CUDA, "%s: %s", #call, cudaGetErrorString(e_));             \
	} while (0)

template <typename T>
cudaError_t dmalloc(T **p, size_t bytes, size_t &total)
{
	total += bytes;
	return cudaMalloc((void **)p, bytes);
}

void lane_params(uint32_t b, size_t D, uint32_t *lb)
{
	const int sh = (31 - __builtin_clz(b)) - 1;
	lb[0] = b;
	lb[1] = (uint32_t)(((uint64_t)1 << (sh + 32)) / b);
	lb[2] = (uint32_t)sh;
	lb[3] = (8.0 * (double)D * (double)b * (double)b < 4.611686018427388e18) ? 1u : 0u;
}

int pool_init(ctw_pool *p)
{
	const size_t D = p->D, S = (size_t)p->slots, nws = (size_t)p->nws;
	size_t &tot = p->bytes;
	if (cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess ||
	    cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking) != cudaSuccess ||
	    cudaStreamCreateWithFlags(&p->rb_stream, cudaStreamNonBlocking) != cudaSuccess)
		return fail(CTW_E_CUDA, "pool stream creation failed");
	const size_t stage_bytes = (size_t)POOL_TMAX * S * nws * 4, aux_bytes = (size_t)POOL_TMAX * 2 * S * sizeof(PrpLaneAux);
	if (dmalloc(&p->d_regs, POOL_REGS * S * D * 4, tot) != cudaSuccess ||
	    dmalloc(&p->d_scratch, S * 3 * D * 4, tot) != cudaSuccess || dmalloc(&p->d_laneb, S * 16, tot) != cudaSuccess ||
	    dmalloc(&p->d_status, 4, tot) != cudaSuccess || dmalloc(&p->d_stage[0], stage_bytes, tot) != cudaSuccess ||
	    dmalloc(&p->d_stage[1], stage_bytes, tot) != cudaSuccess || dmalloc(&p->d_aux[0], aux_bytes, tot) != cudaSuccess ||
	    dmalloc(&p->d_aux[1], aux_bytes, tot) != cudaSuccess)
		return fail(CTW_E_NOMEM, "pool of %d slots at degree 2^%d: device allocation failed", p->slots, p->ln);
	if (cudaMallocHost(&p->h_stage[0], stage_bytes) != cudaSuccess ||
	    cudaMallocHost(&p->h_stage[1], stage_bytes) != cudaSuccess ||
	    cudaMallocHost(&p->h_aux[0], aux_bytes) != cudaSuccess || cudaMallocHost(&p->h_aux[1], aux_bytes) != cudaSuccess ||
	    cudaMallocHost(&p->h_laneb, S * 16) != cudaSuccess || cudaMallocHost(&p->h_read, 3 * D * 4) != cudaSuccess)
		return fail(CTW_E_NOMEM, "pool pinned host allocation failed");
	// every slot holds valid numbers from the start: registers 0, b = 2^16 + 1
	for (size_t s = 0; s < S; ++s) lane_params(65537u, D, p->h_laneb + 4 * s);
	POOL_CUDA(cudaMemcpy(p->d_laneb, p->h_laneb, S * 16, cudaMemcpyHostToDevice));
	POOL_CUDA(cudaMemset(p->d_regs, 0, POOL_REGS * S * D * 4));
	POOL_CUDA(cudaMemset(p->d_scratch, 0, S * 3 * D * 4));
	POOL_CUDA(cudaMemset(p->d_status, 0, 4));
	POOL_CUDA(cudaEventCreateWithFlags(&p->ev[0], cudaEventDisableTiming));
	POOL_CUDA(cudaEventCreateWithFlags(&p->ev[1], cudaEventDisableTiming));

	const size_t words = p->G * 3 * p->M, swords = p->G * 3 * 256 * 2;
	std::vector<uint32_t> tf(words), ti(words), tfs(swords), tis(swords);
	prp_build_tables(p->ln, p->lg, tf.data(), ti.data(), p->proto, tfs.data(), tis.data());
	if (dmalloc(&p->d_tf, words * 4, tot) != cudaSuccess || dmalloc(&p->d_ti, words * 4, tot) != cudaSuccess)
		return fail(CTW_E_NOMEM, "pool root tables");
	POOL_CUDA(cudaMemcpy(p->d_tf, tf.data(), words * 4, cudaMemcpyHostToDevice));
	POOL_CUDA(cudaMemcpy(p->d_ti, ti.data(), words * 4, cudaMemcpyHostToDevice));
	if (p->lm == 12)
	{
		if (dmalloc(&p->d_tfs, swords * 4, tot) != cudaSuccess || dmalloc(&p->d_tis, swords * 4, tot) != cudaSuccess)
			return fail(CTW_E_NOMEM, "pool root tables");
		POOL_CUDA(cudaMemcpy(p->d_tfs, tfs.data(), swords * 4, cudaMemcpyHostToDevice));
		POOL_CUDA(cudaMemcpy(p->d_tis, tis.data(), swords * 4, cudaMemcpyHostToDevice));
	}
	PrpKernelArgs &a = p->proto;
	a.tf = p->d_tf;
	a.ti = p->d_ti;
	a.tfs = p->d_tfs;
	a.tis = p->d_tis;
	a.lane_b = p->d_laneb;
	a.status = p->d_status;
	a.lm = p->lm;
	a.csize = p->csize;
	a.mult = (int)p->base;
	a.tw_smem = p->tw_smem;
	a.narrow = 0;                 // per lane (lane_b[3])
	a.minus = p->minus;
	a.nprime = 3;                 // per launch (pool_primes)
	a.dense = 0;                  // two CTAs per SM when the lanes fill the GPU
	a.scratch = p->d_scratch;
	a.use_dupmask = 0;
	POOL_CUDA(cudaDeviceSynchronize());
	return CTW_OK;
}

int32_t *reg_plane(ctw_pool *p, int r) { return p->d_regs + (size_t)r * p->slots * p->D; }

// NTT primes of a launch over lanes [0, lanes): two when the split has a
// two-prime kernel and every lane's b keeps the product exact with two.
int pool_primes(const ctw_pool *p, int lanes)
{
	if (p->prime_mode == 3 || !prp_two_prime_split(p->lm, p->lg)) return 3;
	uint32_t bmax = 0;
	for (int s = 0; s < lanes; ++s) bmax = std::max(bmax, p->h_laneb[4 * (size_t)s]);
	const double terms = p->minus ? (double)p->Dn : 1.5 * (double)p->D;
	return prp_two_primes_exact(terms, bmax) ? 2 : 3;
}

// The launches of T ticks from buffer k over `lanes` lanes: per tick the
// moves before, the squarings (uniform launches of at most POOL_SQ_CHUNK),
// the multiply d <- x * d, the moves after.  check != 0 synchronises after
// each launch and names the first one that fails.
cudaError_t issue_ticks(ctw_pool *p, int k, int T, int lanes, int np, cudaStream_t cs, bool check, const char **what)
{
	const size_t S = (size_t)p->slots;
	const long long stride = (long long)S * (long long)p->D;
	cudaError_t e = cudaSuccess;
	auto step = [&](const char *name) {
		if (e == cudaSuccess && check) e = cudaStreamSynchronize(cs);
		if (e != cudaSuccess && !*what) *what = name;
	};
	for (int t = 0; t < T && e == cudaSuccess; ++t)
	{
		const PrpLaneAux *aux = p->d_aux[k] + (size_t)t * 2 * S;
		e = prp_aux_launch(aux, p->d_regs, stride, p->ln, lanes, cs);
		step("register moves");
		PrpKernelArgs a = p->proto;
		a.nprime = np;
		a.op = OP_SQUARE;
		a.reg_in = reg_plane(p, 0);
		a.reg_out = reg_plane(p, 0);
		a.bits = p->d_stage[k] + (size_t)t * S * p->nws;
		a.nwords = p->nws;
		for (int off = 0; off < p->B && e == cudaSuccess; off += POOL_SQ_CHUNK)
		{
			a.i_hi = p->B - 1 - off;
			a.count = std::min(POOL_SQ_CHUNK, p->B - off);
			e = prp_launch(a, p->lg, lanes, cs);
			step("squarings");
		}
		if (e != cudaSuccess) break;
		a.op = OP_MUL;
		a.reg_in = reg_plane(p, 0);
		a.reg_y = reg_plane(p, 1);
		a.reg_out = reg_plane(p, 1);
		a.count = 1;
		a.i_hi = 0;
		a.bits = nullptr;
		e = prp_launch(a, p->lg, lanes, cs);
		step("multiply");
		if (e != cudaSuccess) break;
		e = prp_aux_launch(aux + S, p->d_regs, stride, p->ln, lanes, cs);
		step("register moves");
	}
	return e;
}

cudaError_t upload(ctw_pool *p, int k, int T, cudaStream_t cs)
{
	const size_t S = (size_t)p->slots;
	cudaError_t e = cudaMemcpyAsync(p->d_aux[k], p->h_aux[k], (size_t)T * 2 * S * sizeof(PrpLaneAux),
	                                cudaMemcpyHostToDevice, cs);
	if (e != cudaSuccess) return e;
	return cudaMemcpyAsync(p->d_stage[k], p->h_stage[k], (size_t)T * S * p->nws * 4, cudaMemcpyHostToDevice, cs);
}

int get_graph(ctw_pool *p, int k, int T, int lanes, int np, cudaGraphExec_t &exec)
{
	const auto key = std::make_tuple(k, T, lanes, np);
	auto it = p->graphs.find(key);
	if (it != p->graphs.end())
	{
		exec = it->second;
		return CTW_OK;
	}
	cudaStream_t cs = p->cap_stream;
	POOL_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed));
	const char *what = nullptr;
	cudaError_t e = upload(p, k, T, cs);
	if (e == cudaSuccess) e = issue_ticks(p, k, T, lanes, np, cs, false, &what);
	cudaGraph_t graph = nullptr;
	const cudaError_t e2 = cudaStreamEndCapture(cs, &graph);
	if (e != cudaSuccess || e2 != cudaSuccess)
	{
		if (graph) cudaGraphDestroy(graph);
		return fail(CTW_E_CUDA, "pool tick capture: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
	}
	e = cudaGraphInstantiate(&exec, graph, 0);
	cudaGraphDestroy(graph);
	if (e != cudaSuccess) return fail(CTW_E_CUDA, "pool graph instantiate: %s", cudaGetErrorString(e));
	p->graphs[key] = exec;
	return CTW_OK;
}

// Mark launches whose event has completed; wait == true blocks on them.
int retire_events(ctw_pool *p, bool wait)
{
	for (int k = 0; k < 2; ++k)
	{
		if (!p->ev_pending[k]) continue;
		cudaError_t e = wait ? cudaEventSynchronize(p->ev[k]) : cudaEventQuery(p->ev[k]);
		if (e == cudaErrorNotReady) continue;
		if (e != cudaSuccess) return fail(CTW_E_CUDA, "pool launch failed: %s", cudaGetErrorString(e));
		p->ev_pending[k] = false;
		p->seq_complete = std::max(p->seq_complete, p->ev_seq[k] + 1);
	}
	return CTW_OK;
}

int read_status(ctw_pool *p, uint32_t &st)
{
	st = 0;
	POOL_CUDA(cudaMemcpyAsync(&p->h_read[0], p->d_status, 4, cudaMemcpyDeviceToHost, p->rb_stream));
	POOL_CUDA(cudaStreamSynchronize(p->rb_stream));
	st = (uint32_t)p->h_read[0];
	if (st)
	{
		POOL_CUDA(cudaMemsetAsync(p->d_status, 0, 4, p->rb_stream));
		POOL_CUDA(cudaStreamSynchronize(p->rb_stream));
	}
	return CTW_OK;
}

int finish_slot(ctw_pool *p, int s, bool status_bad)
{
	PoolSlot &sl = p->slot[(size_t)s];
	const size_t D = p->D;
	const int regs[3] = { 5, 4, 2 };     // verify result, d(t+1), result
	for (int i = 0; i < 3; ++i)
		POOL_CUDA(cudaMemcpyAsync(p->h_read + i * D, reg_plane(p, regs[i]) + (size_t)s * D, D * 4,
		                          cudaMemcpyDeviceToHost, p->rb_stream));
	POOL_CUDA(cudaStreamSynchronize(p->rb_stream));
	ctw_result r{};
	r.tag = sl.tag;
	r.b = sl.b;
	r.log2_degree = p->ln_test;
	r.slot = s;
	r.squarings = sl.squarings;
	r.t_submit = p->t_submit[(size_t)s];
	r.t_admit = p->t_admit[(size_t)s];
	r.t_done = mono_seconds();
	const size_t Dn = p->Dn;
	std::vector<uint32_t> cy(Dn), cd(Dn), cx(Dn);
	auto canon = [&](const int32_t *x, uint32_t *o) {
		return p->minus ? canonical_minus(x, sl.b, Dn, o) : canonical(x, sl.b, D, o);
	};
	int rc = canon(p->h_read, cy.data());
	if (!rc) rc = canon(p->h_read + D, cd.data());
	if (!rc) rc = canon(p->h_read + 2 * D, cx.data());
	if (rc || status_bad)
		r.status = (int8_t)(rc ? rc : CTW_E_COMPUTE);
	else
	{
		bool prp, zero;
		uint64_t r64;
		res64_of(cx.data(), sl.b, Dn, prp, zero, r64);
		r.is_prp = prp ? 1 : 0;
		r.res64 = r64;
		r.gl_ok = (cy == cd) ? 1 : 0;
		if (zero) r.status = (int8_t)CTW_E_COMPUTE;
		else if (!r.gl_ok) r.status = (int8_t)CTW_E_GERBICZ;
	}
	p->results.push_back(r);
	sl = PoolSlot{};
	--p->active;
	// the free slot computes on zeros with b = 2^16 + 1 (valid for every launch,
	// two primes included) until its next admission
	uint32_t *lb = p->h_laneb + 4 * (size_t)s;
	lane_params(65537u, D, lb);
	POOL_CUDA(cudaMemcpyAsync(p->d_laneb + 4 * (size_t)s, lb, 16, cudaMemcpyHostToDevice, p->stream));
	POOL_CUDA(cudaMemsetAsync(reg_plane(p, 0) + (size_t)s * D, 0, D * 4, p->stream));
	POOL_CUDA(cudaMemsetAsync(reg_plane(p, 1) + (size_t)s * D, 0, D * 4, p->stream));
	return CTW_OK;
}

}  // namespace

namespace ctw {

int pool_admit_prepared(ctw_pool *p, PreparedTest &&t, uint64_t tag, double t_submit)
{
	int s = -1;
	for (int i = 0; i < p->slots; ++i)
		if (p->slot[(size_t)i].state == SLOT_FREE) { s = i; break; }
	if (s < 0) return CTW_E_FULL;
	if (t.B != p->B) return fail(CTW_E_ARG, "prepared block %d differs from the pool's %d", t.B, p->B);
	uint32_t *lb = p->h_laneb + 4 * (size_t)s;
	lane_params(t.b, p->D, lb);
	POOL_CUDA(cudaMemcpyAsync(p->d_laneb + 4 * (size_t)s, lb, 16, cudaMemcpyHostToDevice, p->stream));
	slot_start(p->slot[(size_t)s], std::move(t), tag);
	p->t_admit[(size_t)s] = mono_seconds();
	p->t_submit[(size_t)s] = t_submit;
	++p->active;
	return s;
}

int pool_block(const ctw_pool *p) { return p->B; }
int pool_degree(const ctw_pool *p) { return p->ln_test; }
int pool_free_slots(const ctw_pool *p) { return p->slots - p->active; }
int pool_active(const ctw_pool *p) { return p->active; }
int pool_in_flight(const ctw_pool *p) { return (p->ev_pending[0] ? 1 : 0) + (p->ev_pending[1] ? 1 : 0); }
size_t pool_bytes(const ctw_pool *p) { return p->bytes; }

}  // namespace ctw

extern "C" {

size_t ctw_pool_slot_bytes(int log2_degree)
{
	if (log2_degree < 8 || log2_degree > 18) return 0;
	return pool_slot_bytes(log2_degree, default_gl_block(log2_degree));
}

static int pool_create(int log2_degree, int slots, int log2_ctas, int csize, uint32_t base, int gl_block, int minus,
                       ctw_pool **out);

int ctw_pool_create(int log2_degree, int slots, int log2_ctas, int csize, uint32_t base, int gl_block, ctw_pool **out)
{
	return pool_create(log2_degree, slots, log2_ctas, csize, base, gl_block, 0, out);
}

int ctw_pool_create_minus(int log2_degree, int slots, int csize, uint32_t base, int gl_block, ctw_pool **out)
{
	if (log2_degree < 8 || log2_degree > 16) return fail(CTW_E_ARG, "N- log2_degree %d outside [8, 16]", log2_degree);
	// the split of ctw_prp_create_minus: one CTA up to 2^12 coefficients, else >= 4 CTAs
	const int ln2 = log2_degree + 1;
	const int lg = ln2 <= 12 ? 0 : std::max(2, prp_lg_for(ln2));
	return pool_create(ln2, slots, lg, csize, base, gl_block, 1, out);
}

static int pool_create(int log2_degree, int slots, int log2_ctas, int csize, uint32_t base, int gl_block, int minus,
                       ctw_pool **out)
{
	if (!out) return fail(CTW_E_ARG, "null output pointer");
	*out = nullptr;
	if (log2_degree < 8 || log2_degree > 18) return fail(CTW_E_ARG, "log2_degree %d outside [8, 18]", log2_degree);
	if (slots < 1 || slots > MAX_INLINE_LANES) return fail(CTW_E_ARG, "slots %d outside [1, %d]", slots, MAX_INLINE_LANES);
	if (base != 2 && base != 3) return fail(CTW_E_ARG, "base %u not in {2,3}", base);
	const int lg = log2_ctas < 0 ? prp_lg_for(log2_degree) : log2_ctas;
	const int lm = log2_degree - lg;
	if (!prp_split_supported(lm, lg)) return fail(CTW_E_ARG, "no kernel for degree 2^%d on 2^%d CTAs", log2_degree, lg);
	if (csize == 0) csize = 8;
	if (csize != 8 && csize != 16 && csize != 32 && csize != 64) return fail(CTW_E_ARG, "csize %d not in {8,16,32,64}", csize);
	if ((csize * 2 > (1 << lm)) || (lg > 0 && lm <= 13 && csize > ((1 << lm) >> lg)))
		return fail(CTW_E_ARG, "csize %d too large for this split", csize);
	if (gl_block < 0 || gl_block > 1 << 16) return fail(CTW_E_ARG, "gl_block %d outside [0, 65536]", gl_block);
	if (ctw_device_count() == 0) return fail(CTW_E_CUDA, "no CUDA device");
	ctw_pool *p = new ctw_pool();
	p->ln = log2_degree;
	p->lg = lg;
	p->lm = lm;
	p->slots = slots;
	p->csize = csize;
	p->base = base;
	p->minus = minus;
	p->ln_test = minus ? log2_degree - 1 : log2_degree;
	p->B = gl_block ? gl_block : default_gl_block(p->ln_test);
	p->nws = stage_words(p->B);
	p->D = (size_t)1 << log2_degree;
	p->Dn = minus ? p->D / 2 : p->D;
	p->G = (size_t)1 << lg;
	p->M = p->D / p->G;
	p->tw_smem = prp_smem_bytes(lm, lg, 1) <= 227 * 1024 ? 1 : 0;
	const char *dv = getenv("CTW_POOL_DIRECT");
	p->direct = dv && dv[0] == '1';
	p->slot.assign((size_t)slots, PoolSlot{});
	p->t_admit.assign((size_t)slots, 0.0);
	p->t_submit.assign((size_t)slots, 0.0);
	if (int rc = pool_init(p))
	{
		ctw_pool_destroy(p);
		return rc;
	}
	*out = p;
	return CTW_OK;
}

int ctw_pool_destroy(ctw_pool *p)
{
	if (!p) return CTW_OK;
	if (p->stream) cudaStreamSynchronize(p->stream);
	for (auto &kv : p->graphs) cudaGraphExecDestroy(kv.second);
	cudaFree(p->d_regs);
	cudaFree(p->d_scratch);
	cudaFree(p->d_tf);
	cudaFree(p->d_ti);
	cudaFree(p->d_tfs);
	cudaFree(p->d_tis);
	cudaFree(p->d_laneb);
	cudaFree(p->d_status);
	for (int k = 0; k < 2; ++k)
	{
		cudaFree(p->d_stage[k]);
		cudaFree(p->d_aux[k]);
		cudaFreeHost(p->h_stage[k]);
		cudaFreeHost(p->h_aux[k]);
		if (p->ev[k]) cudaEventDestroy(p->ev[k]);
	}
	cudaFreeHost(p->h_laneb);
	cudaFreeHost(p->h_read);
	if (p->stream) cudaStreamDestroy(p->stream);
	if (p->cap_stream) cudaStreamDestroy(p->cap_stream);
	if (p->rb_stream) cudaStreamDestroy(p->rb_stream);
	delete p;
	return CTW_OK;
}

int ctw_pool_admit(ctw_pool *p, uint32_t b, uint64_t tag)
{
	if (!p) return fail(CTW_E_ARG, "null pool");
	if (b < 64 || b >= 0x80000000u) return fail(CTW_E_ARG, "b = %u outside [64, 2^31)", b);
	if (p->active >= p->slots) return CTW_E_FULL;
	PreparedTest t;
	t.b = b;
	slot_prepare(t, p->ln_test, p->B, p->minus != 0);
	return pool_admit_prepared(p, std::move(t), tag, mono_seconds());
}

int ctw_pool_admit_many(ctw_pool *p, const uint32_t *b, const uint64_t *tags, int count, int threads)
{
	if (!p || (!b && count > 0) || count < 0) return fail(CTW_E_ARG, "bad arguments");
	for (int i = 0; i < count; ++i)
		if (b[i] < 64 || b[i] >= 0x80000000u) return fail(CTW_E_ARG, "b = %u outside [64, 2^31)", b[i]);
	const int n = std::min(count, pool_free_slots(p));
	std::vector<PreparedTest> prep((size_t)n);
	const int nt = std::max(1, std::min(threads > 0 ? threads : (int)std::thread::hardware_concurrency(), n));
	std::vector<std::thread> th;
	for (int t = 0; t < nt; ++t)
		th.emplace_back([&, t] {
			for (int i = t; i < n; i += nt)
			{
				prep[(size_t)i].b = b[i];
				slot_prepare(prep[(size_t)i], p->ln_test, p->B, p->minus != 0);
			}
		});
	for (auto &x : th) x.join();
	const double now = mono_seconds();
	for (int i = 0; i < n; ++i)
	{
		const int s = pool_admit_prepared(p, std::move(prep[(size_t)i]), tags ? tags[i] : (uint64_t)i, now);
		if (s < 0) return s;
	}
	return n;
}

// The host half of T ticks from buffer k = seq_issued & 1 (after that
// buffer's previous launch has completed): the register moves and exponent
// slices of every active slot, and the launch width and prime count.
static int plan_ticks(ctw_pool *p, int T, int &k, int &lanes, int &np)
{
	const size_t S = (size_t)p->slots;
	k = (int)(p->seq_issued & 1);
	if (p->ev_pending[k])
	{
		POOL_CUDA(cudaEventSynchronize(p->ev[k]));
		p->ev_pending[k] = false;
		p->seq_complete = std::max(p->seq_complete, p->ev_seq[k] + 1);
	}
	int hi = 0;
	for (int s = 0; s < p->slots; ++s)
		if (p->slot[(size_t)s].state != SLOT_FREE) hi = s + 1;
	// launch over the lowest slots only, in steps of 8 lanes (one graph per
	// step); from degree 2^15 up a lane fills SMs by itself: steps of one
	const int step = p->ln >= 15 ? 1 : 8;
	lanes = std::min(p->slots, std::max(step, (hi + step - 1) / step * step));
	np = pool_primes(p, lanes);
	memset(p->h_aux[k], 0, (size_t)T * 2 * S * sizeof(PrpLaneAux));
	memset(p->h_stage[k], 0, (size_t)T * S * p->nws * 4);
	for (int t = 0; t < T; ++t)
		for (int s = 0; s < hi; ++s)
		{
			PoolSlot &sl = p->slot[(size_t)s];
			if (sl.state != SLOT_ACTIVE) continue;
			const SlotTick tk = slot_tick(sl, p->B);
			PrpLaneAux *ax = p->h_aux[k] + (size_t)t * 2 * S;
			ax[s] = PrpLaneAux{ tk.before, 1u };
			ax[S + s] = PrpLaneAux{ tk.after, 1u };
			bit_slice(tk.source ? sl.t.res : sl.t.E, tk.lo, p->B,
			          p->h_stage[k] + ((size_t)t * S + s) * p->nws, p->nws);
			p->squarings += p->B + 1;
			if (tk.last) sl.done_seq = p->seq_issued;
		}
	return CTW_OK;
}

int ctw_pool_run(ctw_pool *p, int ticks)
{
	if (!p) return fail(CTW_E_ARG, "null pool");
	if (ticks < 0) return fail(CTW_E_ARG, "negative tick count");
	while (ticks > 0)
	{
		const int T = std::min(ticks, POOL_TMAX);
		int k = 0, lanes = 0, np = 3;
		if (int rc = plan_ticks(p, T, k, lanes, np)) return rc;
		if (p->direct)
		{
			const char *what = nullptr;
			cudaError_t e = upload(p, k, T, p->stream);
			if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
			if (e != cudaSuccess) return fail(CTW_E_CUDA, "pool upload: %s", cudaGetErrorString(e));
			e = issue_ticks(p, k, T, lanes, np, p->stream, true, &what);
			if (e != cudaSuccess) return fail(CTW_E_CUDA, "pool %s launch: %s", what ? what : "?", cudaGetErrorString(e));
		}
		else
		{
			cudaGraphExec_t exec = nullptr;
			if (int rc = get_graph(p, k, T, lanes, np, exec)) return rc;
			POOL_CUDA(cudaGraphLaunch(exec, p->stream));
		}
		POOL_CUDA(cudaEventRecord(p->ev[k], p->stream));
		p->ev_pending[k] = true;
		p->ev_seq[k] = p->seq_issued;
		++p->seq_issued;
		ticks -= T;
	}
	return CTW_OK;
}

int ctw_pool_collect(ctw_pool *p, int wait)
{
	if (!p) return fail(CTW_E_ARG, "null pool");
	if (int rc = retire_events(p, wait != 0)) return rc;
	bool any = false;
	for (const PoolSlot &sl : p->slot)
		if (sl.state == SLOT_FINISHED && sl.done_seq >= 0 && sl.done_seq < p->seq_complete) { any = true; break; }
	if (any)
	{
		uint32_t st = 0;
		if (int rc = read_status(p, st)) return rc;
		for (int s = 0; s < p->slots; ++s)
		{
			const PoolSlot &sl = p->slot[(size_t)s];
			if (sl.state == SLOT_FINISHED && sl.done_seq >= 0 && sl.done_seq < p->seq_complete)
				if (int rc = finish_slot(p, s, st != 0)) return rc;
		}
	}
	return (int)p->results.size();
}

int ctw_pool_results(ctw_pool *p, ctw_result *out, int max)
{
	if (!p || (!out && max > 0)) return fail(CTW_E_ARG, "bad arguments");
	const int n = std::min(max, (int)p->results.size());
	for (int i = 0; i < n; ++i) out[i] = p->results[(size_t)i];
	p->results.erase(p->results.begin(), p->results.begin() + n);
	return n;
}

int ctw_pool_info(ctw_pool *p, int *slots, int *active, int *in_flight, int *gl_block, int *log2_ctas, int *csize,
                  long long *squarings)
{
	if (!p) return fail(CTW_E_ARG, "null pool");
	if (slots) *slots = p->slots;
	if (active) *active = p->active;
	if (in_flight) *in_flight = pool_in_flight(p);
	if (gl_block) *gl_block = p->B;
	if (log2_ctas) *log2_ctas = p->lg;
	if (csize) *csize = p->csize;
	if (squarings) *squarings = p->squarings;
	return CTW_OK;
}

int ctw_pool_set_prime_count(ctw_pool *p, int count)
{
	if (!p) return fail(CTW_E_ARG, "null pool");
	if (count != 0 && count != 3) return fail(CTW_E_ARG, "prime count %d not in {0 (automatic), 3}", count);
	p->prime_mode = count;
	return CTW_OK;
}

int ctw_pool_prime_count(ctw_pool *p)
{
	if (!p) return 0;
	int hi = 0;
	for (int s = 0; s < p->slots; ++s)
		if (p->slot[(size_t)s].state != SLOT_FREE) hi = s + 1;
	return pool_primes(p, std::min(p->slots, std::max(8, (hi + 7) / 8 * 8)));
}

int ctw_pool_read_slot(ctw_pool *p, int slot, int reg, int32_t *out)
{
	if (!p || !out || slot < 0 || slot >= p->slots || reg < 0 || reg >= POOL_REGS)
		return fail(CTW_E_ARG, "bad arguments");
	POOL_CUDA(cudaStreamSynchronize(p->stream));
	POOL_CUDA(cudaMemcpy(out, reg_plane(p, reg) + (size_t)slot * p->D, p->D * 4, cudaMemcpyDeviceToHost));
	return CTW_OK;
}

void *ctw_pool_stream(ctw_pool *p) { return p ? (void *)p->stream : nullptr; }

int ctw_pool_schedule(int log2_degree, uint32_t b, int gl_block, int32_t *ticks_out, int max_ticks, int *block)
{
	if (log2_degree < 8 || log2_degree > 18) return fail(CTW_E_ARG, "log2_degree %d outside [8, 18]", log2_degree);
	if (b < 64 || b >= 0x80000000u) return fail(CTW_E_ARG, "b = %u outside [64, 2^31)", b);
	const int B = gl_block ? gl_block : default_gl_block(log2_degree);
	if (block) *block = B;
	PreparedTest t;
	t.b = b;
	slot_prepare(t, log2_degree, B);
	PoolSlot s;
	slot_start(s, std::move(t), 0);
	int n = 0;
	for (bool done = false; !done; ++n)
	{
		const SlotTick k = slot_tick(s, B);
		done = k.last;
		if (ticks_out && n < max_ticks)
		{
			int32_t *o = ticks_out + 4 * (size_t)n;
			o[0] = (int32_t)k.before;
			o[1] = (int32_t)k.after;
			o[2] = k.source;
			o[3] = (int32_t)k.lo;
		}
	}
	return n;
}

// ---------------------------------------------------------------------------
// Autotuner: time every supported (split, csize) of a degree for `lanes`
// resident candidates and keep the fastest (per process).
// ---------------------------------------------------------------------------
int ctw_prp_autotune(int log2_degree, int lanes, int *log2_ctas, int *csize, double *us_per_squaring)
{
	return ctw_prp_autotune_primes(log2_degree, lanes, 2, log2_ctas, csize, us_per_squaring);
}

int ctw_prp_autotune_primes(int log2_degree, int lanes, int primes, int *log2_ctas, int *csize,
                            double *us_per_squaring)
{
	static std::mutex mu;
	static std::map<std::tuple<int, int, int>, std::tuple<int, int, double>> cache;
	if (log2_degree < 8 || log2_degree > 18) return fail(CTW_E_ARG, "log2_degree %d outside [8, 18]", log2_degree);
	if (lanes < 1) return fail(CTW_E_ARG, "lanes must be >= 1");
	if (primes != 2 && primes != 3) return fail(CTW_E_ARG, "primes %d not in {2, 3}", primes);
	const int tl = std::min(lanes, 512);
	std::lock_guard<std::mutex> lk(mu);
	auto it = cache.find({ log2_degree, tl, primes });
	if (it == cache.end())
	{
		int best_lg = prp_lg_for(log2_degree), best_cs = 8;
		double best = 1e300;
		// b < 2^20 keeps every degree <= 2^16 within the two-prime bound; primes = 3
		// holds the engine to three
		std::vector<uint32_t> bv((size_t)tl);
		for (int l = 0; l < tl; ++l) bv[(size_t)l] = (1u << 16) + 1009u * (uint32_t)l;
		const int nw = 4;
		std::vector<uint32_t> ew((size_t)tl * nw);
		for (size_t i = 0; i < ew.size(); ++i) ew[i] = 0x9E3779B9u * (uint32_t)(i + 1);
		for (int lg = 0; lg <= MAX_LG; ++lg)
		{
			const int lm = log2_degree - lg;
			if (!prp_split_supported(lm, lg)) continue;
			ctw_prp *h = nullptr;
			if (ctw_prp_create_split(log2_degree, tl, lg, &h) != CTW_OK) continue;
			for (int cs = 8; cs <= 64; cs *= 2)
			{
				if (ctw_prp_set_csize(h, cs) != CTW_OK) continue;
				if (ctw_prp_set_prime_count(h, primes == 3 ? 3 : 0) != CTW_OK) break;
				if (ctw_prp_set_b(h, bv.data(), tl) != CTW_OK || ctw_prp_set(h, 3) != CTW_OK) break;
				const int count = 8;
				cudaStream_t st = (cudaStream_t)ctw_prp_stream(h);
				if (ctw_prp_load_exponent(h, ew.data(), nw) != CTW_OK) break;
				if (ctw_prp_square_resident(h, 127, count) != CTW_OK) break;
				cudaEvent_t e0, e1;
				cudaEventCreate(&e0);
				cudaEventCreate(&e1);
				cudaEventRecord(e0, st);
				bool ok = true;
				for (int r = 0; r < 3 && ok; ++r) ok = ctw_prp_square_resident(h, 127, count) == CTW_OK;
				cudaEventRecord(e1, st);
				cudaEventSynchronize(e1);
				float ms = 0;
				cudaEventElapsedTime(&ms, e0, e1);
				cudaEventDestroy(e0);
				cudaEventDestroy(e1);
				if (!ok || ctw_prp_sync(h) != CTW_OK) continue;
				const double us = ms * 1e3 / (3.0 * count * tl);
				if (us < best) { best = us; best_lg = lg; best_cs = cs; }
			}
			ctw_prp_destroy(h);
		}
		if (best >= 1e300) return fail(CTW_E_CUDA, "autotune: no configuration ran");
		it = cache.emplace(std::make_tuple(log2_degree, tl, primes), std::make_tuple(best_lg, best_cs, best)).first;
	}
	if (log2_ctas) *log2_ctas = std::get<0>(it->second);
	if (csize) *csize = std::get<1>(it->second);
	if (us_per_squaring) *us_per_squaring = std::get<2>(it->second);
	return CTW_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batches: the ticks of several pools (degrees 2^12..2^15, 4096 coefficients
// per CTA) with every pool's squarings in one persistent launch (and every
// pool's Gerbicz-Li multiply in a second), per prime count, from one graph.
// ---------------------------------------------------------------------------

struct ctw_batch {
	std::vector<ctw_pool *> pools;             // largest degree first
	cudaStream_t stream = nullptr, cap_stream = nullptr;
	PrpBatchClass *d_cls[2] = { nullptr, nullptr }, *h_cls[2] = { nullptr, nullptr };
	unsigned *d_heads[2] = { nullptr, nullptr };
	size_t cap = 0;                            // entries per buffer: POOL_TMAX * 2 ops * pools
	cudaEvent_t ev[2] = { nullptr, nullptr };
	bool ev_pending[2] = { false, false };
	long long seq = 0;
	std::map<std::vector<int>, cudaGraphExec_t> graphs;
	long long launches = 0;
	int occ = 2;                               // CTAs per SM of the batch kernel build
};

namespace {

// Entries of a buffer's class array: per (tick t, op, prime count) the pools of
// that prime count in order (one persistent launch each).
struct BatchPlan {
	int T = 0;
	std::vector<int> k, lanes, np;
	struct Launch { int np, first, ncls, items; };
	std::vector<Launch> launches;              // [t][op][prime count index]
};

void batch_fill(ctw_batch *bt, int kb, BatchPlan &pl)
{
	const int P = (int)bt->pools.size();
	PrpBatchClass *h = bt->h_cls[kb];
	pl.launches.clear();
	int e = 0;
	for (int t = 0; t < pl.T; ++t)
		for (int op = 0; op < 2; ++op)
			for (int npi = 0; npi < 2; ++npi)
			{
				const int npv = npi == 0 ? 2 : 3;
				BatchPlan::Launch L{ npv, e, 0, 0 };
				for (int q = 0; q < P; ++q)
				{
					if (pl.np[(size_t)q] != npv) continue;
					ctw_pool *p = bt->pools[(size_t)q];
					const int k = pl.k[(size_t)q];
					PrpBatchClass &c = h[e++];
					memset(&c, 0, sizeof(c));
					PrpKernelArgs a = p->proto;
					a.nprime = npv;
					a.tw_smem = 0;                       // root tables through L1/L2
					if (op == 0)
					{
						a.op = OP_SQUARE;
						a.reg_in = reg_plane(p, 0);
						a.reg_out = reg_plane(p, 0);
						a.bits = p->d_stage[k] + (size_t)t * p->slots * p->nws;
						a.nwords = p->nws;
						a.i_hi = p->B - 1;
						a.count = p->B;
					}
					else
					{
						a.op = OP_MUL;
						a.reg_in = reg_plane(p, 0);
						a.reg_y = reg_plane(p, 1);
						a.reg_out = reg_plane(p, 1);
						a.count = 1;
						a.i_hi = 0;
						a.bits = nullptr;
					}
					c.a = a;
					c.lg = p->lg;
					c.items = pl.lanes[(size_t)q] / (8 >> p->lg);
					++L.ncls;
					L.items += c.items;
				}
				pl.launches.push_back(L);
			}
}

cudaError_t batch_issue(ctw_batch *bt, int kb, const BatchPlan &pl, cudaStream_t cs)
{
	const int P = (int)bt->pools.size();
	cudaError_t e = cudaMemsetAsync(bt->d_heads[kb], 0, bt->cap * sizeof(unsigned), cs);
	for (int q = 0; q < P && e == cudaSuccess; ++q) e = upload(bt->pools[(size_t)q], pl.k[(size_t)q], pl.T, cs);
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(bt->d_cls[kb], bt->h_cls[kb], bt->cap * sizeof(PrpBatchClass), cudaMemcpyHostToDevice, cs);
	for (int t = 0; t < pl.T && e == cudaSuccess; ++t)
	{
		for (int q = 0; q < P && e == cudaSuccess; ++q)
		{
			ctw_pool *p = bt->pools[(size_t)q];
			const PrpLaneAux *aux = p->d_aux[pl.k[(size_t)q]] + (size_t)t * 2 * p->slots;
			e = prp_aux_launch(aux, p->d_regs, (long long)p->slots * (long long)p->D, p->ln, pl.lanes[(size_t)q], cs);
		}
		for (int op = 0; op < 2 && e == cudaSuccess; ++op)
			for (int npi = 0; npi < 2 && e == cudaSuccess; ++npi)
			{
				const BatchPlan::Launch &L = pl.launches[(size_t)((t * 2 + op) * 2 + npi)];
				e = prp_batch_launch(L.np, bt->occ, bt->d_cls[kb] + L.first, L.ncls, L.items, bt->d_heads[kb] + L.first,
				                     cs);
			}
		for (int q = 0; q < P && e == cudaSuccess; ++q)
		{
			ctw_pool *p = bt->pools[(size_t)q];
			const PrpLaneAux *aux = p->d_aux[pl.k[(size_t)q]] + (size_t)t * 2 * p->slots + p->slots;
			e = prp_aux_launch(aux, p->d_regs, (long long)p->slots * (long long)p->D, p->ln, pl.lanes[(size_t)q], cs);
		}
	}
	return e;
}

}  // namespace

extern "C" {

int ctw_batch_create(ctw_pool *const *pools, int count, ctw_batch **out)
{
	if (!out) return fail(CTW_E_ARG, "null output pointer");
	*out = nullptr;
	if (!pools || count < 1 || count > 64) return fail(CTW_E_ARG, "count %d outside [1, 64]", count);
	std::vector<ctw_pool *> v(pools, pools + count);
	for (ctw_pool *p : v)
	{
		if (!p) return fail(CTW_E_ARG, "null pool");
		if (p->minus || p->lm != 12 || p->lg > 3)
			return fail(CTW_E_ARG, "batch pools need degrees 2^12..2^15 on CTAs of 4096 coefficients (N+)");
		if (p->slots % (8 >> p->lg) != 0)
			return fail(CTW_E_ARG, "a pool of degree 2^%d in a batch needs a multiple of %d slots", p->ln, 8 >> p->lg);
	}
	for (size_t i = 0; i < v.size(); ++i)
		for (size_t j = i + 1; j < v.size(); ++j)
			if (v[i] == v[j]) return fail(CTW_E_ARG, "a pool appears twice in the batch");
	std::stable_sort(v.begin(), v.end(), [](const ctw_pool *a, const ctw_pool *b) { return a->lg > b->lg; });
	ctw_batch *bt = new ctw_batch();
	bt->pools = v;
	bt->cap = (size_t)POOL_TMAX * 2 * v.size();
	bool ok = cudaStreamCreateWithFlags(&bt->stream, cudaStreamNonBlocking) == cudaSuccess &&
	          cudaStreamCreateWithFlags(&bt->cap_stream, cudaStreamNonBlocking) == cudaSuccess &&
	          cudaEventCreateWithFlags(&bt->ev[0], cudaEventDisableTiming) == cudaSuccess &&
	          cudaEventCreateWithFlags(&bt->ev[1], cudaEventDisableTiming) == cudaSuccess;
	for (int k = 0; k < 2 && ok; ++k)
		ok = cudaMalloc(&bt->d_cls[k], bt->cap * sizeof(PrpBatchClass)) == cudaSuccess &&
		     cudaMallocHost(&bt->h_cls[k], bt->cap * sizeof(PrpBatchClass)) == cudaSuccess &&
		     cudaMalloc(&bt->d_heads[k], bt->cap * sizeof(unsigned)) == cudaSuccess;
	if (!ok)
	{
		ctw_batch_destroy(bt);
		return fail(CTW_E_NOMEM, "batch buffers");
	}
	*out = bt;
	return CTW_OK;
}

int ctw_batch_destroy(ctw_batch *bt)
{
	if (!bt) return CTW_OK;
	if (bt->stream) cudaStreamSynchronize(bt->stream);
	for (auto &kv : bt->graphs) cudaGraphExecDestroy(kv.second);
	for (int k = 0; k < 2; ++k)
	{
		cudaFree(bt->d_cls[k]);
		cudaFreeHost(bt->h_cls[k]);
		cudaFree(bt->d_heads[k]);
		if (bt->ev[k]) cudaEventDestroy(bt->ev[k]);
	}
	if (bt->stream) cudaStreamDestroy(bt->stream);
	if (bt->cap_stream) cudaStreamDestroy(bt->cap_stream);
	delete bt;
	return CTW_OK;
}

int ctw_batch_run(ctw_batch *bt, int ticks)
{
	if (!bt) return fail(CTW_E_ARG, "null batch");
	if (ticks < 0) return fail(CTW_E_ARG, "negative tick count");
	const int P = (int)bt->pools.size();
	while (ticks > 0)
	{
		BatchPlan pl;
		pl.T = std::min(ticks, POOL_TMAX);
		const int kb = (int)(bt->seq & 1);
		if (bt->ev_pending[kb])
		{
			POOL_CUDA(cudaEventSynchronize(bt->ev[kb]));
			bt->ev_pending[kb] = false;
		}
		pl.k.resize((size_t)P);
		pl.lanes.resize((size_t)P);
		pl.np.resize((size_t)P);
		for (int q = 0; q < P; ++q)
		{
			int k = 0, lanes = 0, np = 3;
			if (int rc = plan_ticks(bt->pools[(size_t)q], pl.T, k, lanes, np)) return rc;
			pl.k[(size_t)q] = k;
			pl.lanes[(size_t)q] = lanes;
			pl.np[(size_t)q] = np;
		}
		batch_fill(bt, kb, pl);
		std::vector<int> key{ kb, pl.T, bt->occ };
		for (int q = 0; q < P; ++q)
		{
			key.push_back(pl.k[(size_t)q]);
			key.push_back(pl.lanes[(size_t)q]);
			key.push_back(pl.np[(size_t)q]);
		}
		cudaGraphExec_t exec = nullptr;
		auto it = bt->graphs.find(key);
		if (it != bt->graphs.end()) exec = it->second;
		else
		{
			POOL_CUDA(cudaStreamBeginCapture(bt->cap_stream, cudaStreamCaptureModeRelaxed));
			cudaError_t e = batch_issue(bt, kb, pl, bt->cap_stream);
			cudaGraph_t graph = nullptr;
			const cudaError_t e2 = cudaStreamEndCapture(bt->cap_stream, &graph);
			if (e != cudaSuccess || e2 != cudaSuccess)
			{
				if (graph) cudaGraphDestroy(graph);
				return fail(CTW_E_CUDA, "batch tick capture: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
			}
			e = cudaGraphInstantiate(&exec, graph, 0);
			cudaGraphDestroy(graph);
			if (e != cudaSuccess) return fail(CTW_E_CUDA, "batch graph instantiate: %s", cudaGetErrorString(e));
			bt->graphs[key] = exec;
		}
		POOL_CUDA(cudaGraphLaunch(exec, bt->stream));
		for (const BatchPlan::Launch &L : pl.launches) bt->launches += L.items > 0 ? 1 : 0;
		POOL_CUDA(cudaEventRecord(bt->ev[kb], bt->stream));
		bt->ev_pending[kb] = true;
		++bt->seq;
		for (int q = 0; q < P; ++q)
		{
			ctw_pool *p = bt->pools[(size_t)q];
			const int k = pl.k[(size_t)q];
			POOL_CUDA(cudaEventRecord(p->ev[k], bt->stream));
			p->ev_pending[k] = true;
			p->ev_seq[k] = p->seq_issued;
			++p->seq_issued;
		}
		ticks -= pl.T;
	}
	return CTW_OK;
}

void *ctw_batch_stream(ctw_batch *bt) { return bt ? (void *)bt->stream : nullptr; }

int ctw_batch_set_ctas_per_sm(ctw_batch *bt, int ctas)
{
	if (!bt) return fail(CTW_E_ARG, "null batch");
	if (ctas != 1 && ctas != 2) return fail(CTW_E_ARG, "CTAs per SM must be 1 or 2");
	if (prp_batch_max_clusters(2, ctas) < 1) return fail(CTW_E_CUDA, "the batch kernel does not fit the device");
	bt->occ = ctas;
	return CTW_OK;
}

long long ctw_batch_launches(ctw_batch *bt) { return bt ? bt->launches : 0; }

}  // extern "C"
