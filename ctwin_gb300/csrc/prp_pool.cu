// Pools of resident PRP tests of one degree (continuous batching) and the
// autotuner of the cluster split and carry chunk.
//
// A pool keeps, for each of its slots, four registers, the exponent bits, the
// Gerbicz-Li block sum and the multiply's scratch in HBM.  Each slot runs the
// program of cyclo::check (cyclo/src/cyclo.h:252-377) as a sequence of ticks:
//
//   main      B squarings of x = reg0 over bits pos .. pos-B+1 of E, then
//             d <- d * x (reg1) at every block boundary but the last, where
//             reg2 <- d * x (d(t+1)) instead;
//   verify 1  reg3 <- reg0 (the result), reg0 <- 1, squarings over the bits of
//             the block sum above B, reg0 <- reg0 * d(t);
//   verify 2  B squarings over the low B bits of the block sum.
//
// E is padded with leading zero bits to a multiple of B, so every block, and
// every Gerbicz-Li checkpoint, is where the reference puts it (x stays 1 over
// the padding).  One tick is three launches over all slots (register set-up,
// squarings, multiply) driven by per-slot commands, so slots admitted at
// different times share every launch.  Ticks are replayed from CUDA graphs.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/ctwin_gb300.h"
#include "bignum.h"
#include "prp_arith.cuh"
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

// Exponent words of one slot: E (b < 2^31, so below 2^(31 D)) padded to a
// multiple of B, then the block sum at word ewE.
void slot_words(int ln, int B, int &ewE, int &ewR)
{
	const long long D = 1LL << ln;
	ewE = (int)((31 * D + B + 31) / 32) + 1;
	ewR = (B + 64 + 31) / 32 + 1;
}

size_t pool_slot_bytes(int ln, int B)
{
	int ewE, ewR;
	slot_words(ln, B, ewE, ewR);
	const size_t D = (size_t)1 << ln;
	return 4 * D * 4 + 3 * D * 4 + (size_t)(ewE + ewR) * 4 + 16 + 2 * (size_t)POOL_TMAX * 3 * sizeof(PrpLaneCmd);
}

size_t pool_bytes_estimate(int ln, int lg, int slots, int B)
{
	const size_t D = (size_t)1 << ln, G = (size_t)1 << lg;
	const size_t shoup = (ln - lg == 12) ? 2 * G * 3 * 256 * 2 * 4 : 0;
	return (size_t)slots * pool_slot_bytes(ln, B) + 2 * 3 * D * 4 + shoup + 4;
}

void slot_prepare(PreparedTest &t, int ln, int B)
{
	t.E = prp_exponent(t.b, ln);
	t.res = big_block_sum(t.E, B);
	t.B = B;
}

void slot_start(PoolSlot &s, const PreparedTest &t, uint64_t tag)
{
	const long long L = (long long)big_bitlen(t.E);
	const long long P = ((L + t.B - 1) / t.B) * t.B;
	s.state = SLOT_MAIN;
	s.fresh = true;
	s.pos = (P > 0 ? P : t.B) - 1;
	s.j0 = (int)big_bitlen(t.res) - 1;
	s.tag = tag;
	s.b = t.b;
	s.squarings = 0;
	s.done_seq = -1;
}

// Commands of one slot for one tick; returns true when this tick finishes the test.
bool slot_tick(PoolSlot &s, int B, int r0, PrpLaneCmd &aux, PrpLaneCmd &sq, PrpLaneCmd &mul)
{
	aux = PrpLaneCmd{};
	sq = PrpLaneCmd{};
	mul = PrpLaneCmd{};
	switch (s.state)
	{
	case SLOT_MAIN:
		if (s.fresh)
		{
			aux.aux = 2 | 4;   // x = 1, d = 1
			aux.aux_arg = 1;
			s.fresh = false;
		}
		sq.count = B;
		sq.i_hi = (int32_t)s.pos;
		sq.r_in = sq.r_out = 0;
		mul.count = 1;
		mul.r_in = 0;
		mul.r_y = 1;
		if (s.pos - B + 1 > 0)
		{
			mul.r_out = 1;                 // d <- d * x at a block boundary
			s.pos -= B;
		}
		else
		{
			mul.r_out = 2;                 // d(t+1) = d(t) * x
			s.state = SLOT_VERIFY1;
		}
		s.squarings += B + 1;
		return false;
	case SLOT_VERIFY1:
		aux.aux = 1 | 2;                   // reg3 <- result, reg0 <- 1
		aux.aux_arg = 1;
		if (s.j0 >= B)
		{
			sq.count = s.j0 - B + 1;
			sq.i_hi = r0 + s.j0;
			s.squarings += sq.count;
		}
		mul.count = 1;
		mul.r_in = 0;
		mul.r_y = 1;
		mul.r_out = 0;
		s.squarings += 1;
		s.state = SLOT_VERIFY2;
		return false;
	case SLOT_VERIFY2:
		sq.count = B;
		sq.i_hi = r0 + B - 1;
		s.squarings += B;
		s.state = SLOT_FINISHED;
		return true;
	default:
		return false;
	}
}

}  // namespace ctw

using namespace ctw;

struct ctw_pool {
	int ln = 0, lg = 0, lm = 0, slots = 0, csize = 8, B = 0;
	uint32_t base = 2;
	size_t D = 0, M = 0, G = 1;
	int tw_smem = 0;
	int ewE = 0, ewR = 0, nwords = 0, r0 = 0;
	cudaStream_t stream = nullptr, cap_stream = nullptr, rb_stream = nullptr;
	int32_t *d_regs = nullptr;                 // [4][slots][D]
	uint32_t *d_scratch = nullptr, *d_tf = nullptr, *d_ti = nullptr, *d_tfs = nullptr, *d_tis = nullptr;
	uint32_t *d_laneb = nullptr, *d_exp = nullptr, *d_status = nullptr;
	PrpLaneCmd *d_cmd[2] = { nullptr, nullptr };
	PrpLaneCmd *h_cmd[2] = { nullptr, nullptr };   // pinned [POOL_TMAX][3][slots]
	uint32_t *h_stage = nullptr;                    // pinned [slots][4 + nwords]
	int32_t *h_read = nullptr;                      // pinned [3][D]
	cudaEvent_t ev[2] = { nullptr, nullptr };
	bool ev_pending[2] = { false, false };
	long long ev_seq[2] = { -1, -1 };
	long long seq_issued = 0, seq_complete = 0;
	std::map<std::tuple<int, int, int>, cudaGraphExec_t> graphs;
	std::vector<PoolSlot> slot;
	std::vector<double> t_admit, t_submit;
	std::vector<ctw_result> results;
	PrpKernelArgs proto{};
	int active = 0;
	long long squarings = 0;
	size_t bytes = 0;
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

int pool_init(ctw_pool *p)
{
	const size_t D = p->D, S = (size_t)p->slots;
	size_t &tot = p->bytes;
	if (cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess ||
	    cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking) != cudaSuccess ||
	    cudaStreamCreateWithFlags(&p->rb_stream, cudaStreamNonBlocking) != cudaSuccess)
		return fail(CTW_E_CUDA, "pool stream creation failed");
	if (dmalloc(&p->d_regs, 4 * S * D * 4, tot) != cudaSuccess || dmalloc(&p->d_scratch, S * 3 * D * 4, tot) != cudaSuccess ||
	    dmalloc(&p->d_laneb, S * 16, tot) != cudaSuccess || dmalloc(&p->d_exp, S * (size_t)p->nwords * 4, tot) != cudaSuccess ||
	    dmalloc(&p->d_status, 4, tot) != cudaSuccess ||
	    dmalloc(&p->d_cmd[0], (size_t)POOL_TMAX * 3 * S * sizeof(PrpLaneCmd), tot) != cudaSuccess ||
	    dmalloc(&p->d_cmd[1], (size_t)POOL_TMAX * 3 * S * sizeof(PrpLaneCmd), tot) != cudaSuccess)
		return fail(CTW_E_NOMEM, "pool of %d slots at degree 2^%d: device allocation failed", p->slots, p->ln);
	if (cudaMallocHost(&p->h_cmd[0], (size_t)POOL_TMAX * 3 * S * sizeof(PrpLaneCmd)) != cudaSuccess ||
	    cudaMallocHost(&p->h_cmd[1], (size_t)POOL_TMAX * 3 * S * sizeof(PrpLaneCmd)) != cudaSuccess ||
	    cudaMallocHost(&p->h_stage, S * (4 + (size_t)p->nwords) * 4) != cudaSuccess ||
	    cudaMallocHost(&p->h_read, 3 * D * 4) != cudaSuccess)
		return fail(CTW_E_NOMEM, "pool pinned host allocation failed");
	POOL_CUDA(cudaMemset(p->d_regs, 0, 4 * S * D * 4));
	POOL_CUDA(cudaMemset(p->d_laneb, 0, S * 16));
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
	a.scratch = p->d_scratch;
	a.bits = p->d_exp;
	a.nwords = p->nwords;
	a.regs = p->d_regs;
	a.reg_stride = (long long)S * (long long)D;
	a.use_dupmask = 0;
	POOL_CUDA(cudaDeviceSynchronize());
	return CTW_OK;
}

int get_graph(ctw_pool *p, int k, int T, int lanes, cudaGraphExec_t &exec)
{
	const auto key = std::make_tuple(k, T, lanes);
	auto it = p->graphs.find(key);
	if (it != p->graphs.end())
	{
		exec = it->second;
		return CTW_OK;
	}
	const size_t S = (size_t)p->slots;
	cudaStream_t cs = p->cap_stream;
	POOL_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed));
	cudaError_t e = cudaMemcpyAsync(p->d_cmd[k], p->h_cmd[k], (size_t)T * 3 * S * sizeof(PrpLaneCmd),
	                                cudaMemcpyHostToDevice, cs);
	for (int t = 0; t < T && e == cudaSuccess; ++t)
	{
		PrpLaneCmd *c = p->d_cmd[k] + (size_t)t * 3 * S;
		e = prp_aux_launch(c, p->d_regs, p->proto.reg_stride, p->ln, lanes, cs);
		if (e != cudaSuccess) break;
		PrpKernelArgs a = p->proto;
		a.op = OP_SQUARE;
		a.cmd = c + S;
		// squarings in launches of at most POOL_SQ_CHUNK, so that pools of
		// other degrees on other streams interleave with long ticks
		for (int off = 0; off < p->B && e == cudaSuccess; off += POOL_SQ_CHUNK)
		{
			a.i_hi = off;
			a.count = POOL_SQ_CHUNK;
			e = prp_launch(a, p->lg, lanes, cs);
		}
		if (e != cudaSuccess) break;
		a.op = OP_MUL;
		a.cmd = c + 2 * S;
		a.i_hi = 0;
		a.count = 1;
		e = prp_launch(a, p->lg, lanes, cs);
	}
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
	const size_t D = p->D, S = (size_t)p->slots;
	const int regs[3] = { 0, 2, 3 };
	for (int i = 0; i < 3; ++i)
		POOL_CUDA(cudaMemcpyAsync(p->h_read + i * D, p->d_regs + ((size_t)regs[i] * S + s) * D, D * 4,
		                          cudaMemcpyDeviceToHost, p->rb_stream));
	POOL_CUDA(cudaStreamSynchronize(p->rb_stream));
	ctw_result r{};
	r.tag = sl.tag;
	r.b = sl.b;
	r.log2_degree = p->ln;
	r.slot = s;
	r.squarings = sl.squarings;
	r.t_submit = p->t_submit[(size_t)s];
	r.t_admit = p->t_admit[(size_t)s];
	r.t_done = mono_seconds();
	std::vector<uint32_t> cv(D), c2(D), c3(D);
	int rc = canonical(p->h_read, sl.b, D, cv.data());
	if (!rc) rc = canonical(p->h_read + D, sl.b, D, c2.data());
	if (!rc) rc = canonical(p->h_read + 2 * D, sl.b, D, c3.data());
	if (rc || status_bad)
		r.status = (int8_t)(rc ? rc : CTW_E_COMPUTE);
	else
	{
		bool prp, zero;
		uint64_t r64;
		res64_of(c3.data(), sl.b, D, prp, zero, r64);
		r.is_prp = prp ? 1 : 0;
		r.res64 = r64;
		r.gl_ok = (cv == c2) ? 1 : 0;
		if (zero) r.status = (int8_t)CTW_E_COMPUTE;
		else if (!r.gl_ok) r.status = (int8_t)CTW_E_GERBICZ;
	}
	p->results.push_back(r);
	sl = PoolSlot{};
	--p->active;
	return CTW_OK;
}

}  // namespace

namespace ctw {

int pool_admit_prepared(ctw_pool *p, const PreparedTest &t, uint64_t tag, double t_submit)
{
	int s = -1;
	for (int i = 0; i < p->slots; ++i)
		if (p->slot[(size_t)i].state == SLOT_FREE) { s = i; break; }
	if (s < 0) return CTW_E_FULL;
	if (t.B != p->B) return fail(CTW_E_ARG, "prepared block %d differs from the pool's %d", t.B, p->B);
	const size_t D = p->D;
	uint32_t *st = p->h_stage + (size_t)s * (4 + p->nwords);
	const uint32_t b = t.b;
	const int sh = (31 - __builtin_clz(b)) - 1;
	st[0] = b;
	st[1] = (uint32_t)(((uint64_t)1 << (sh + 32)) / b);
	st[2] = (uint32_t)sh;
	st[3] = (8.0 * (double)D * (double)b * (double)b < 4.611686018427388e18) ? 1u : 0u;
	uint32_t *w = st + 4;
	memset(w, 0, (size_t)p->nwords * 4);
	if ((int)t.E.size() > p->ewE - 1 || (int)t.res.size() > p->ewR) return fail(CTW_E_ARG, "exponent too long for the pool");
	std::copy(t.E.begin(), t.E.end(), w);
	std::copy(t.res.begin(), t.res.end(), w + p->ewE);
	POOL_CUDA(cudaMemcpyAsync(p->d_laneb + 4 * (size_t)s, st, 16, cudaMemcpyHostToDevice, p->stream));
	POOL_CUDA(cudaMemcpyAsync(p->d_exp + (size_t)s * p->nwords, w, (size_t)p->nwords * 4, cudaMemcpyHostToDevice,
	                          p->stream));
	slot_start(p->slot[(size_t)s], t, tag);
	p->t_admit[(size_t)s] = mono_seconds();
	p->t_submit[(size_t)s] = t_submit;
	++p->active;
	return s;
}

int pool_block(const ctw_pool *p) { return p->B; }
int pool_degree(const ctw_pool *p) { return p->ln; }
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

int ctw_pool_create(int log2_degree, int slots, int log2_ctas, int csize, uint32_t base, int gl_block, ctw_pool **out)
{
	if (!out) return fail(CTW_E_ARG, "null output pointer");
	*out = nullptr;
	if (log2_degree < 8 || log2_degree > 18) return fail(CTW_E_ARG, "log2_degree %d outside [8, 18]", log2_degree);
	if (slots < 1 || slots > 65535) return fail(CTW_E_ARG, "slots %d outside [1, 65535]", slots);
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
	p->B = gl_block ? gl_block : default_gl_block(log2_degree);
	p->D = (size_t)1 << log2_degree;
	p->G = (size_t)1 << lg;
	p->M = p->D / p->G;
	p->tw_smem = prp_smem_bytes(lm, lg, 1) <= 227 * 1024 ? 1 : 0;
	slot_words(log2_degree, p->B, p->ewE, p->ewR);
	p->nwords = p->ewE + p->ewR;
	p->r0 = 32 * p->ewE;
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
	cudaFree(p->d_exp);
	cudaFree(p->d_status);
	cudaFree(p->d_cmd[0]);
	cudaFree(p->d_cmd[1]);
	cudaFreeHost(p->h_cmd[0]);
	cudaFreeHost(p->h_cmd[1]);
	cudaFreeHost(p->h_stage);
	cudaFreeHost(p->h_read);
	for (int k = 0; k < 2; ++k)
		if (p->ev[k]) cudaEventDestroy(p->ev[k]);
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
	slot_prepare(t, p->ln, p->B);
	const double now = mono_seconds();
	return pool_admit_prepared(p, t, tag, now);
}

int ctw_pool_run(ctw_pool *p, int ticks)
{
	if (!p) return fail(CTW_E_ARG, "null pool");
	if (ticks < 0) return fail(CTW_E_ARG, "negative tick count");
	const size_t S = (size_t)p->slots;
	while (ticks > 0)
	{
		const int T = std::min(ticks, POOL_TMAX);
		const int k = (int)(p->seq_issued & 1);
		if (p->ev_pending[k])
		{
			POOL_CUDA(cudaEventSynchronize(p->ev[k]));
			p->ev_pending[k] = false;
			p->seq_complete = std::max(p->seq_complete, p->ev_seq[k] + 1);
		}
		int hi = 0;
		for (int s = 0; s < p->slots; ++s)
			if (p->slot[(size_t)s].state != SLOT_FREE) hi = s + 1;
		// launch over the lowest slots only, rounded up to a power of two (few graphs)
		int lanes = 8;
		while (lanes < hi) lanes *= 2;
		lanes = std::min(lanes, p->slots);
		PrpLaneCmd *hc = p->h_cmd[k];
		memset(hc, 0, (size_t)T * 3 * S * sizeof(PrpLaneCmd));
		for (int t = 0; t < T; ++t)
			for (int s = 0; s < hi; ++s)
			{
				PoolSlot &sl = p->slot[(size_t)s];
				if (sl.state == SLOT_FREE || sl.state == SLOT_FINISHED) continue;
				PrpLaneCmd *c = hc + (size_t)t * 3 * S;
				const long long before = sl.squarings;
				if (slot_tick(sl, p->B, p->r0, c[s], c[S + s], c[2 * S + s])) sl.done_seq = p->seq_issued;
				p->squarings += sl.squarings - before;
			}
		cudaGraphExec_t exec = nullptr;
		if (int rc = get_graph(p, k, T, lanes, exec)) return rc;
		POOL_CUDA(cudaGraphLaunch(exec, p->stream));
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

int ctw_pool_read_slot(ctw_pool *p, int slot, int reg, int32_t *out)
{
	if (!p || !out || slot < 0 || slot >= p->slots || reg < 0 || reg > 3) return fail(CTW_E_ARG, "bad arguments");
	POOL_CUDA(cudaStreamSynchronize(p->stream));
	POOL_CUDA(cudaMemcpy(out, p->d_regs + ((size_t)reg * p->slots + slot) * p->D, p->D * 4, cudaMemcpyDeviceToHost));
	return CTW_OK;
}

void *ctw_pool_stream(ctw_pool *p) { return p ? (void *)p->stream : nullptr; }

int ctw_pool_schedule(int log2_degree, uint32_t b, int gl_block, int32_t *ticks_out, int max_ticks, int *r0)
{
	if (log2_degree < 8 || log2_degree > 18) return fail(CTW_E_ARG, "log2_degree %d outside [8, 18]", log2_degree);
	if (b < 64 || b >= 0x80000000u) return fail(CTW_E_ARG, "b = %u outside [64, 2^31)", b);
	const int B = gl_block ? gl_block : default_gl_block(log2_degree);
	int ewE, ewR;
	slot_words(log2_degree, B, ewE, ewR);
	if (r0) *r0 = 32 * ewE;
	PreparedTest t;
	t.b = b;
	slot_prepare(t, log2_degree, B);
	PoolSlot s;
	slot_start(s, t, 0);
	int n = 0;
	for (bool done = false; !done; ++n)
	{
		PrpLaneCmd aux, sq, mul;
		done = slot_tick(s, B, 32 * ewE, aux, sq, mul);
		if (ticks_out && n < max_ticks)
		{
			int32_t *o = ticks_out + 8 * (size_t)n;
			o[0] = aux.aux;
			o[1] = sq.count;
			o[2] = sq.i_hi;
			o[3] = mul.count;
			o[4] = mul.r_in;
			o[5] = mul.r_y;
			o[6] = mul.r_out;
			o[7] = 0;
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
	static std::mutex mu;
	static std::map<std::pair<int, int>, std::tuple<int, int, double>> cache;
	if (log2_degree < 8 || log2_degree > 18) return fail(CTW_E_ARG, "log2_degree %d outside [8, 18]", log2_degree);
	if (lanes < 1) return fail(CTW_E_ARG, "lanes must be >= 1");
	const int tl = std::min(lanes, 512);
	std::lock_guard<std::mutex> lk(mu);
	auto it = cache.find({ log2_degree, tl });
	if (it == cache.end())
	{
		int best_lg = prp_lg_for(log2_degree), best_cs = 8;
		double best = 1e300;
		std::vector<uint32_t> bv((size_t)tl);
		for (int l = 0; l < tl; ++l) bv[(size_t)l] = (1u << 20) + 7919u * (uint32_t)l;
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
		it = cache.emplace(std::make_pair(log2_degree, tl), std::make_tuple(best_lg, best_cs, best)).first;
	}
	if (log2_ctas) *log2_ctas = std::get<0>(it->second);
	if (csize) *csize = std::get<1>(it->second);
	if (us_per_squaring) *us_per_squaring = std::get<2>(it->second);
	return CTW_OK;
}

}  // extern "C"
