// Host emulation of the grid kernel (prp_grid.cu): every CTA of one lane runs
// at once, one host thread per GPU thread; __syncthreads is a std::barrier per
// CTA, the grid barriers and carry publications are the kernel's own counters
// on host atomics.  It squares a seeded register twice (doubling both times),
// multiplies it by a second one, and compares the digits with the oracle's C
// restatement (bit-exact).  Test infrastructure (tests/test_kernels_emu_cpu.py).
//
// usage: grid_emu <log2 D> <log2 M> <primes> <csize> <b> <threads per CTA> [base multiplier, 2]
#include "emu_shim.h"
#include <barrier>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <pthread.h>
#include <random>
#include <vector>
#include "prp_tables.h"

extern "C" {
typedef struct orc_prp_tables orc_prp_tables;
orc_prp_tables *orc_prp_tables_create(int ln);
void orc_prp_tables_destroy(orc_prp_tables *t);
void orc_square_dup(const orc_prp_tables *t, int32_t *x, uint32_t b, int mult, int csize);
void orc_mul(const orc_prp_tables *t, int32_t *x, const int32_t *yv, uint32_t b, int csize);
}

thread_local dim3 threadIdx, blockIdx;
thread_local int t_cta;
dim3 blockDim, gridDim;
static std::vector<std::vector<uint32_t>> g_sm;
static std::vector<std::barrier<> *> g_bar;
static std::vector<std::barrier<> *> g_wbar;      // [CTA][warp]: 32 threads each
static int g_warps = 1;
void __syncthreads() { g_bar[t_cta]->arrive_and_wait(); }
void emu_syncwarp() { g_wbar[(size_t)t_cta * g_warps + threadIdx.x / 32]->arrive_and_wait(); }
uint32_t *emu_smem() { return g_sm[t_cta].data(); }
// the grid kernel uses no cluster: these abort the emulation if reached
int emu_cta_rank() { abort(); }
void emu_cluster_sync() { abort(); }
void *emu_map_shared(void *, int) { abort(); }
// the kernel's wait budget is 50 ms of this clock; host threads are far slower
// than the GPU, so the clock runs 2000 times slow
unsigned long long emu_timer_ns()
{
	using namespace std::chrono;
	return (unsigned long long)duration_cast<nanoseconds>(steady_clock::now().time_since_epoch()).count() / 2000;
}

namespace ctw {
template <int LG, int NP, int LM> void prp_kernel_grid(const PrpKernelArgs a, const PrpGridArgs ga);
template <int LG, int NP, int LM> void prp_kernel_grid2(const PrpKernelArgs a, const PrpGridArgs ga);
}
using namespace ctw;
typedef void (*Kern)(const PrpKernelArgs, const PrpGridArgs);

static Kern pick(int lg, int lm, int np)
{
#define CTW_EMU_SHAPE(LG, NP, LM, K) if (lg == LG && np == NP && lm == LM) return K<LG, NP, LM>;
	CTW_EMU_SHAPES
#undef CTW_EMU_SHAPE
	return nullptr;
}

// shared-memory words of a grid CTA (the layouts at the top of prp_kernel_grid
// for 4096 coefficients and of prp_kernel_grid2 for 1024 and 2048)
static size_t grid_words(int lg, int lm, int tw, int np)
{
	const size_t M = (size_t)1 << lm, G = (size_t)1 << lg;
	if (lm <= 11)
	{
		// the column planes' pads: 16 words after every 2^r rows of 16 words, r
		// the radix exponent of the last cross pass
		const int npass = (lg + 2) / 3, r = lg / npass + (npass - 1 < lg % npass ? 1 : 0);
		const size_t pad = (M >> lg) == 16 ? (G >> r) * 16 : 0;
		return 2 * np * M + np * pad + M + M / 4 + 2 * G + 2 * np * G + 4 * np * M + np * M + M;
	}
	return 2 * np * M + M / 4 + 2 * G + 2 * np * G + (tw ? 2 * np * M : 0) + (lm == 12 ? 2 * (size_t)np * 512 : 0);
}

struct Job { Kern k; const PrpKernelArgs *a; const PrpGridArgs *ga; int g, t; };
static void *run(void *p)
{
	Job *j = (Job *)p;
	t_cta = j->g;
	threadIdx = dim3(j->t);
	blockIdx = dim3(j->g);
	j->k(*j->a, *j->ga);
	return nullptr;
}

static int launch(Kern k, const PrpKernelArgs &a, const PrpGridArgs &ga, int G, int threads, size_t smem_words,
                  size_t pub_words)
{
	gridDim = dim3(G);
	blockDim = dim3(threads);
	g_sm.assign(G, std::vector<uint32_t>(smem_words, 0xdeadbeefu));
	g_bar.clear();
	for (int g = 0; g < G; ++g) g_bar.push_back(new std::barrier<>(threads));
	g_warps = threads / 32;
	g_wbar.clear();
	for (int w = 0; w < G * g_warps; ++w) g_wbar.push_back(new std::barrier<>(32));
	memset(ga.bar, 0, GRID_BAR_WORDS * sizeof(unsigned));
	memset(ga.gx, 0, pub_words * sizeof(uint32_t));      // as the engine zeroes them before every launch
	memset(ga.gr, 0, pub_words * sizeof(uint32_t));
	std::vector<Job> jobs((size_t)G * threads);
	std::vector<pthread_t> th((size_t)G * threads);
	pthread_attr_t attr;
	pthread_attr_init(&attr);
	pthread_attr_setstacksize(&attr, 1 << 18);
	int rc = 0;
	size_t started = 0;
	for (int g = 0; g < G && !rc; ++g)
		for (int t = 0; t < threads; ++t)
		{
			Job &j = jobs[(size_t)g * threads + t];
			j = Job{ k, &a, &ga, g, t };
			if (pthread_create(&th[started], &attr, run, &j) != 0) { rc = 1; break; }
			++started;
		}
	if (rc) { fprintf(stderr, "pthread_create failed after %zu threads\n", started); _exit(3); }
	for (size_t i = 0; i < started; ++i) pthread_join(th[i], nullptr);
	for (auto *b : g_bar) delete b;
	g_bar.clear();
	for (auto *b : g_wbar) delete b;
	g_wbar.clear();
	return 0;
}

int main(int argc, char **argv)
{
	if (argc < 7) { fprintf(stderr, "usage: grid_emu ln lm primes csize b threads\n"); return 2; }
	const int ln = atoi(argv[1]), lm = atoi(argv[2]), np = atoi(argv[3]), csize = atoi(argv[4]);
	const uint32_t bs = (uint32_t)strtoul(argv[5], nullptr, 10);
	const int nth = atoi(argv[6]);
	const int mult = argc > 7 ? atoi(argv[7]) : 2;
	const int lg = ln - lm, G = 1 << lg;
	const size_t D = (size_t)1 << ln, M = (size_t)1 << lm;
	Kern k = pick(lg, lm, np);
	if (!k) { fprintf(stderr, "shape (%d, %d, %d) not compiled\n", lg, lm, np); return 2; }
	PrpKernelArgs a{};
	std::vector<uint32_t> tf(G * 3 * M), ti(G * 3 * M), tfs(G * 3 * 256 * 2), tis(G * 3 * 256 * 2), xr(768);
	prp_build_tables(ln, lg, tf.data(), ti.data(), a, tfs.data(), tis.data(), xr.data());
	if (lm <= 11)
	{
		tf.assign(2 * tf.size(), 0);
		ti.assign(2 * ti.size(), 0);
		prp_build_grid2_tables(ln, lg, tf.data(), ti.data());
	}
	std::vector<int32_t> x(D), y(D), out(D);
	std::vector<uint32_t> scratch(3 * D), laneb(4), status(1, 0), gx(3 * D), gr(3 * D), bar(GRID_BAR_WORDS);
	std::vector<long long> gc((size_t)G * G);
	std::mt19937 rng(ln * 7 + csize);
	const int sh = (31 - __builtin_clz(bs)) - 1;
	laneb[0] = bs;
	laneb[1] = (uint32_t)(((uint64_t)1 << (sh + 32)) / bs);
	laneb[2] = (uint32_t)sh;
	laneb[3] = (8.0 * D * (double)bs * bs < 4.611686018427388e18) ? 1 : 0;
	for (size_t j = 0; j < D; ++j)
	{
		x[j] = (int32_t)(rng() % bs) - (int32_t)(bs / 2);
		y[j] = (int32_t)(rng() % bs) - (int32_t)(bs / 2);
	}
	a.tf = tf.data(); a.ti = ti.data(); a.tfs = tfs.data(); a.tis = tis.data(); a.lane_b = laneb.data();
	a.status = status.data(); a.lm = lm; a.csize = csize; a.mult = mult; a.scratch = scratch.data(); a.nprime = np;
	a.tw_smem = grid_words(lg, lm, 1, np) * 4 <= 227 * 1024 ? 1 : 0;
	if (lm <= 11 && ((1 << lm) >> lg) < 32) a.swz_b = 20;   // the launch's swizzle for 16-word runs
	PrpGridArgs ga{ gx.data(), gr.data(), gc.data(), bar.data(), xr.data(), 0 };
	const size_t words = grid_words(lg, lm, a.tw_smem, np);
	uint32_t bits[2] = { 3u, 3u };
	std::vector<int32_t> x0 = x;
	a.op = OP_SQUARE; a.reg_in = x.data(); a.reg_out = x.data(); a.bits = bits; a.nwords = 1; a.i_hi = 1; a.count = 2;
	launch(k, a, ga, G, nth, words, gx.size());
	a.op = OP_MUL; a.reg_in = x.data(); a.reg_y = y.data(); a.reg_out = out.data(); a.count = 1;
	launch(k, a, ga, G, nth, words, gx.size());
	orc_prp_tables *t = orc_prp_tables_create(ln);
	std::vector<int32_t> r = x0;
	orc_square_dup(t, r.data(), bs, mult, csize);
	orc_square_dup(t, r.data(), bs, mult, csize);
	int bad = 0, bad2 = 0;
	for (size_t j = 0; j < D; ++j) bad += r[j] != x[j];
	orc_mul(t, r.data(), y.data(), bs, csize);
	for (size_t j = 0; j < D; ++j) bad2 += r[j] != out[j];
	orc_prp_tables_destroy(t);
	printf("status %u mismatches square %d mul %d\n", status[0], bad, bad2);
	return (bad || bad2 || status[0]) ? 1 : 0;
}
