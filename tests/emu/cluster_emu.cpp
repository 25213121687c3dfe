// Host emulation of the one-CTA and thread-block-cluster PRP kernels
// (prp_kernel_impl.cuh): the CTAs of one lane's cluster run at once, one host
// thread per GPU thread; __syncthreads is a std::barrier per CTA, the cluster
// barrier one over the cluster, and distributed shared memory maps a word to
// the same offset in the peer CTA's buffer.  Two lanes (b given), one doubling
// squaring and one multiply, digits compared with the oracle's C restatement
// (bit-exact).  With minus = 1 the registers are N- values on the degree-2D
// transform (upper halves zero) and the digits are printed for a check of
// x1 = mult x0^2 and out = x1 y mod N- by the caller.  Test infrastructure
// (tests/test_kernels_emu_cpu.py).
//
// usage: cluster_emu <log2 D> <log2 G> <primes> <dense 0|1> <csize> <b0> <b1> [minus mult]
#include "emu_shim.h"
#include <barrier>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <thread>
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
static std::barrier<> *g_cbar;
void __syncthreads() { g_bar[t_cta]->arrive_and_wait(); }
uint32_t *emu_smem() { return g_sm[t_cta].data(); }
unsigned long long emu_timer_ns() { return 0; }
int emu_cta_rank() { return t_cta; }
void emu_cluster_sync() { g_cbar->arrive_and_wait(); }
void *emu_map_shared(void *p, int r)
{
	const char *base = (const char *)g_sm[t_cta].data();
	const ptrdiff_t off = (const char *)p - base;
	if (off < 0 || (size_t)off >= g_sm[t_cta].size() * 4 || r < 0 || (size_t)r >= g_sm.size())
	{
		fprintf(stderr, "map_shared_rank: pointer outside shared memory or rank out of range\n");
		abort();
	}
	return (char *)g_sm[r].data() + off;
}

namespace ctw {
template <int LG, bool M12, int NP, bool DENSE> void prp_kernel(const PrpKernelArgs a);
template <int LG, bool M12, int NP, bool DENSE> void prp_kernel_cols(const PrpKernelArgs a);
size_t prp_smem_bytes(int lm, int lg, int tw_smem, int np);
int prp_threads(int lm, int np, int lg);
}
using namespace ctw;
typedef void (*Kern)(const PrpKernelArgs);

// CTW_EMU_SHAPE(COLS, LG, M12, NP, DENSE) for every compiled instantiation
static Kern pick(int lg, bool m12, int np, bool dense)
{
#define CTW_EMU_SHAPE(COLS, LG, M12, NP, DENSE)                                           \
	if (lg == LG && m12 == M12 && np == NP && dense == DENSE)                             \
		return COLS ? prp_kernel_cols<LG, M12, NP, DENSE> : prp_kernel<LG, M12, NP, DENSE>;
	CTW_EMU_SHAPES
#undef CTW_EMU_SHAPE
	return nullptr;
}

static void launch(Kern k, const PrpKernelArgs &a, int lanes, int G, int threads, size_t smem)
{
	gridDim = dim3(lanes * G);
	blockDim = dim3(threads);
	for (int lane = 0; lane < lanes; ++lane)
	{
		g_sm.assign(G, std::vector<uint32_t>(smem / 4, 0xdeadbeefu));
		g_bar.clear();
		for (int g = 0; g < G; ++g) g_bar.push_back(new std::barrier<>(threads));
		std::barrier<> cbar(G * threads);
		g_cbar = &cbar;
		std::vector<std::thread> th;
		th.reserve((size_t)G * threads);
		for (int g = 0; g < G; ++g)
			for (int t = 0; t < threads; ++t)
				th.emplace_back([&, g, t, lane] {
					t_cta = g;
					threadIdx = dim3(t);
					blockIdx = dim3(lane * G + g);
					k(a);
				});
		for (auto &x : th) x.join();
		for (auto *b : g_bar) delete b;
		g_bar.clear();
	}
}

int main(int argc, char **argv)
{
	if (argc < 8) { fprintf(stderr, "usage: cluster_emu ln lg primes dense csize b0 b1\n"); return 2; }
	const int ln = atoi(argv[1]), lg = atoi(argv[2]), np = atoi(argv[3]), dense = atoi(argv[4]), csize = atoi(argv[5]);
	const uint32_t bs[2] = { (uint32_t)strtoul(argv[6], nullptr, 10), (uint32_t)strtoul(argv[7], nullptr, 10) };
	const int minus = argc > 8 ? atoi(argv[8]) : 0, mult = argc > 9 ? atoi(argv[9]) : 2;
	const int lm = ln - lg, G = 1 << lg, lanes = 2;
	const size_t D = (size_t)1 << ln, M = D / G;
	Kern k = pick(lg, lm == 12, np, dense != 0);
	if (!k) { fprintf(stderr, "shape not compiled\n"); return 2; }
	PrpKernelArgs a{};
	std::vector<uint32_t> tf(G * 3 * M), ti(G * 3 * M), tfs(G * 3 * 256 * 2), tis(G * 3 * 256 * 2);
	prp_build_tables(ln, lg, tf.data(), ti.data(), a, tfs.data(), tis.data());
	std::vector<int32_t> x(lanes * D), y(lanes * D), out(lanes * D);
	std::vector<uint32_t> scratch(lanes * D * 3), laneb(lanes * 4), status(1, 0);
	std::mt19937 rng(ln * 131 + lg);
	for (int l = 0; l < lanes; ++l)
	{
		const uint32_t b = bs[l];
		const int sh = (31 - __builtin_clz(b)) - 1;
		laneb[4 * l] = b;
		laneb[4 * l + 1] = (uint32_t)(((uint64_t)1 << (sh + 32)) / b);
		laneb[4 * l + 2] = (uint32_t)sh;
		laneb[4 * l + 3] = (8.0 * D * (double)b * b < 4.611686018427388e18) ? 1 : 0;
		for (size_t j = 0; j < D; ++j)
		{
			const bool upper = minus && j >= D / 2;
			x[l * D + j] = upper ? 0 : (int32_t)(rng() % b) - (int32_t)(b / 2);
			y[l * D + j] = upper ? 0 : (int32_t)(rng() % b) - (int32_t)(b / 2);
		}
	}
	a.tf = tf.data(); a.ti = ti.data(); a.tfs = tfs.data(); a.tis = tis.data(); a.lane_b = laneb.data();
	a.status = status.data(); a.lm = lm; a.csize = csize; a.mult = mult; a.scratch = scratch.data(); a.nprime = np;
	a.minus = minus;
	// the launch's choices (launch_lg): the dense three-prime build keeps roots and
	// Shoup tables in global memory and runs 384 threads
	const bool dense3 = dense && np == 3;
	a.tw_smem = dense ? 0 : (prp_smem_bytes(lm, lg, 1, np) <= 227 * 1024 ? 1 : 0);
	const size_t smem = prp_smem_bytes(lm, lg, a.tw_smem, np) - (dense3 ? prp_shoup_words(12, 3) * 4 : 0);
	const int threads = dense3 ? 384 : prp_threads(lm, np, lg);
	uint32_t bits[2] = { 1u, 1u };
	std::vector<int32_t> x0 = x;
	a.op = OP_SQUARE; a.reg_in = x.data(); a.reg_out = x.data(); a.bits = bits; a.nwords = 1; a.i_hi = 0; a.count = 1;
	launch(k, a, lanes, G, threads, smem);
	a.op = OP_MUL; a.reg_in = x.data(); a.reg_y = y.data(); a.reg_out = out.data(); a.count = 1;
	launch(k, a, lanes, G, threads, smem);
	if (minus)
	{
		// lanes of four lines each: x0, y, x after the squaring, x * y
		for (int l = 0; l < lanes; ++l)
			for (const std::vector<int32_t> *v : { &x0, &y, &x, &out })
			{
				for (size_t j = 0; j < D; ++j) printf("%d ", (*v)[l * D + j]);
				printf("\n");
			}
		printf("status %u\n", status[0]);
		return status[0] ? 1 : 0;
	}
	orc_prp_tables *t = orc_prp_tables_create(ln);
	int bad = 0, bad2 = 0;
	for (int l = 0; l < lanes; ++l)
	{
		std::vector<int32_t> r(x0.begin() + l * D, x0.begin() + (l + 1) * D);
		orc_square_dup(t, r.data(), bs[l], 2, csize);
		for (size_t j = 0; j < D; ++j) bad += r[j] != x[l * D + j];
		orc_mul(t, r.data(), y.data() + l * D, bs[l], csize);
		for (size_t j = 0; j < D; ++j) bad2 += r[j] != out[l * D + j];
	}
	orc_prp_tables_destroy(t);
	printf("status %u mismatches square %d mul %d\n", status[0], bad, bad2);
	return (bad || bad2 || status[0]) ? 1 : 0;
}
