// Host emulation of the sieve path (ctwin_gb300/csrc/sieve.cu, compiled with
// sieve_shim.h): runs ctw_sieve_run on the CPU and prints the struck bitmap
// and the last p, for a comparison with the oracle's sieve by the caller.
// Test infrastructure (tests/test_kernels_emu_cpu.py).
//
// usage: sieve_emu <n> <b_min> <b_max> <p_min> <p_max> <mode +1|-1>
//        sieve_emu case <n> <b_min> <b_max> <p_max_pos> <p_max_neg> <mode 1|0|-1> <dir>
//        sieve_emu factors <n> <k_begin> <k_end> <mode +1|-1> <b_max>
// The second form runs a reference sieve case as the reference's Sieve class
// does (+ from 3*2^n + 1, - from 11, each pass raising its last p) and writes
// sv_*.dat / cand_*.txt into dir with ctw_sieve_write_files.
#include "sieve_shim.h"
#include "../../include/ctwin_gb300.h"

thread_local dim3 threadIdx, blockIdx;
dim3 blockDim, gridDim;
static std::barrier<> *g_bar = nullptr;
static std::vector<uint32_t> g_dyn;
void __syncthreads() { g_bar->arrive_and_wait(); }
uint32_t *emu_dyn_smem() { return g_dyn.data(); }
int emu_sms() { return 2; }

// CTAs one after another (their static shared variables are plain statics),
// the threads of a CTA at once
void emu_run_blocks(const EmuCfg &c, void (*body)(void *), void *ctx)
{
	gridDim = c.grid;
	blockDim = c.block;
	const unsigned nt = c.block.x * c.block.y * c.block.z;
	for (unsigned bz = 0; bz < c.grid.z; ++bz)
		for (unsigned by = 0; by < c.grid.y; ++by)
			for (unsigned bx = 0; bx < c.grid.x; ++bx)
			{
				g_dyn.assign(c.smem / 4 + 1, 0xdeadbeefu);
				std::barrier<> bar(nt);
				g_bar = &bar;
				std::vector<std::thread> th;
				th.reserve(nt);
				for (unsigned t = 0; t < nt; ++t)
					th.emplace_back([=] {
						threadIdx = dim3(t % c.block.x, (t / c.block.x) % c.block.y, t / (c.block.x * c.block.y));
						blockIdx = dim3(bx, by, bz);
						body(ctx);
					});
				for (auto &x : th) x.join();
			}
}

namespace ctw {
int fail(int code, const char *fmt, ...)
{
	va_list ap;
	va_start(ap, fmt);
	vfprintf(stderr, fmt, ap);
	va_end(ap);
	fprintf(stderr, "\n");
	return code;
}
}
extern "C" int ctw_device_count(void) { return 1; }

static int run_case(char **argv)
{
	const int n = atoi(argv[2]), mode = atoi(argv[7]);
	const uint64_t b_min = strtoull(argv[3], nullptr, 10), b_max = strtoull(argv[4], nullptr, 10);
	const uint64_t pmax_pos = strtoull(argv[5], nullptr, 10), pmax_neg = strtoull(argv[6], nullptr, 10);
	std::vector<uint32_t> words((b_max - b_min + 1 + 31) / 32, 0);
	uint64_t p_pos = 3 * (1ull << n) + 1, p_neg = 11;
	int rc = 0;
	if (mode >= 0) rc = ctw_sieve_run(n, b_min, b_max, p_pos, pmax_pos, 1, words.data(), &p_pos);
	if (!rc && mode <= 0) rc = ctw_sieve_run(n, b_min, b_max, p_neg, pmax_neg, -1, words.data(), &p_neg);
	if (!rc) rc = ctw_sieve_write_files(n, b_min, b_max, words.data(), p_pos, p_neg, argv[8]);
	printf("rc %d p_last %llu %llu\n", rc, (unsigned long long)p_pos, (unsigned long long)p_neg);
	return rc ? 1 : 0;
}

// ctw_sieve_factors: prints the pair count, then "p b" per line
static int run_factors(char **argv)
{
	const int n = atoi(argv[2]), mode = atoi(argv[5]);
	const uint64_t k_b = strtoull(argv[3], nullptr, 10), k_e = strtoull(argv[4], nullptr, 10);
	const uint64_t b_max = strtoull(argv[6], nullptr, 10), cap = 1 << 20;
	std::vector<uint64_t> pairs(2 * cap);
	uint64_t count = 0;
	const int rc = ctw_sieve_factors(n, k_b, k_e, mode, b_max, pairs.data(), cap, &count);
	printf("rc %d count %llu\n", rc, (unsigned long long)count);
	for (uint64_t i = 0; i < count && !rc; ++i)
		printf("%llu %llu\n", (unsigned long long)pairs[2 * i], (unsigned long long)pairs[2 * i + 1]);
	return rc ? 1 : 0;
}

int main(int argc, char **argv)
{
	if (argc >= 9 && strcmp(argv[1], "case") == 0) return run_case(argv);
	if (argc >= 7 && strcmp(argv[1], "factors") == 0) return run_factors(argv);
	if (argc < 7) { fprintf(stderr, "usage: sieve_emu n b_min b_max p_min p_max mode\n"); return 2; }
	const int n = atoi(argv[1]), mode = atoi(argv[6]);
	const uint64_t b_min = strtoull(argv[2], nullptr, 10), b_max = strtoull(argv[3], nullptr, 10);
	const uint64_t p_min = strtoull(argv[4], nullptr, 10), p_max = strtoull(argv[5], nullptr, 10);
	std::vector<uint32_t> words((b_max - b_min + 1 + 31) / 32, 0);
	uint64_t p_last = 0;
	const int rc = ctw_sieve_run(n, b_min, b_max, p_min, p_max, mode, words.data(), &p_last);
	printf("rc %d p_last %llu\n", rc, (unsigned long long)p_last);
	for (uint32_t w : words) printf("%u ", w);
	printf("\n");
	return rc ? 1 : 0;
}
