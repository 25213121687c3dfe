// Host emulation of the PRP engine (prp_engine.cu with the kernels of
// prp_kernels.cu, prp_kernels_np2.cu and prp_grid.cu on the stand-in runtime
// of engine_stub/cuda_runtime.h): whole Fermat tests through ctw_prp_run on
// the CPU; prints, per lane, b, the PRP flag, RES64 and the Gerbicz-Li check.
// Test infrastructure (tests/test_kernels_emu_cpu.py).
//
// usage: engine_emu <log2 D> <base 2|3> <minus 0|1> <b> [<b> ...]
//        engine_emu pool <log2 D> <slots> <base 2|3> <b> [<b> ...]
//        engine_emu server <log2 D> <max slots> <base 2|3> <b> [<b> ...]
//        engine_emu mul <log2 D> <csize> <in file> <out file> <b> [<b> ...]
//        engine_emu resume <log2 D> <base 2|3> <context file> <b>
//        engine_emu batch <ticks>
// resume: the whole test stops at its first Gerbicz-Li checkpoint, saves the
// reference's context file there, and a fresh engine reads it and finishes.
// batch: pools of degrees 2^12 (two and three primes), 2^13 and 2^14 (ticks
// of 8 squarings) run <ticks> ticks through one batch (ctw_batch_run: the persistent kernel with
// per-degree queues) and, as a second set of the same pools, through
// ctw_pool_run; prints the number of register words that differ.
// mul: ctw_prp_mul_noalloc of the lanes' x and y (int32 digits, x then y, read
// from the in file) into z (written to the out file).
// The second form runs the tests as a pool (continuous batching, ticks
// replayed from recorded graphs) and prints the same line per test.
#include "emu_shim.h"
#include <barrier>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <memory>
#include <thread>
#include <vector>
#include "cuda_runtime.h"
#include "../../include/ctwin_gb300.h"

std::vector<std::function<void()>> *emu_capture = nullptr;
thread_local dim3 threadIdx, blockIdx;
thread_local int t_cta;
dim3 blockDim, gridDim;
static std::vector<std::vector<uint32_t>> g_sm;
static std::vector<std::unique_ptr<std::barrier<>>> g_bar;
static std::unique_ptr<std::barrier<>> g_cbar;
static std::vector<std::unique_ptr<std::barrier<>>> g_wbar;   // [CTA][warp] of 32 threads
static unsigned g_nwarps = 1;
void __syncthreads() { g_bar[t_cta]->arrive_and_wait(); }
void emu_syncwarp() { g_wbar[(size_t)t_cta * g_nwarps + threadIdx.x / 32]->arrive_and_wait(); }
uint32_t *emu_smem() { return g_sm[t_cta].data(); }
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
unsigned long long emu_timer_ns()
{
	using namespace std::chrono;
	return (unsigned long long)duration_cast<nanoseconds>(steady_clock::now().time_since_epoch()).count() / 2000;
}

// CTAs in groups (a cluster, or the whole cooperative grid) that run at once;
// groups one after another
void emu_run_ctas(dim3 grid, dim3 block, size_t smem, int group, void (*body)(void *), void *ctx)
{
	gridDim = grid;
	blockDim = block;
	const unsigned nt = block.x * block.y * block.z, nb = grid.x * grid.y * grid.z;
	if (group < 1) group = 1;
	for (unsigned g0 = 0; g0 < nb; g0 += (unsigned)group)
	{
		const unsigned ng = std::min<unsigned>((unsigned)group, nb - g0);
		g_sm.assign(ng, std::vector<uint32_t>(smem / 4 + 4, 0xdeadbeefu));
		g_bar.clear();
		for (unsigned c = 0; c < ng; ++c) g_bar.emplace_back(new std::barrier<>(nt));
		g_cbar.reset(new std::barrier<>(ng * nt));
		g_nwarps = nt / 32 ? nt / 32 : 1;
		g_wbar.clear();
		for (unsigned w = 0; w < ng * g_nwarps; ++w) g_wbar.emplace_back(new std::barrier<>(nt < 32 ? nt : 32));
		std::vector<std::thread> th;
		th.reserve((size_t)ng * nt);
		for (unsigned c = 0; c < ng; ++c)
			for (unsigned t = 0; t < nt; ++t)
				th.emplace_back([=] {
					t_cta = (int)c;
					const unsigned b = g0 + c;
					threadIdx = dim3(t % block.x, (t / block.x) % block.y, t / (block.x * block.y));
					blockIdx = dim3(b % grid.x, (b / grid.x) % grid.y, b / (grid.x * grid.y));
					body(ctx);
				});
		for (auto &x : th) x.join();
	}
}

static int run_batch(int argc, char **argv)
{
	const int ticks = atoi(argv[2]);
	struct Spec { int ln, slots; std::vector<uint32_t> b; };
	const std::vector<Spec> specs = {
		{ 14, 2, { 100003, 65537 } },
		{ 13, 4, { 70001, 1000003, 64 } },
		{ 12, 8, { 65537, 100, 9000001, 123457, 2000003 } },
		{ 12, 8, { 9999991, 16777213 } },                 // above the two-prime bound: three primes
	};
	std::vector<ctw_pool *> batched, alone;
	int rc = 0;
	for (int set = 0; set < 2 && !rc; ++set)
		for (const Spec &sp : specs)
		{
			ctw_pool *p = nullptr;
			// Gerbicz-Li blocks of 8 squarings keep the emulated ticks short
			if ((rc = ctw_pool_create(sp.ln, sp.slots, sp.ln - 12, 8, 3, 8, &p))) break;
			(set ? alone : batched).push_back(p);
			for (size_t i = 0; i < sp.b.size() && !rc; ++i) rc = ctw_pool_admit(p, sp.b[i], i) < 0;
		}
	ctw_batch *bt = nullptr;
	if (!rc) rc = ctw_batch_create(batched.data(), (int)batched.size(), &bt);
	if (!rc) rc = ctw_batch_run(bt, ticks);
	for (size_t i = 0; i < alone.size() && !rc; ++i) rc = ctw_pool_run(alone[i], ticks);
	long long bad = 0, words = 0;
	for (size_t i = 0; i < alone.size() && !rc; ++i)
	{
		rc = ctw_pool_collect(batched[i], 1) < 0 || ctw_pool_collect(alone[i], 1) < 0;
		const size_t D = (size_t)1 << specs[i].ln;
		std::vector<int32_t> x(D), y(D);
		for (int s = 0; s < specs[i].slots && !rc; ++s)
			for (int r = 0; r < 6 && !rc; ++r)
			{
				rc = ctw_pool_read_slot(batched[i], s, r, x.data()) || ctw_pool_read_slot(alone[i], s, r, y.data());
				for (size_t j = 0; j < D; ++j) bad += x[j] != y[j];
				words += (long long)D;
			}
	}
	if (rc) fprintf(stderr, "batch: %s\n", ctw_last_error());
	ctw_batch_destroy(bt);
	for (ctw_pool *p : batched) ctw_pool_destroy(p);
	for (ctw_pool *p : alone) ctw_pool_destroy(p);
	printf("batch registers compared %lld differ %lld\n", words, bad);
	return (rc || bad || !words) ? 1 : 0;
}

static int run_pool(int argc, char **argv)
{
	const int ln = atoi(argv[2]), slots = atoi(argv[3]), base = atoi(argv[4]);
	std::vector<uint32_t> bs;
	for (int i = 5; i < argc; ++i) bs.push_back((uint32_t)strtoul(argv[i], nullptr, 10));
	ctw_pool *p = nullptr;
	int rc = ctw_pool_create(ln, slots, -1, 0, (uint32_t)base, 0, &p);
	size_t next = 0, done = 0;
	std::vector<ctw_result> res(64);
	while (!rc && done < bs.size())
	{
		// admit while slots are free, one tick at a time
		while (next < bs.size() && ctw_pool_admit(p, bs[next], next) >= 0) ++next;
		if ((rc = ctw_pool_run(p, 1)) < 0) break;
		const int n = ctw_pool_collect(p, 1);
		if (n < 0) { rc = n; break; }
		rc = 0;
		for (int got; (got = ctw_pool_results(p, res.data(), (int)res.size())) > 0;)
			for (int i = 0; i < got; ++i, ++done)
				printf("%u %d %016llX %d %d\n", res[(size_t)i].b, res[(size_t)i].is_prp,
				       (unsigned long long)res[(size_t)i].res64, res[(size_t)i].gl_ok, res[(size_t)i].status);
	}
	if (rc) fprintf(stderr, "error %d: %s\n", rc, ctw_last_error());
	if (p) ctw_pool_destroy(p);
	return rc ? 1 : 0;
}

// the request loop: submit every b, poll until each has a result
static int run_server(int argc, char **argv)
{
	const int ln = atoi(argv[2]), max_slots = atoi(argv[3]), base = atoi(argv[4]);
	std::vector<uint32_t> bs;
	for (int i = 5; i < argc; ++i) bs.push_back((uint32_t)strtoul(argv[i], nullptr, 10));
	ctw_server *s = nullptr;
	int rc = ctw_server_create((size_t)1 << 30, max_slots, (uint32_t)base, 1, 0, &s);
	// CTW_EMU_GRID_LANE=<ln>:<b>[,<b>...]: more requests of degree 2^ln, served
	// by the server's grid lanes (threshold ln), while the others run in pools
	const char *gl = getenv("CTW_EMU_GRID_LANE");
	const size_t npool = bs.size();
	int gln = 0;
	if (gl && sscanf(gl, "%d:", &gln) == 1 && !rc)
	{
		rc = ctw_server_set_grid_lane(s, gln);
		const char *nl = getenv("CTW_EMU_GRID_LANES");
		if (!rc) rc = ctw_server_set_grid_lanes(s, nl ? atoi(nl) : 2);
		for (const char *q = strchr(gl, ':'); q && !rc; q = strchr(q + 1, ','))
		{
			const uint32_t gb = (uint32_t)strtoul(q + 1, nullptr, 10);
			rc = ctw_server_submit(s, gln, gb, bs.size());
			bs.push_back(gb);
		}
	}
	for (size_t i = 0; i < npool && !rc; ++i) rc = ctw_server_submit(s, ln, bs[i], i);
	size_t done = 0;
	std::vector<ctw_result> res(16);
	const auto t0 = std::chrono::steady_clock::now();
	while (!rc && done < bs.size())
	{
		const int got = ctw_server_poll(s, res.data(), (int)res.size(), 1000);
		if (got < 0) { rc = got; break; }
		for (int i = 0; i < got; ++i, ++done)
			printf("%u %d %016llX %d %d %d\n", res[(size_t)i].b, res[(size_t)i].is_prp,
			       (unsigned long long)res[(size_t)i].res64, res[(size_t)i].gl_ok, res[(size_t)i].status,
			       res[(size_t)i].slot);
		if (std::chrono::steady_clock::now() - t0 > std::chrono::minutes(10)) { rc = -100; break; }
	}
	if (rc) fprintf(stderr, "error %d: %s\n", rc, ctw_last_error());
	if (s) ctw_server_destroy(s);
	return rc ? 1 : 0;
}

static int run_mul(int argc, char **argv)
{
	const int ln = atoi(argv[2]), csize = atoi(argv[3]);
	std::vector<uint32_t> bs;
	for (int i = 6; i < argc; ++i) bs.push_back((uint32_t)strtoul(argv[i], nullptr, 10));
	const size_t lanes = bs.size(), D = (size_t)1 << ln;
	std::vector<int32_t> xy(2 * lanes * D), z(lanes * D);
	FILE *f = fopen(argv[4], "rb");
	if (!f || fread(xy.data(), 4, xy.size(), f) != xy.size()) { fprintf(stderr, "bad input file\n"); return 2; }
	fclose(f);
	const int rc = ctw_prp_mul_noalloc(ln, (int)lanes, bs.data(), xy.data(), xy.data() + lanes * D, z.data(), csize,
	                                   nullptr);
	if (rc) { fprintf(stderr, "error %d: %s\n", rc, ctw_last_error()); return 1; }
	f = fopen(argv[5], "wb");
	if (!f || fwrite(z.data(), 4, z.size(), f) != z.size()) return 2;
	fclose(f);
	return 0;
}

static ctw_prp *g_stop_h = nullptr;
static const char *g_stop_path = nullptr;
static int stop_at_checkpoint(void *, long long i)
{
	return ctw_prp_save_context(g_stop_h, g_stop_path, 0, (int)i, 0.0) == CTW_OK ? 1 : -1;
}

static int run_resume(char **argv)
{
	const int ln = atoi(argv[2]), base = atoi(argv[3]);
	g_stop_path = argv[4];
	const uint32_t b = (uint32_t)strtoul(argv[5], nullptr, 10);
	uint8_t prp = 0, gl = 0;
	uint64_t r64 = 0;
	ctw_prp *h = nullptr;
	int rc = ctw_prp_create(ln, 1, &h);
	if (!rc) rc = ctw_prp_set_base(h, (uint32_t)base);
	g_stop_h = h;
	if (!rc) rc = ctw_prp_run_ex(h, &b, 1, -1, stop_at_checkpoint, nullptr, &prp, &r64, &gl);
	if (h) ctw_prp_destroy(h);
	if (rc != CTW_STOPPED) { fprintf(stderr, "first run: %d (expected a stop) %s\n", rc, ctw_last_error()); return 1; }
	h = nullptr;
	int k = 0, i = 0;
	double el = 0;
	rc = ctw_prp_create(ln, 1, &h);
	if (!rc) rc = ctw_prp_set_base(h, (uint32_t)base);
	if (!rc) rc = ctw_prp_set_b(h, &b, 1);
	if (!rc) rc = ctw_prp_read_context(h, g_stop_path, &k, &i, &el);
	if (!rc) rc = ctw_prp_run_ex(h, &b, 1, i, nullptr, nullptr, &prp, &r64, &gl);
	if (rc) fprintf(stderr, "resume: %d %s\n", rc, ctw_last_error());
	else printf("%u %d %016llX %d %d\n", b, prp, (unsigned long long)r64, gl, i);
	if (h) ctw_prp_destroy(h);
	return rc ? 1 : 0;
}

int main(int argc, char **argv)
{
	if (argc >= 6 && strcmp(argv[1], "resume") == 0) return run_resume(argv);
	if (argc >= 7 && strcmp(argv[1], "mul") == 0) return run_mul(argc, argv);
	if (argc >= 6 && strcmp(argv[1], "pool") == 0) return run_pool(argc, argv);
	if (argc >= 3 && strcmp(argv[1], "batch") == 0) return run_batch(argc, argv);
	if (argc >= 6 && strcmp(argv[1], "server") == 0) return run_server(argc, argv);
	if (argc < 5) { fprintf(stderr, "usage: engine_emu ln base minus b...\n"); return 2; }
	const int ln = atoi(argv[1]), base = atoi(argv[2]), minus = atoi(argv[3]);
	std::vector<uint32_t> bs;
	for (int i = 4; i < argc; ++i) bs.push_back((uint32_t)strtoul(argv[i], nullptr, 10));
	const int lanes = (int)bs.size();
	ctw_prp *h = nullptr;
	int rc = minus ? ctw_prp_create_minus(ln, lanes, &h) : ctw_prp_create(ln, lanes, &h);
	if (!rc) rc = ctw_prp_set_base(h, (uint32_t)base);
	std::vector<uint8_t> prp(lanes), gl(lanes);
	std::vector<uint64_t> r64(lanes);
	if (!rc) rc = ctw_prp_run(h, bs.data(), lanes, prp.data(), r64.data(), gl.data());
	if (rc) fprintf(stderr, "error %d: %s\n", rc, ctw_last_error());
	for (int l = 0; l < lanes && !rc; ++l)
		printf("%u %d %016llX %d\n", bs[(size_t)l], prp[(size_t)l], (unsigned long long)r64[(size_t)l], gl[(size_t)l]);
	if (h) ctw_prp_destroy(h);
	return rc ? 1 : 0;
}
