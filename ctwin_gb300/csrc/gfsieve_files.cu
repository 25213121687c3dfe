// File-level compatibility with the reference's GPU sieve (ctsieveg,
// sieve/GPU/src/ctsieve.h:248-421): factor files fp<n>_<pmin>_<pmax>.txt /
// fn..., the text context ctx<...> / ctx_n<...> (blocks done, elapsed time),
// the block-aligned k range and the host check of every factor.  Host code.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/ctwin_gb300.h"
#include "prp_host.h"

using namespace ctw;

namespace {

constexpr int LOG2_BLOCK = 21;                 // the reference's _log2GlobalWorkSize
constexpr uint64_t TERA = 1000000000000ull;

uint64_t mulmod(uint64_t a, uint64_t b, uint64_t p) { return (uint64_t)((unsigned __int128)a * b % p); }

uint64_t powmod(uint64_t a, uint64_t e, uint64_t p)
{
	uint64_t r = 1 % p;
	for (; e; e >>= 1, a = mulmod(a, a, p))
		if (e & 1) r = mulmod(r, a, p);
	return r;
}

// bMax of the reference's kernels (sieve/GPU/ocl/kernel.cl:304, 434)
uint64_t b_max_of(uint64_t p, int mode)
{
	const uint64_t thr = (mode > 0) ? 10000000000000000ull : 10000000000000ull;
	return (p < thr) ? 5000000000ull : 10000000000ull;
}

}  // namespace

extern "C" int ctw_gfsieve_check(int n, uint64_t p_min, uint64_t p_max, int mode, const char *workdir,
                                 volatile int *quit, int stop_after_blocks, uint64_t *factors_written)
{
	if (n < 8 || n > 24) return fail(CTW_E_ARG, "n = %d outside [8, 24]", n);
	if (mode != 1 && mode != -1) return fail(CTW_E_ARG, "mode must be +1 or -1");
	if (p_max <= p_min) return fail(CTW_E_ARG, "p_max must exceed p_min");
	const std::string dir = (workdir && *workdir) ? std::string(workdir) : std::string(".");
	std::ostringstream es;
	es << n << "_" << (p_min / TERA) << "_" << (p_max / TERA) << ".txt";
	const std::string ext = es.str();
	const std::string ctx = dir + "/" + (mode > 0 ? "ctx" : "ctx_n") + ext;
	const std::string out = dir + "/" + (mode > 0 ? "fp" : "fn") + ext;

	uint64_t cnt = 0;
	double elapsed0 = 0;
	{
		std::ifstream f(ctx);
		if (f.is_open()) f >> cnt >> elapsed0;
	}
	// block range of the reference (ctsieve.h:345-349), in the same double arithmetic
	const double fr = (mode > 0) ? 1.0 / double(3ull << (LOG2_BLOCK + n)) : 1.0 / double(10u << LOG2_BLOCK);
	const uint64_t i_min = uint64_t(floor(double(p_min) * fr)), i_max = uint64_t(ceil(double(p_max) * fr));

	using clk = std::chrono::steady_clock;
	const auto t0 = clk::now();
	uint64_t written = 0;
	int blocks = 0;
	std::vector<uint64_t> pairs;
	for (uint64_t i = i_min + cnt; i < i_max; ++i)
	{
		if ((quit && *quit) || (stop_after_blocks > 0 && blocks >= stop_after_blocks))
		{
			if (factors_written) *factors_written = written;
			return CTW_STOPPED;
		}
		const uint64_t k_b = std::max<uint64_t>(1, i << LOG2_BLOCK), k_e = (i + 1) << LOG2_BLOCK;
		uint64_t m = 0;
		if (pairs.size() < (size_t)2 << 22) pairs.resize((size_t)2 << 22);
		int rc = ctw_sieve_factors(n, k_b, k_e, mode, 10000000000ull, pairs.data(), pairs.size() / 2, &m);
		if (rc == CTW_E_NOMEM && 2 * m > pairs.size())
		{
			pairs.resize(2 * (size_t)m);
			rc = ctw_sieve_factors(n, k_b, k_e, mode, 10000000000ull, pairs.data(), m, &m);
		}
		if (rc) return rc;
		// keep p in [p_min, p_max] and b <= bMax(p); check each factor on the host
		// (ctsieve.h:248-293)
		std::ostringstream ss;
		for (size_t j = 0; j < m; ++j)
		{
			const uint64_t p = pairs[2 * j], b = pairs[2 * j + 1];
			if (p < p_min || p > p_max || b > b_max_of(p, mode)) continue;
			const uint64_t x = powmod(b % p, 1ull << (n - 1), p);
			const uint64_t r = (mulmod(x, x, p) + p - x) % p;
			if ((mode > 0 && r != p - 1) || (mode < 0 && r != 1))
				return fail(CTW_E_COMPUTE, "%llu doesn't divide %llu^%d - %llu^%d %c 1", (unsigned long long)p,
				            (unsigned long long)b, 1 << n, (unsigned long long)b, 1 << (n - 1), mode > 0 ? '+' : '-');
			ss << p << " " << b << "\n";
			++written;
		}
		{
			std::ofstream f(out, std::ios::app);
			if (!f.is_open() || !(f << ss.str())) return fail(CTW_E_ARG, "cannot write %s", out.c_str());
		}
		++cnt;
		++blocks;
		const double el = elapsed0 + std::chrono::duration<double>(clk::now() - t0).count();
		std::ofstream f(ctx);
		if (!f.is_open() || !(f << cnt << "\n" << el << "\n")) return fail(CTW_E_ARG, "cannot write %s", ctx.c_str());
	}
	if (factors_written) *factors_written = written;
	return CTW_OK;
}
