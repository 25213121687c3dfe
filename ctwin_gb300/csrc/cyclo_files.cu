// File-level compatibility with the reference's cyclog: the context file
// (cyclo.ctx), the result files and the <file>.ini CSIZE, and the file loop
// that ties them to the engine.  Host code only.
#include <cerrno>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "../../include/ctwin_gb300.h"
#include "prp_host.h"

using namespace ctw;

namespace {

// The reference stores each digit d as its residues mod these three primes
// (cyclo/src/transform.h:26-28, seti_P* of cyclo/ocl/kernel.cl:133-135); the
// context format depends on them, so they are repeated here.
constexpr uint32_t RP1 = 4293918721u, RP2 = 4253024257u, RP3 = 4231004161u;
constexpr uint32_t CTX_VERSION = 1, CRC_MASK = 0xa23777acu;

uint32_t crc32_update(uint32_t crc, const uint8_t *p, size_t n)
{
	static uint32_t table[256];
	static bool ready = false;
	if (!ready)
	{
		for (uint32_t i = 0; i < 256; ++i)
		{
			uint32_t r = i;
			for (int j = 0; j < 8; ++j) r = (r & 1) ? (r >> 1) ^ 0xedb88320u : r >> 1;
			table[i] = r;
		}
		ready = true;
	}
	uint32_t c = ~crc;
	for (size_t i = 0; i < n; ++i) c = (c >> 8) ^ table[(c ^ p[i]) & 0xff];
	return ~c;
}

uint32_t residue(int32_t d, uint32_t p) { return d < 0 ? (uint32_t)((int64_t)d + p) : (uint32_t)d; }

bool digit_of(uint32_t r1, uint32_t r2, uint32_t r3, int32_t &d)
{
	const int64_t v = (r1 > RP1 / 2) ? (int64_t)r1 - RP1 : (int64_t)r1;
	if (v != (int32_t)v) return false;
	d = (int32_t)v;
	return residue(d, RP2) == r2 && residue(d, RP3) == r3;
}

template <typename T>
void put(std::vector<uint8_t> &b, size_t &o, T v)
{
	memcpy(b.data() + o, &v, sizeof(T));
	o += sizeof(T);
}

bool file_exists(const std::string &p)
{
	struct stat st;
	return stat(p.c_str(), &st) == 0;
}

}  // namespace

extern "C" {

size_t ctw_context_bytes(int log2_degree, int lanes, int nregs)
{
	if (log2_degree < 1 || log2_degree > 20 || lanes < 1 || nregs < 1) return 0;
	const size_t n = (size_t)nregs * ((size_t)1 << log2_degree) * (size_t)lanes;
	return 4 + 4 + 4 + 8 + n * 12 + 4;
}

// digits: [nregs][lanes][D] (the engine's register order); the file's order is
// (reg * D + j) * lanes + lane (cyclo/src/transform.h:458-468).
int ctw_context_encode(int log2_degree, int lanes, int nregs, const int32_t *digits, int k, int i, double elapsed,
                       uint8_t *out)
{
	const size_t bytes = ctw_context_bytes(log2_degree, lanes, nregs);
	if (!bytes || !digits || !out) return fail(CTW_E_ARG, "bad context arguments");
	const size_t D = (size_t)1 << log2_degree, n = (size_t)nregs * D * lanes;
	std::vector<uint8_t> b(bytes);
	size_t o = 0;
	put<uint32_t>(b, o, CTX_VERSION);
	put<int32_t>(b, o, k);
	put<int32_t>(b, o, i);
	put<double>(b, o, elapsed);
	const size_t o3 = o + n * 8;
	for (int r = 0; r < nregs; ++r)
		for (size_t j = 0; j < D; ++j)
			for (int l = 0; l < lanes; ++l)
			{
				const int32_t d = digits[((size_t)r * lanes + l) * D + j];
				const size_t idx = ((size_t)r * D + j) * lanes + l;
				const uint32_t r1 = residue(d, RP1), r2 = residue(d, RP2), r3 = residue(d, RP3);
				memcpy(b.data() + o + idx * 8, &r1, 4);
				memcpy(b.data() + o + idx * 8 + 4, &r2, 4);
				memcpy(b.data() + o3 + idx * 4, &r3, 4);
			}
	o = o3 + n * 4;
	const uint32_t trailer = ~crc32_update(0, b.data(), o) ^ CRC_MASK;
	put<uint32_t>(b, o, trailer);
	memcpy(out, b.data(), bytes);
	return CTW_OK;
}

int ctw_context_decode(int log2_degree, int lanes, int nregs, const uint8_t *in, size_t size, int32_t *digits,
                       int *k, int *i, double *elapsed)
{
	const size_t bytes = ctw_context_bytes(log2_degree, lanes, nregs);
	if (!bytes || !in || !digits) return fail(CTW_E_ARG, "bad context arguments");
	if (size != bytes) return fail(CTW_E_ARG, "invalid context: %zu bytes, expected %zu", size, bytes);
	uint32_t version, trailer;
	memcpy(&version, in, 4);
	if (version != CTX_VERSION) return fail(CTW_E_ARG, "invalid context: version %u", version);
	memcpy(&trailer, in + bytes - 4, 4);
	if (trailer != (~crc32_update(0, in, bytes - 4) ^ CRC_MASK)) return fail(CTW_E_ARG, "invalid context: bad crc32");
	int32_t kk, ii;
	double el;
	memcpy(&kk, in + 4, 4);
	memcpy(&ii, in + 8, 4);
	memcpy(&el, in + 12, 8);
	const size_t D = (size_t)1 << log2_degree, n = (size_t)nregs * D * lanes, o = 20, o3 = o + n * 8;
	for (int r = 0; r < nregs; ++r)
		for (size_t j = 0; j < D; ++j)
			for (int l = 0; l < lanes; ++l)
			{
				const size_t idx = ((size_t)r * D + j) * lanes + l;
				uint32_t r1, r2, r3;
				memcpy(&r1, in + o + idx * 8, 4);
				memcpy(&r2, in + o + idx * 8 + 4, 4);
				memcpy(&r3, in + o3 + idx * 4, 4);
				int32_t d;
				if (!digit_of(r1, r2, r3, d)) return fail(CTW_E_ARG, "invalid context: inconsistent residues");
				digits[((size_t)r * lanes + l) * D + j] = d;
			}
	if (k) *k = kk;
	if (i) *i = ii;
	if (elapsed) *elapsed = el;
	return CTW_OK;
}

}  // extern "C"

namespace {

// Geometry of a handle as the context sees it: digits per lane (D, or Dn for
// N-) and the register words per lane on the device.
struct CtxShape {
	int log2n = 0, lanes = 0;
	size_t regD = 0;
};

int ctx_shape(ctw_prp *h, CtxShape &c)
{
	int ln = 0, lanes = 0, minus = 0;
	if (int rc = ctw_prp_shape(h, &ln, &lanes, &minus)) return rc;
	c.log2n = ln;
	c.lanes = lanes;
	c.regD = (size_t)1 << (minus ? ln + 1 : ln);
	return CTW_OK;
}

int read_one(ctw_prp *h, const std::string &path, int *k, int *i, double *el)
{
	std::ifstream f(path, std::ios::binary);
	if (!f.is_open()) return 1;
	std::vector<uint8_t> buf((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
	CtxShape c;
	if (int rc = ctx_shape(h, c)) return rc;
	const size_t D = (size_t)1 << c.log2n;
	std::vector<int32_t> dig(2 * (size_t)c.lanes * D);
	if (int rc = ctw_context_decode(c.log2n, c.lanes, 2, buf.data(), buf.size(), dig.data(), k, i, el))
		return fail(rc, "%s: %s", path.c_str(), ctw_last_error());
	std::vector<int32_t> regs(2 * (size_t)c.lanes * c.regD, 0);
	for (size_t rl = 0; rl < 2 * (size_t)c.lanes; ++rl)
		memcpy(regs.data() + rl * c.regD, dig.data() + rl * D, D * 4);
	return ctw_prp_write_regs(h, 0, 2, regs.data());
}

}  // namespace

extern "C" {

int ctw_prp_save_context(ctw_prp *h, const char *path, int k, int i, double elapsed)
{
	if (!h || !path) return fail(CTW_E_ARG, "bad arguments");
	CtxShape c;
	if (int rc = ctx_shape(h, c)) return rc;
	const size_t D = (size_t)1 << c.log2n;
	std::vector<int32_t> regs(2 * (size_t)c.lanes * c.regD), dig(2 * (size_t)c.lanes * D);
	if (int rc = ctw_prp_read_regs(h, 0, 2, regs.data())) return rc;
	for (size_t rl = 0; rl < 2 * (size_t)c.lanes; ++rl) memcpy(dig.data() + rl * D, regs.data() + rl * c.regD, D * 4);
	std::vector<uint8_t> buf(ctw_context_bytes(c.log2n, c.lanes, 2));
	if (int rc = ctw_context_encode(c.log2n, c.lanes, 2, dig.data(), k, i, elapsed, buf.data())) return rc;
	// the reference's rotation (cyclo/src/cyclo.h:146-177): write .new, move the
	// current file to .old, move .new into place
	const std::string p(path), pnew = p + ".new", pold = p + ".old";
	{
		std::ofstream f(pnew, std::ios::binary | std::ios::trunc);
		if (!f.is_open() || !f.write(reinterpret_cast<const char *>(buf.data()), (std::streamsize)buf.size()))
			return fail(CTW_E_ARG, "cannot write %s", pnew.c_str());
	}
	std::remove(pold.c_str());
	if (file_exists(p) && std::rename(p.c_str(), pold.c_str()) != 0) return fail(CTW_E_ARG, "cannot save context");
	if (std::rename(pnew.c_str(), p.c_str()) != 0) return fail(CTW_E_ARG, "cannot save context");
	return CTW_OK;
}

int ctw_prp_read_context(ctw_prp *h, const char *path, int *k, int *i, double *elapsed)
{
	if (!h || !path) return fail(CTW_E_ARG, "bad arguments");
	// the file, else its .old copy (cyclo/src/cyclo.h:122-143)
	const int r1 = read_one(h, path, k, i, elapsed);
	if (r1 == 0) return 0;
	const int r2 = read_one(h, std::string(path) + ".old", k, i, elapsed);
	if (r2 == 0) return 0;
	return r1 < 0 ? r1 : r2;
}

int ctw_cyclo_check_file(int n, const char *filename, const char *workdir, int minus, double save_every_s,
                         volatile int *quit, int stop_after)
{
	if (!filename) return fail(CTW_E_ARG, "null file name");
	if (n < 8 || n > (minus ? 16 : 18)) return fail(CTW_E_ARG, "n = %d outside the supported range", n);
	const std::string dir = (workdir && *workdir) ? std::string(workdir) : std::string(".");
	const int V = 64;   // VSIZE of the reference

	// <file>.ini: CSIZE, tuned and written when absent (cyclo/src/cyclo.h:416-433)
	const std::string ini = std::string(filename) + ".ini";
	int csize = 0;
	{
		std::ifstream f(ini);
		if (f.is_open()) f >> csize;
	}
	int lg = -1;
	if (csize != 8 && csize != 16 && csize != 32 && csize != 64)
	{
		double us = 0;
		if (ctw_prp_autotune(minus ? n + 1 : n, V, &lg, &csize, &us) != CTW_OK) csize = 8;
		if (minus) lg = -1;
	}
	{
		std::ofstream f(ini);
		if (f.is_open()) f << csize << std::endl;
	}

	// candidates: one b per line, vectors of 64, the last padded (cyclo.h:216-241)
	std::vector<std::vector<uint32_t>> vecs;
	{
		std::ifstream f(filename);
		if (!f.is_open()) return fail(CTW_E_ARG, "cannot open input file %s", filename);
		std::vector<uint32_t> cur;
		std::string line;
		while (std::getline(f, line))
		{
			if (line.find_first_not_of(" \t\r") == std::string::npos) continue;
			long long v = std::stoll(line);
			if (v < 64 || v >= 0x80000000ll) return fail(CTW_E_ARG, "b = %lld outside [64, 2^31)", v);
			cur.push_back((uint32_t)v);
			if ((int)cur.size() == V)
			{
				vecs.push_back(cur);
				cur.clear();
			}
		}
		if (!cur.empty())
		{
			while ((int)cur.size() < V) cur.push_back(cur.back());
			vecs.push_back(cur);
		}
	}

	ctw_prp *h = nullptr;
	int rc = minus ? ctw_prp_create_minus(n, V, &h) : ctw_prp_create_split(n, V, lg, &h);
	if (rc) return rc;
	struct Guard { ctw_prp *h; ~Guard() { ctw_prp_destroy(h); } } guard{ h };
	if ((rc = ctw_prp_set_csize(h, csize))) return rc;

	const std::string ctx = dir + (minus ? "/cyclom.ctx" : "/cyclo.ctx");
	int rk = 0, ri = 0;
	double restored = 0;
	rc = ctw_prp_read_context(h, ctx.c_str(), &rk, &ri, &restored);
	if (rc < 0) return rc;
	const bool found = (rc == 0);
	if (found && (rk < 0 || rk >= (int)vecs.size())) return fail(CTW_E_ARG, "%s: vector %d outside the input", ctx.c_str(), rk);

	using clk = std::chrono::steady_clock;
	const auto t0 = clk::now();
	auto elapsed = [&]() { return restored + std::chrono::duration<double>(clk::now() - t0).count(); };
	auto last_save = clk::now();
	int checkpoints = 0;

	for (int k = found ? rk : 0; k < (int)vecs.size(); ++k)
	{
		const std::vector<uint32_t> &b = vecs[(size_t)k];
		struct State {
			ctw_prp *h;
			const std::string *ctx;
			int k;
			double (*el)(void *);
			void *elu;
			double save_every;
			volatile int *quit;
			int stop_after;
			int *checkpoints;
			clk::time_point *last;
			int err;
		};
		auto el_thunk = [](void *u) { return (*static_cast<decltype(elapsed) *>(u))(); };
		State st{ h, &ctx, k, el_thunk, &elapsed, save_every_s, quit, stop_after, &checkpoints, &last_save, 0 };
		auto cb = [](void *user, long long i) -> int {
			State &s = *static_cast<State *>(user);
			++*s.checkpoints;
			const bool stop = (s.quit && *s.quit) || (s.stop_after > 0 && *s.checkpoints >= s.stop_after);
			const double since = std::chrono::duration<double>(clk::now() - *s.last).count();
			if (stop || (s.save_every > 0 && since >= s.save_every))
			{
				s.err = ctw_prp_save_context(s.h, s.ctx->c_str(), s.k, (int)i, s.el(s.elu));
				*s.last = clk::now();
				if (s.err) return 1;
			}
			return stop ? 1 : 0;
		};
		std::vector<uint8_t> prp(V), ok(V);
		std::vector<uint64_t> r64(V);
		const long long i_start = (found && k == rk) ? (long long)ri : -1;
		rc = ctw_prp_run_ex(h, b.data(), V, i_start, cb, &st, prp.data(), r64.data(), ok.data());
		if (st.err) return st.err;
		if (rc == CTW_STOPPED) return CTW_STOPPED;
		if (rc) return rc;

		// result lines (cyclo/src/cyclo.h:379-408), duplicates of the padding skipped
		std::ostringstream ss, sp;
		const char *sign = minus ? " - 1 is " : " + 1 is ";
		for (int l = 0; l < V; ++l)
		{
			if (l > 0 && b[(size_t)l] == b[(size_t)l - 1]) continue;
			ss << b[(size_t)l] << "^" << (1 << n) << " - " << b[(size_t)l] << "^" << (1 << (n - 1)) << sign;
			if (prp[(size_t)l]) ss << "a probable prime.";
			else
			{
				char hex[20];
				snprintf(hex, sizeof(hex), "%016llX", (unsigned long long)r64[(size_t)l]);
				ss << "composite. RES64: " << hex;
			}
			ss << "\n";
			if (prp[(size_t)l]) sp << b[(size_t)l] << "\n";
		}
		{
			std::ofstream f(dir + "/result_c.txt", std::ios::app);
			if (!f.is_open() || !(f << ss.str())) return fail(CTW_E_ARG, "cannot write result_c.txt");
		}
		if (!sp.str().empty())
		{
			std::ostringstream fn;
			fn << dir << (minus ? "/prpm_" : "/prp_") << n << ".txt";
			std::ofstream f(fn.str(), std::ios::app);
			if (!f.is_open() || !(f << sp.str())) return fail(CTW_E_ARG, "cannot write %s", fn.str().c_str());
		}
	}
	// all vectors done: the context is spent
	std::remove(ctx.c_str());
	std::remove((ctx + ".old").c_str());
	return CTW_OK;
}

}  // extern "C"
