// Host side of the PRP engine: root tables, launches, canonical digits,
// RES64 and the Gerbicz-Li driver, behind the C ABI of include/ctwin_gb300.h.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/ctwin_gb300.h"
#include "bignum.h"
#include "prp_arith.cuh"
#include "prp_kernels.cuh"
#include "prp_host.h"
#include "prp_tables.h"

namespace ctw {

thread_local std::string g_last_error;

int fail(int code, const char *fmt, ...)
{
	char buf[512];
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(buf, sizeof(buf), fmt, ap);
	va_end(ap);
	g_last_error = buf;
	return code;
}

#define CTW_CUDA(call)                                                                                       \
	do {                                                                                                     \
		cudaError_t e_ = (call);                                                                             \
		if (e_ != cudaSuccess) return fail(CTW_E_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_),     \
		                                   __FILE__, __LINE__);                                              \
	} while (0)

// Canonical digits of x mod N = b^D - b^{D/2} + 1 (cyclo/src/transform.h:501-597):
// carry the signed digits base b, fold the top carry T as -T at 0 and +T at
// D/2 (b^D = b^{D/2} - 1 mod N) until it vanishes, then subtract N once if the
// value is >= N.
int canonical(const int32_t *x, uint32_t b, size_t D, uint32_t *out)
{
	const int64_t B = b;
	auto divmod = [B](int64_t &v) -> uint32_t {
		int64_t q = v / B, r = v % B;
		if (r < 0) { r += B; --q; }
		v = q;
		return (uint32_t)r;
	};
	int64_t c = 0;
	for (size_t j = 0; j < D; ++j)
	{
		int64_t v = c + x[j];
		out[j] = divmod(v);
		c = v;
	}
	for (int guard = 0; c != 0; ++guard)
	{
		if (guard > 64) return fail(CTW_E_COMPUTE, "getInt: carry does not settle");
		int64_t v = -c;
		for (size_t j = 0; j < D / 2; ++j) { v += out[j]; out[j] = divmod(v); }
		v += c;
		for (size_t j = D / 2; j < D; ++j) { v += out[j]; out[j] = divmod(v); if (v == 0) break; }
		c = v;
	}
	bool ge = true;
	for (size_t j = D / 2; j < D; ++j) if (out[j] != b - 1) { ge = false; break; }
	if (ge)
	{
		bool low_zero = true;
		for (size_t j = 0; j < D / 2; ++j) if (out[j] != 0) { low_zero = false; break; }
		ge = !low_zero;
	}
	if (ge)
	{
		// value - N: lower half minus 1, upper half cleared
		size_t j = 0;
		while (j < D / 2 && out[j] == 0) { out[j] = b - 1; ++j; }
		if (j == D / 2) return fail(CTW_E_COMPUTE, "getInt failed");
		out[j] -= 1;
		for (size_t k = D / 2; k < D; ++k) out[k] = 0;
	}
	return CTW_OK;
}

// Canonical digits of x mod N- = b^Dn - b^{Dn/2} - 1 (the twin partner,
// sieve/CPU/ctsieve.cpp:434-439): carry base b, fold the top carry T as +T at
// 0 and +T at Dn/2 (b^Dn = b^{Dn/2} + 1 mod N-) until it vanishes, then
// subtract N- once if the value is >= N-.
int canonical_minus(const int32_t *x, uint32_t b, size_t Dn, uint32_t *out)
{
	const int64_t B = b;
	auto divmod = [B](int64_t &v) -> uint32_t {
		int64_t q = v / B, r = v % B;
		if (r < 0) { r += B; --q; }
		v = q;
		return (uint32_t)r;
	};
	int64_t c = 0;
	for (size_t j = 0; j < Dn; ++j)
	{
		int64_t v = c + x[j];
		out[j] = divmod(v);
		c = v;
	}
	for (int guard = 0; c != 0; ++guard)
	{
		if (guard > 64) return fail(CTW_E_COMPUTE, "getInt: carry does not settle");
		int64_t v = c;
		for (size_t j = 0; j < Dn / 2; ++j) { v += out[j]; out[j] = divmod(v); }
		v += c;
		for (size_t j = Dn / 2; j < Dn; ++j) { v += out[j]; out[j] = divmod(v); }
		c = v;
	}
	// N- digits: b-1 below Dn/2, b-2 at Dn/2, b-1 above
	auto ndig = [&](size_t j) -> uint32_t { return j == Dn / 2 ? b - 2 : b - 1; };
	bool ge = true;
	for (size_t j = Dn; j-- > 0;)
		if (out[j] != ndig(j)) { ge = out[j] > ndig(j); break; }
	if (ge)
	{
		int64_t borrow = 0;
		for (size_t j = 0; j < Dn; ++j)
		{
			int64_t v = (int64_t)out[j] - ndig(j) - borrow;
			borrow = v < 0;
			if (v < 0) v += B;
			out[j] = (uint32_t)v;
		}
	}
	return CTW_OK;
}

void res64_of(const uint32_t *c, uint32_t b, size_t D, bool &prp, bool &zero, uint64_t &r64)
{
	prp = (c[0] == 1);
	zero = (c[0] == 0);
	uint64_t r = c[0], bp = b;
	for (size_t j = 1; j < D; ++j)
	{
		prp &= (c[j] == 0);
		zero &= (c[j] == 0);
		r += (uint64_t)c[j] * bp;
		bp *= b;
	}
	r64 = r;
}

}  // namespace ctw

using namespace ctw;

struct ctw_prp {
	int ln = 0, lanes = 0, lg = 0, lm = 0, csize = 8;
	uint32_t base = 2;
	size_t D = 0, M = 0, G = 1;
	int threads = 0;
	size_t smem = 0;
	int tw_smem = 0;
	int narrow = 0;                   // 64-bit carry arithmetic is exact for the current b
	int nprime = 3;                   // NTT primes of the launches (2 when exact for the current b)
	int prime_mode = 0;               // 0: two primes whenever exact; 3: always three
	uint32_t bmax = 0;                // largest b of the lanes
	int minus = 0;                    // N- = b^Dn - b^{Dn/2} - 1 on the transform of degree D = 2 Dn
	size_t Dn = 0;                    // degree of the tested numbers (D, or D/2 for N-)
	cudaStream_t stream = nullptr;
	int32_t *d_regs = nullptr;        // [3][lanes][D]
	uint32_t *d_scratch = nullptr;    // [lanes][G][3][M]
	uint32_t *d_tf = nullptr, *d_ti = nullptr;
	uint32_t *d_tfs = nullptr, *d_tis = nullptr;
	uint32_t *d_laneb = nullptr;      // [lanes][4]
	uint32_t *d_bits = nullptr;
	size_t bits_cap = 0;
	uint32_t *d_exp = nullptr;        // resident exponent words [lanes][exp_nwords]
	int exp_nwords = 0;
	uint32_t *d_status = nullptr;
	int grid = 0;                     // 1: grid kernel (2^lg CTAs of one cooperative launch per lane)
	uint32_t *d_gx = nullptr, *d_gr = nullptr, *d_xr = nullptr;
	long long *d_gc = nullptr;
	unsigned *d_bar = nullptr;
	int bar_unreachable = 0;          // testing: the next grid launch starts its barrier out of reach
	std::vector<uint32_t> b;
	PrpKernelArgs proto{};
	long long launches = 0;

	int32_t *reg(int r) const { return d_regs + (size_t)r * lanes * D; }
};

namespace {

int check_handle(ctw_prp *h)
{
	if (!h) return fail(CTW_E_ARG, "null handle");
	return CTW_OK;
}

// Launch shape of the handle's split: CTAs, coefficients per CTA, shared memory.
void set_shape(ctw_prp *h)
{
	h->lm = h->ln - h->lg;
	h->G = (size_t)1 << h->lg;
	h->M = h->D / h->G;
	if (h->grid)
	{
		h->tw_smem = prp_grid_smem_bytes(h->lg, h->lm, 1, 3) <= 227 * 1024 ? 1 : 0;
		h->smem = prp_grid_smem_bytes(h->lg, h->lm, h->tw_smem, 3);
		h->threads = prp_grid_threads(h->lm, 3);
	}
	else
	{
		h->tw_smem = prp_smem_bytes(h->lm, h->lg, 1) <= 227 * 1024 ? 1 : 0;
		h->smem = prp_smem_bytes(h->lm, h->lg, h->tw_smem);
		h->threads = prp_threads(h->lm, 3, h->lg);
	}
}

// Exchange buffers of a grid split.
int alloc_grid(ctw_prp *h)
{
	if (!h->grid) return CTW_OK;
	const size_t xw = (size_t)h->lanes * 3 * h->D;        // [lanes][G][3][M] words
	if (cudaMalloc(&h->d_gx, xw * 4) != cudaSuccess || cudaMalloc(&h->d_gr, xw * 4) != cudaSuccess ||
	    cudaMalloc(&h->d_gc, (size_t)h->lanes * h->G * h->G * sizeof(long long)) != cudaSuccess ||
	    cudaMalloc(&h->d_bar, (size_t)h->lanes * GRID_BAR_WORDS * sizeof(unsigned)) != cudaSuccess)
		return fail(CTW_E_NOMEM, "grid exchange buffers");
	CTW_CUDA(cudaMemset(h->d_bar, 0, (size_t)h->lanes * GRID_BAR_WORDS * sizeof(unsigned)));
	return CTW_OK;
}

int build_tables(ctw_prp *h);
void choose_primes(ctw_prp *h);

// Change the split of a handle; the registers keep their natural digit order in
// HBM, so their contents carry over.  The new shape's buffers are made first:
// on failure the handle keeps its old split.
int reshape(ctw_prp *h, int lg, bool grid)
{
	CTW_CUDA(cudaStreamSynchronize(h->stream));
	ctw_prp old = *h;                    // shape, tables and buffers in use
	h->d_tf = h->d_ti = h->d_tfs = h->d_tis = h->d_xr = h->d_gx = h->d_gr = nullptr;
	h->d_gc = nullptr;
	h->d_bar = nullptr;
	h->grid = grid ? 1 : 0;
	h->lg = lg;
	set_shape(h);
	int rc = alloc_grid(h);
	if (!rc) rc = build_tables(h);
	auto release = [](ctw_prp &x) {
		cudaFree(x.d_tf);
		cudaFree(x.d_ti);
		cudaFree(x.d_tfs);
		cudaFree(x.d_tis);
		cudaFree(x.d_xr);
		cudaFree(x.d_gx);
		cudaFree(x.d_gr);
		cudaFree(x.d_gc);
		cudaFree(x.d_bar);
	};
	if (rc)
	{
		release(*h);
		h->grid = old.grid;
		h->lg = old.lg;
		h->proto = old.proto;
		set_shape(h);
		h->d_tf = old.d_tf;
		h->d_ti = old.d_ti;
		h->d_tfs = old.d_tfs;
		h->d_tis = old.d_tis;
		h->d_xr = old.d_xr;
		h->d_gx = old.d_gx;
		h->d_gr = old.d_gr;
		h->d_gc = old.d_gc;
		h->d_bar = old.d_bar;
		return rc;
	}
	release(old);
	choose_primes(h);
	return CTW_OK;
}

// Root tables and launch constants (prp_tables.h), uploaded once per handle.
int build_tables(ctw_prp *h)
{
	const size_t words = h->G * 3 * h->M, swords = h->G * 3 * 256 * 2;
	std::vector<uint32_t> tf(words), ti(words), tfs(swords), tis(swords), xr(3 * 2 * 128);
	prp_build_tables(h->ln, h->lg, tf.data(), ti.data(), h->proto, tfs.data(), tis.data(), xr.data());
	// the grid kernel of 1024- and 2048-coefficient CTAs lays its local roots out
	// per sub-block, as Shoup pairs
	if (h->grid && h->lm <= 11)
	{
		tf.assign(2 * words, 0);
		ti.assign(2 * words, 0);
		prp_build_grid2_tables(h->ln, h->lg, tf.data(), ti.data());
	}
	const size_t bytes = tf.size() * sizeof(uint32_t);
	if (h->grid)
	{
		CTW_CUDA(cudaMalloc(&h->d_xr, xr.size() * 4));
		CTW_CUDA(cudaMemcpy(h->d_xr, xr.data(), xr.size() * 4, cudaMemcpyHostToDevice));
	}
	CTW_CUDA(cudaMalloc(&h->d_tf, bytes));
	CTW_CUDA(cudaMalloc(&h->d_ti, bytes));
	CTW_CUDA(cudaMemcpy(h->d_tf, tf.data(), bytes, cudaMemcpyHostToDevice));
	CTW_CUDA(cudaMemcpy(h->d_ti, ti.data(), bytes, cudaMemcpyHostToDevice));
	if (h->lm == 12)
	{
		CTW_CUDA(cudaMalloc(&h->d_tfs, swords * 4));
		CTW_CUDA(cudaMalloc(&h->d_tis, swords * 4));
		CTW_CUDA(cudaMemcpy(h->d_tfs, tfs.data(), swords * 4, cudaMemcpyHostToDevice));
		CTW_CUDA(cudaMemcpy(h->d_tis, tis.data(), swords * 4, cudaMemcpyHostToDevice));
	}
	return CTW_OK;
}

PrpKernelArgs make_args(ctw_prp *h)
{
	PrpKernelArgs a = h->proto;
	a.tf = h->d_tf;
	a.ti = h->d_ti;
	a.tfs = h->d_tfs;
	a.tis = h->d_tis;
	a.lane_b = h->d_laneb;
	a.status = h->d_status;
	a.lm = h->lm;
	a.csize = h->csize;
	a.mult = (int)h->base;
	a.tw_smem = h->tw_smem;
	a.narrow = h->narrow;
	a.minus = h->minus;
	a.nprime = h->nprime;
	a.scratch = h->d_scratch;
	return a;
}

// Two NTT primes when the split has a two-prime kernel and the product of two
// residues stays exact with them for every lane's b (prp_two_primes_exact).
void choose_primes(ctw_prp *h)
{
	const double terms = h->minus ? (double)h->Dn : 1.5 * (double)h->D;
	h->nprime = (h->prime_mode != 3 && h->bmax > 0 && (h->grid || prp_two_prime_split(h->lm, h->lg)) &&
	             prp_two_primes_exact(terms, h->bmax)) ? 2 : 3;
}

int launch(ctw_prp *h, const PrpKernelArgs &a)
{
	cudaError_t e;
	if (h->grid)
	{
		// barrier counters and the published columns and rows (whose words carry
		// the parity of their publication in the launch) start at zero
		const size_t xw = (size_t)h->lanes * 3 * h->D;
		e = cudaMemsetAsync(h->d_bar, 0, (size_t)h->lanes * GRID_BAR_WORDS * sizeof(unsigned), h->stream);
		if (e == cudaSuccess) e = cudaMemsetAsync(h->d_gx, 0, xw * 4, h->stream);
		if (e == cudaSuccess) e = cudaMemsetAsync(h->d_gr, 0, xw * 4, h->stream);
		// testing only (ctw_prp_test_unreachable_barrier): word 0 of every lane
		// starts at 0x80808080, 2^31 arrivals short of any target this launch
		// sets, and CTA 0 skips its first publication of columns
		for (int l = 0; e == cudaSuccess && h->bar_unreachable && l < h->lanes; ++l)
			e = cudaMemsetAsync(h->d_bar + (size_t)l * GRID_BAR_WORDS, 0x80, sizeof(unsigned), h->stream);
		const int mute = h->bar_unreachable ? 1 : 0;
		h->bar_unreachable = 0;
		if (e == cudaSuccess)
		{
			const PrpGridArgs ga{ h->d_gx, h->d_gr, h->d_gc, h->d_bar, h->d_xr, mute };
			e = prp_grid_launch(a, ga, h->lg, h->lanes, h->stream);
		}
	}
	else
		e = prp_launch(a, h->lg, h->lanes, h->stream);
	if (e != cudaSuccess) return fail(CTW_E_CUDA, "PRP kernel launch: %s", cudaGetErrorString(e));
	++h->launches;
	return CTW_OK;
}

int ensure_bits(ctw_prp *h, size_t words)
{
	if (words <= h->bits_cap) return CTW_OK;
	if (h->d_bits) cudaFree(h->d_bits);
	h->d_bits = nullptr;
	h->bits_cap = 0;
	CTW_CUDA(cudaMalloc(&h->d_bits, words * sizeof(uint32_t)));
	h->bits_cap = words;
	return CTW_OK;
}

int check_status(ctw_prp *h)
{
	uint32_t st = 0;
	CTW_CUDA(cudaMemcpyAsync(&st, h->d_status, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
	CTW_CUDA(cudaStreamSynchronize(h->stream));
	if (st != 0)
	{
		cudaMemsetAsync(h->d_status, 0, sizeof(uint32_t), h->stream);
		if (st & ST_GRID_WAIT)
			return fail(CTW_E_COMPUTE,
			            "grid kernel: a wait for other CTAs (grid barrier or published words) ran out, the launch's "
			            "results are void (status 0x%x)", st);
		return fail(CTW_E_COMPUTE, "device arithmetic range check failed (status 0x%x)", st);
	}
	return CTW_OK;
}

int read_reg_host(ctw_prp *h, int reg, std::vector<int32_t> &v)
{
	v.resize((size_t)h->lanes * h->D);
	CTW_CUDA(cudaMemcpyAsync(v.data(), h->reg(reg), v.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
	CTW_CUDA(cudaStreamSynchronize(h->stream));
	return CTW_OK;
}

int canonical_reg(ctw_prp *h, int reg, std::vector<uint32_t> &c)
{
	std::vector<int32_t> v;
	int rc = check_status(h);
	if (rc) return rc;
	if ((rc = read_reg_host(h, reg, v))) return rc;
	c.resize((size_t)h->lanes * h->Dn);
	for (int l = 0; l < h->lanes; ++l)
	{
		const int32_t *x = v.data() + (size_t)l * h->D;
		uint32_t *o = c.data() + (size_t)l * h->Dn;
		rc = h->minus ? canonical_minus(x, h->b[(size_t)l], h->Dn, o) : canonical(x, h->b[(size_t)l], h->D, o);
		if (rc) return rc;
	}
	return CTW_OK;
}

int op_square_bits(ctw_prp *h, const uint32_t *d_bits, int nwords, long long i_hi, int count)
{
	PrpKernelArgs a = make_args(h);
	a.op = OP_SQUARE;
	a.reg_in = h->reg(0);
	a.reg_out = h->reg(0);
	a.bits = d_bits;
	a.nwords = nwords;
	a.i_hi = i_hi;
	a.count = count;
	a.use_dupmask = 0;
	return launch(h, a);
}

int op_mul(ctw_prp *h, int out, int x, int y)
{
	PrpKernelArgs a = make_args(h);
	a.op = OP_MUL;
	a.reg_in = h->reg(x);
	a.reg_y = h->reg(y);
	a.reg_out = h->reg(out);
	a.count = 1;
	return launch(h, a);
}

int op_set(ctw_prp *h, int reg, uint32_t v)
{
	const size_t n = (size_t)h->lanes * h->D;
	CTW_CUDA(cudaMemsetAsync(h->reg(reg), 0, n * sizeof(int32_t), h->stream));
	if (v != 0)
	{
		// coefficient 0 of every lane; a strided 2D copy of one int32 per lane
		static thread_local std::vector<int32_t> one;
		one.assign((size_t)h->lanes, (int32_t)v);
		CTW_CUDA(cudaMemcpy2DAsync(h->reg(reg), h->D * sizeof(int32_t), one.data(), sizeof(int32_t), sizeof(int32_t),
		                           (size_t)h->lanes, cudaMemcpyHostToDevice, h->stream));
		CTW_CUDA(cudaStreamSynchronize(h->stream));
	}
	return CTW_OK;
}

}  // namespace

extern "C" {

const char *ctw_last_error(void) { return g_last_error.c_str(); }
const char *ctw_version(void) { return "ctwin_gb300 0.1 (sm_103a)"; }
int ctw_device_count(void)
{
	int n = 0;
	if (cudaGetDeviceCount(&n) != cudaSuccess) { cudaGetLastError(); return 0; }
	return n;
}

int ctw_prp_create(int log2_degree, int lanes, ctw_prp **out)
{
	return ctw_prp_create_split(log2_degree, lanes, -1, out);
}

int ctw_prp_create_minus(int log2_degree, int lanes, ctw_prp **out)
{
	if (!out) return fail(CTW_E_ARG, "null output pointer");
	*out = nullptr;
	if (log2_degree < 8 || log2_degree > 16) return fail(CTW_E_ARG, "N- log2_degree %d outside [8, 16]", log2_degree);
	// the product of two degree < Dn polynomials is exact on the transform of
	// degree 2 Dn; one CTA up to 2^12 coefficients, else a column-layout
	// cluster of >= 4 CTAs (the fold stays inside each CTA's columns)
	const int ln2 = log2_degree + 1;
	const int lg = ln2 <= 12 ? 0 : std::max(2, prp_lg_for(ln2));
	ctw_prp *h = nullptr;
	if (int rc = ctw_prp_create_split(ln2, lanes, lg, &h)) return rc;
	h->minus = 1;
	h->Dn = h->D / 2;
	*out = h;
	return CTW_OK;
}

int ctw_prp_create_split(int log2_degree, int lanes, int log2_ctas, ctw_prp **out)
{
	if (!out) return fail(CTW_E_ARG, "null output pointer");
	*out = nullptr;
	if (log2_degree < 8 || log2_degree > 18) return fail(CTW_E_ARG, "log2_degree %d outside [8, 18]", log2_degree);
	if (lanes < 1 || lanes > MAX_INLINE_LANES) return fail(CTW_E_ARG, "lanes %d outside [1, %d]", lanes, MAX_INLINE_LANES);
	// an explicit split must have a kernel (host-only check, before the device is asked)
	if (log2_ctas >= 0 && !(log2_ctas > MAX_LG ? prp_grid_supported(log2_ctas, log2_degree - log2_ctas)
	                                            : prp_split_supported(log2_degree - log2_ctas, log2_ctas)))
		return fail(CTW_E_ARG, "no kernel for degree 2^%d on 2^%d CTAs", log2_degree, log2_ctas);
	if (ctw_device_count() == 0) return fail(CTW_E_CUDA, "no CUDA device");
	// Degrees 2^16..2^18 default to the grid kernel with the most CTAs per lane
	// that has a kernel (2^16: 64 of 1024 coefficients, 2^17: 64 of 2048, 2^18:
	// 128 of 2048, else 64 of 4096) when the lanes fit in one cooperative launch,
	// else to 16-CTA clusters.
	int lg = log2_ctas < 0 ? prp_lg_for(log2_degree) : log2_ctas;
	bool grid = false;
	if (log2_ctas < 0 && log2_degree >= 16)
	{
		for (int lm = 10; lm <= 12 && !grid; ++lm)
			if (prp_grid_supported(log2_degree - lm, lm) && lanes <= prp_grid_max_lanes(log2_degree - lm, lm, 3))
			{
				lg = log2_degree - lm;
				grid = true;
			}
		if (!grid && !prp_split_supported(log2_degree - lg, lg))
			return fail(CTW_E_ARG, "no kernel for degree 2^%d on 2^%d CTAs", log2_degree, lg);
	}
	else if (log2_ctas > MAX_LG)
	{
		if (!prp_grid_supported(lg, log2_degree - lg))
			return fail(CTW_E_ARG, "no kernel for degree 2^%d on 2^%d CTAs", log2_degree, lg);
		const int cap = prp_grid_max_lanes(lg, log2_degree - lg, 3);
		if (lanes > cap) return fail(CTW_E_ARG, "%d lanes of degree 2^%d exceed one grid launch (%d)", lanes, log2_degree, cap);
		grid = true;
	}
	else if (!prp_split_supported(log2_degree - lg, lg))
		return fail(CTW_E_ARG, "no kernel for degree 2^%d on 2^%d CTAs", log2_degree, lg);
	ctw_prp *h = new ctw_prp();
	h->ln = log2_degree;
	h->lanes = lanes;
	h->grid = grid ? 1 : 0;
	h->lg = lg;
	h->lm = log2_degree - h->lg;
	h->D = (size_t)1 << log2_degree;
	h->Dn = h->D;
	set_shape(h);
	h->b.assign((size_t)lanes, 0);
	int rc = CTW_OK;
	auto cleanup = [&](int code) { ctw_prp_destroy(h); return code; };
	if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
		return cleanup(fail(CTW_E_CUDA, "stream creation failed"));
	const size_t rbytes = 3 * (size_t)lanes * h->D * sizeof(int32_t);
	if (cudaMalloc(&h->d_regs, rbytes) != cudaSuccess) return cleanup(fail(CTW_E_NOMEM, "register allocation"));
	if (cudaMalloc(&h->d_scratch, (size_t)lanes * h->D * 3 * sizeof(uint32_t)) != cudaSuccess)
		return cleanup(fail(CTW_E_NOMEM, "scratch allocation"));
	if (cudaMalloc(&h->d_laneb, (size_t)lanes * 4 * sizeof(uint32_t)) != cudaSuccess)
		return cleanup(fail(CTW_E_NOMEM, "lane allocation"));
	if (cudaMalloc(&h->d_status, sizeof(uint32_t)) != cudaSuccess) return cleanup(fail(CTW_E_NOMEM, "status"));
	if ((rc = alloc_grid(h))) return cleanup(rc);
	cudaMemset(h->d_regs, 0, rbytes);
	cudaMemset(h->d_status, 0, sizeof(uint32_t));
	cudaMemset(h->d_laneb, 0, (size_t)lanes * 4 * sizeof(uint32_t));
	if ((rc = build_tables(h))) return cleanup(rc);
	if (cudaDeviceSynchronize() != cudaSuccess) return cleanup(fail(CTW_E_CUDA, "device init failed"));
	*out = h;
	return CTW_OK;
}

int ctw_prp_destroy(ctw_prp *h)
{
	if (!h) return CTW_OK;
	if (h->stream) cudaStreamSynchronize(h->stream);
	cudaFree(h->d_regs);
	cudaFree(h->d_scratch);
	cudaFree(h->d_tf);
	cudaFree(h->d_ti);
	cudaFree(h->d_tfs);
	cudaFree(h->d_tis);
	cudaFree(h->d_laneb);
	cudaFree(h->d_bits);
	cudaFree(h->d_exp);
	cudaFree(h->d_status);
	cudaFree(h->d_gx);
	cudaFree(h->d_gr);
	cudaFree(h->d_gc);
	cudaFree(h->d_bar);
	cudaFree(h->d_xr);
	if (h->stream) cudaStreamDestroy(h->stream);
	delete h;
	return CTW_OK;
}

int ctw_prp_set_csize(ctw_prp *h, int csize)
{
	if (int rc = check_handle(h)) return rc;
	if (csize != 8 && csize != 16 && csize != 32 && csize != 64) return fail(CTW_E_ARG, "csize %d not in {8,16,32,64}", csize);
	if (h->grid && (size_t)csize > (h->M >> h->lg))
	{
		// a grid shape of this degree with column runs of at least csize, else
		// the 16-CTA cluster split
		int to_lg = -1;
		bool to_grid = false;
		for (int lm = h->lm + 1; lm <= 12 && to_lg < 0; ++lm)
		{
			const int lg = h->ln - lm;
			if (prp_grid_supported(lg, lm) && h->lanes <= prp_grid_max_lanes(lg, lm, 3) &&
			    (size_t)csize <= (((size_t)1 << lm) >> lg))
			{
				to_lg = lg;
				to_grid = true;
			}
		}
		if (to_lg < 0) to_lg = prp_lg_for(h->ln);
		if (int rc = reshape(h, to_lg, to_grid)) return rc;
	}
	if ((size_t)csize * 2 > h->M) return fail(CTW_E_ARG, "csize too large for this degree");
	if (h->lg > 0 && h->lm <= 13 && (size_t)csize > (h->M >> h->lg))
		return fail(CTW_E_ARG, "csize %d longer than a column run of this split", csize);
	if (h->minus && h->lg == 0 && (size_t)csize * 4 > h->M) return fail(CTW_E_ARG, "csize too large for this degree");
	h->csize = csize;
	return CTW_OK;
}

int ctw_prp_set_base(ctw_prp *h, uint32_t base)
{
	if (int rc = check_handle(h)) return rc;
	if (base != 2 && base != 3) return fail(CTW_E_ARG, "base %u not in {2,3}", base);
	h->base = base;
	return CTW_OK;
}

int ctw_prp_set_b(ctw_prp *h, const uint32_t *b, int count)
{
	if (int rc = check_handle(h)) return rc;
	if (!b || count != h->lanes) return fail(CTW_E_ARG, "set_b expects lanes (%d) values", h->lanes);
	std::vector<uint32_t> lb((size_t)h->lanes * 4);
	uint32_t bmax = 0;
	for (int l = 0; l < h->lanes; ++l)
	{
		bmax = std::max(bmax, b[l]);
		const uint32_t bl = b[l];
		if (bl < 64 || bl >= 0x80000000u) return fail(CTW_E_ARG, "b = %u outside [64, 2^31)", bl);
		const int s = (31 - __builtin_clz(bl)) - 1;
		lb[4 * l + 0] = bl;
		lb[4 * l + 1] = (uint32_t)(((uint64_t)1 << (s + 32)) / bl);
		lb[4 * l + 2] = (uint32_t)s;
		lb[4 * l + 3] = 0;
		h->b[(size_t)l] = bl;
	}
	// |coefficient| <= 1.5 D b^2, accumulated x3 plus carries: 64-bit when 8 D b^2 < 2^62
	h->narrow = (8.0 * (double)h->D * (double)bmax * (double)bmax < 4.611686018427388e18) ? 1 : 0;
	h->bmax = bmax;
	choose_primes(h);
	CTW_CUDA(cudaMemcpyAsync(h->d_laneb, lb.data(), lb.size() * 4, cudaMemcpyHostToDevice, h->stream));
	CTW_CUDA(cudaStreamSynchronize(h->stream));
	return CTW_OK;
}

int ctw_prp_two_primes(int log2_degree, int minus, uint32_t b)
{
	if (minus ? (log2_degree < 8 || log2_degree > 16) : (log2_degree < 8 || log2_degree > 18)) return 0;
	const int ln = minus ? log2_degree + 1 : log2_degree;
	const int lg = minus ? (ln <= 12 ? 0 : std::max(2, prp_lg_for(ln))) : prp_lg_for(ln);
	const double Dn = (double)((size_t)1 << log2_degree);
	// one N+ candidate of degree 2^17 or 2^18 runs on the grid kernel, which has both
	const bool split = prp_two_prime_split(ln - lg, lg) || (!minus && prp_grid_supported(ln - 12, 12));
	return (split && prp_two_primes_exact(minus ? Dn : 1.5 * Dn, b)) ? 1 : 0;
}

int ctw_prp_set_prime_count(ctw_prp *h, int count)
{
	if (int rc = check_handle(h)) return rc;
	if (count != 0 && count != 3) return fail(CTW_E_ARG, "prime count %d not in {0 (automatic), 3}", count);
	h->prime_mode = count;
	choose_primes(h);
	return CTW_OK;
}

int ctw_prp_prime_count(ctw_prp *h) { return h ? h->nprime : 0; }

int ctw_prp_set(ctw_prp *h, uint32_t a)
{
	if (int rc = check_handle(h)) return rc;
	return op_set(h, 0, a);
}

int ctw_prp_copy(ctw_prp *h, int dst, int src)
{
	if (int rc = check_handle(h)) return rc;
	if (dst < 0 || dst > 2 || src < 0 || src > 2) return fail(CTW_E_ARG, "register index outside 0..2");
	if (dst == src) return CTW_OK;
	CTW_CUDA(cudaMemcpyAsync(h->reg(dst), h->reg(src), (size_t)h->lanes * h->D * sizeof(int32_t),
	                         cudaMemcpyDeviceToDevice, h->stream));
	return CTW_OK;
}

int ctw_prp_square_dup(ctw_prp *h, const uint64_t *mask)
{
	if (int rc = check_handle(h)) return rc;
	PrpKernelArgs a = make_args(h);
	a.op = OP_SQUARE;
	a.reg_in = h->reg(0);
	a.reg_out = h->reg(0);
	a.count = 1;
	a.i_hi = 0;
	a.use_dupmask = 1;
	const int nw = (h->lanes + 63) / 64;
	for (int w = 0; w < nw; ++w) a.dupmask[w] = mask ? mask[w] : 0;
	return launch(h, a);
}

int ctw_prp_mul(ctw_prp *h)
{
	if (int rc = check_handle(h)) return rc;
	return op_mul(h, 0, 0, 1);
}

int ctw_prp_mul_regs(ctw_prp *h, int reg_out, int reg_a, int reg_b)
{
	if (int rc = check_handle(h)) return rc;
	if (reg_out < 0 || reg_out > 2 || reg_a < 0 || reg_a > 2 || reg_b < 0 || reg_b > 2)
		return fail(CTW_E_ARG, "register index outside 0..2");
	return op_mul(h, reg_out, reg_a, reg_b);
}

int ctw_prp_square_bits(ctw_prp *h, const uint32_t *e_words, int nwords, long long i_hi, int count)
{
	if (int rc = check_handle(h)) return rc;
	if (!e_words || nwords < 1 || count < 0) return fail(CTW_E_ARG, "bad exponent arguments");
	if (count == 0) return CTW_OK;
	const size_t words = (size_t)h->lanes * nwords;
	if (int rc = ensure_bits(h, words)) return rc;
	CTW_CUDA(cudaMemcpyAsync(h->d_bits, e_words, words * 4, cudaMemcpyHostToDevice, h->stream));
	CTW_CUDA(cudaStreamSynchronize(h->stream));   // e_words may be reused by the caller
	return op_square_bits(h, h->d_bits, nwords, i_hi, count);
}

int ctw_prp_load_exponent(ctw_prp *h, const uint32_t *e_words, int nwords)
{
	if (int rc = check_handle(h)) return rc;
	if (!e_words || nwords < 1) return fail(CTW_E_ARG, "bad exponent arguments");
	const size_t words = (size_t)h->lanes * nwords;
	CTW_CUDA(cudaStreamSynchronize(h->stream));
	cudaFree(h->d_exp);
	h->d_exp = nullptr;
	h->exp_nwords = 0;
	CTW_CUDA(cudaMalloc(&h->d_exp, words * 4));
	CTW_CUDA(cudaMemcpy(h->d_exp, e_words, words * 4, cudaMemcpyHostToDevice));
	h->exp_nwords = nwords;
	return CTW_OK;
}

int ctw_prp_square_resident(ctw_prp *h, long long i_hi, int count)
{
	if (int rc = check_handle(h)) return rc;
	if (!h->d_exp) return fail(CTW_E_ARG, "no resident exponent (ctw_prp_load_exponent)");
	if (count < 0) return fail(CTW_E_ARG, "negative count");
	if (count == 0) return CTW_OK;
	return op_square_bits(h, h->d_exp, h->exp_nwords, i_hi, count);
}

int ctw_prp_get_digits(ctw_prp *h, int reg, uint32_t *out)
{
	if (int rc = check_handle(h)) return rc;
	if (!out || reg < 0 || reg > 2) return fail(CTW_E_ARG, "bad arguments");
	std::vector<uint32_t> c;
	if (int rc = canonical_reg(h, reg, c)) return rc;
	memcpy(out, c.data(), c.size() * sizeof(uint32_t));
	return CTW_OK;
}

int ctw_prp_is_prime(ctw_prp *h, int reg, uint8_t *is_prp, uint64_t *res64)
{
	if (int rc = check_handle(h)) return rc;
	if (reg < 0 || reg > 2) return fail(CTW_E_ARG, "bad register");
	std::vector<uint32_t> c;
	if (int rc = canonical_reg(h, reg, c)) return rc;
	bool any_zero = false;
	for (int l = 0; l < h->lanes; ++l)
	{
		bool prp, zero;
		uint64_t r;
		res64_of(c.data() + (size_t)l * h->Dn, h->b[(size_t)l], h->Dn, prp, zero, r);
		if (is_prp) is_prp[l] = prp ? 1 : 0;
		if (res64) res64[l] = r;
		any_zero |= zero;
	}
	return any_zero ? fail(CTW_E_COMPUTE, "computation failed (zero residue)") : CTW_OK;
}

int ctw_prp_read_regs(ctw_prp *h, int first, int nregs, int32_t *out)
{
	if (int rc = check_handle(h)) return rc;
	if (!out || first < 0 || nregs < 1 || first + nregs > 3) return fail(CTW_E_ARG, "bad register range");
	CTW_CUDA(cudaMemcpyAsync(out, h->reg(first), (size_t)nregs * h->lanes * h->D * 4, cudaMemcpyDeviceToHost, h->stream));
	CTW_CUDA(cudaStreamSynchronize(h->stream));
	return CTW_OK;
}

int ctw_prp_write_regs(ctw_prp *h, int first, int nregs, const int32_t *in)
{
	if (int rc = check_handle(h)) return rc;
	if (!in || first < 0 || nregs < 1 || first + nregs > 3) return fail(CTW_E_ARG, "bad register range");
	CTW_CUDA(cudaMemcpyAsync(h->reg(first), in, (size_t)nregs * h->lanes * h->D * 4, cudaMemcpyHostToDevice, h->stream));
	CTW_CUDA(cudaStreamSynchronize(h->stream));
	return CTW_OK;
}

int ctw_prp_run(ctw_prp *h, const uint32_t *bv, int count, uint8_t *is_prp, uint64_t *res64, uint8_t *gl_ok)
{
	return ctw_prp_run_ex(h, bv, count, -1, nullptr, nullptr, is_prp, res64, gl_ok);
}

int ctw_prp_run_ex(ctw_prp *h, const uint32_t *bv, int count, long long i_start, ctw_checkpoint_fn checkpoint,
                   void *user, uint8_t *is_prp, uint64_t *res64, uint8_t *gl_ok)
{
	if (int rc = check_handle(h)) return rc;
	if (!bv || count < 1 || count > h->lanes) return fail(CTW_E_ARG, "count must be in [1, lanes]");
	const int V = h->lanes;
	std::vector<uint32_t> b((size_t)V);
	for (int l = 0; l < V; ++l) b[(size_t)l] = bv[l < count ? l : count - 1];
	int rc;
	if ((rc = ctw_prp_set_b(h, b.data(), V))) return rc;

	// Exponents E_l = b_l^D - b_l^{D/2} and the shared bit range (cyclo/src/cyclo.h:254-272).
	std::vector<Big> E((size_t)V);
	long long i0 = 0;
	for (int l = 0; l < V; ++l)
	{
		if (l > 0 && b[(size_t)l] == b[(size_t)l - 1]) E[(size_t)l] = E[(size_t)l - 1];
		else
		{
			// N+ - 1 = b^D - b^{D/2}; N- - 1 = b^Dn - b^{Dn/2} - 2
			const int lnn = h->minus ? h->ln - 1 : h->ln;
			E[(size_t)l] = prp_exponent(b[(size_t)l], lnn);
			if (h->minus) big_sub_inplace(E[(size_t)l], big_from_u64(2));
		}
		i0 = std::max(i0, (long long)big_bitlen(E[(size_t)l]) - 1);
	}
	const int L = 2 << ((31 - __builtin_clz((uint32_t)i0)) / 2);
	const long long B_GL = (i0 - 1) / L + 1;

	auto upload = [&](const std::vector<Big> &ex, int &nw) -> int {
		size_t maxw = 1;
		for (const Big &e : ex) maxw = std::max(maxw, e.size());
		nw = (int)maxw;
		std::vector<uint32_t> words((size_t)V * maxw, 0);
		for (int l = 0; l < V; ++l) std::copy(ex[(size_t)l].begin(), ex[(size_t)l].end(), words.begin() + (size_t)l * maxw);
		int r = ensure_bits(h, words.size());
		if (r) return r;
		CTW_CUDA(cudaMemcpyAsync(h->d_bits, words.data(), words.size() * 4, cudaMemcpyHostToDevice, h->stream));
		CTW_CUDA(cudaStreamSynchronize(h->stream));
		return CTW_OK;
	};

	int nw = 0;
	if ((rc = upload(E, nw))) return rc;
	if (i_start > i0) return fail(CTW_E_ARG, "resume bit %lld above the exponent's top bit %lld", i_start, i0);
	if (i_start < 0)
	{
		if ((rc = op_set(h, 0, 1)) || (rc = op_set(h, 1, 1))) return rc;
	}

	// bits i0..0; after bit i with i % B_GL == 0 and i / B_GL != 0: d <- d * x.
	// The checkpoint callback runs right after each Gerbicz-Li multiply, with
	// i the next bit to square; the reference saves its context one squaring
	// earlier (cyclo/src/cyclo.h:281-294) and resumes from any i just as well.
	long long i = i_start < 0 ? i0 : i_start;
	bool first = true;
	while (i >= 0)
	{
		if (checkpoint && !first)
		{
			CTW_CUDA(cudaStreamSynchronize(h->stream));
			if (checkpoint(user, i)) return CTW_STOPPED;
		}
		first = false;
		const long long stop = (i / B_GL) * B_GL;    // next checkpoint at or below i
		const int cnt = (int)(i - stop + 1);
		if ((rc = op_square_bits(h, h->d_bits, nw, i, cnt))) return rc;
		if (stop / B_GL != 0)
		{
			if ((rc = op_mul(h, 1, 0, 1))) return rc;
		}
		i = stop - 1;
	}
	std::vector<uint32_t> c0;
	if ((rc = canonical_reg(h, 0, c0))) return rc;

	// d(t+1) = d(t) * x in reg2; reg1 keeps d(t)
	if ((rc = op_mul(h, 2, 0, 1))) return rc;

	std::vector<Big> res((size_t)V);
	long long j0 = 0;
	for (int l = 0; l < V; ++l)
	{
		res[(size_t)l] = big_block_sum(E[(size_t)l], (int)B_GL);
		j0 = std::max(j0, (long long)big_bitlen(res[(size_t)l]) - 1);
	}
	if ((rc = upload(res, nw))) return rc;
	if ((rc = op_set(h, 0, 1))) return rc;
	if (j0 >= B_GL)
	{
		if ((rc = op_square_bits(h, h->d_bits, nw, j0, (int)(j0 - B_GL + 1)))) return rc;
	}
	if ((rc = op_mul(h, 0, 0, 1))) return rc;
	// remaining bits B_GL-1..0 (bits above j0 are zero in the exponent words)
	if ((rc = op_square_bits(h, h->d_bits, nw, B_GL - 1, (int)B_GL))) return rc;

	std::vector<uint32_t> c1, c2;
	if ((rc = canonical_reg(h, 0, c1))) return rc;
	if ((rc = canonical_reg(h, 2, c2))) return rc;
	bool any_zero = false;
	for (int l = 0; l < count; ++l)
	{
		bool prp, zero;
		uint64_t r;
		const size_t off = (size_t)l * h->Dn;
		res64_of(c0.data() + off, b[(size_t)l], h->Dn, prp, zero, r);
		if (is_prp) is_prp[l] = prp ? 1 : 0;
		if (res64) res64[l] = r;
		if (gl_ok) gl_ok[l] = (memcmp(c1.data() + off, c2.data() + off, h->Dn * sizeof(uint32_t)) == 0) ? 1 : 0;
		any_zero |= zero;
	}
	// reset like the reference between vectors (cyclo/src/cyclo.h:475-477)
	if ((rc = op_set(h, 0, 1)) || (rc = op_set(h, 1, 1))) return rc;
	if (any_zero) return fail(CTW_E_COMPUTE, "computation failed (zero residue)");
	for (int l = 0; l < count; ++l)
		if (gl_ok && !gl_ok[l]) return fail(CTW_E_GERBICZ, "Gerbicz failed (lane %d)", l);
	return CTW_OK;
}

int ctw_prp_sync(ctw_prp *h)
{
	if (int rc = check_handle(h)) return rc;
	CTW_CUDA(cudaStreamSynchronize(h->stream));
	return check_status(h);
}

void *ctw_prp_stream(ctw_prp *h) { return h ? (void *)h->stream : nullptr; }

int ctw_prp_geometry(ctw_prp *h, int *ctas, int *threads, int *smem)
{
	if (int rc = check_handle(h)) return rc;
	// the launch shape of the current prime count
	const int np = h->nprime;
	if (ctas) *ctas = (int)h->G;
	if (h->grid)
	{
		const int tw = prp_grid_smem_bytes(h->lg, h->lm, 1, np) <= 227 * 1024 ? 1 : 0;
		if (threads) *threads = prp_grid_threads(h->lm, np);
		if (smem) *smem = (int)prp_grid_smem_bytes(h->lg, h->lm, tw, np);
		return CTW_OK;
	}
	const int tw = np == 2 ? (prp_smem_bytes(h->lm, h->lg, 1, 2) <= 227 * 1024 ? 1 : 0) : h->tw_smem;
	if (threads) *threads = prp_threads(h->lm, np, h->lg);
	if (smem) *smem = (int)prp_smem_bytes(h->lm, h->lg, tw, np);
	return CTW_OK;
}

long long ctw_prp_launches(ctw_prp *h) { return h ? h->launches : 0; }

int ctw_prp_test_unreachable_barrier(ctw_prp *h)
{
	if (int rc = check_handle(h)) return rc;
	if (!h->grid) return fail(CTW_E_ARG, "the handle's split is not the grid kernel");
	h->bar_unreachable = 1;
	return CTW_OK;
}

int ctw_prp_shape(ctw_prp *h, int *log2_degree, int *lanes, int *minus)
{
	if (int rc = check_handle(h)) return rc;
	if (log2_degree) *log2_degree = h->minus ? h->ln - 1 : h->ln;
	if (lanes) *lanes = h->lanes;
	if (minus) *minus = h->minus;
	return CTW_OK;
}

double ctw_imad_peak(void)
{
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess) return 0.0;
	return imad_peak(dev);
}

double ctw_modmul_peak(int kind)
{
	int dev = 0;
	if ((kind != 0 && kind != 1) || cudaGetDevice(&dev) != cudaSuccess) return 0.0;
	return modmul_peak(dev, kind);
}

}  // extern "C"
