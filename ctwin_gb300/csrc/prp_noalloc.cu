// Residue multiply for callers that must not allocate device memory.
//
// Some hosts run this engine inside a GPU memory budget that belongs to
// someone else: a volunteer-computing client or plugin host that reserves the
// device when it starts, an application with its own pooling allocator that
// forbids further cudaMalloc, or a pipeline that cannot afford the implicit
// device-wide synchronisation of cudaMalloc/cudaFree in the middle of its work.
// Those callers cannot create a ctw_prp handle (creation allocates registers,
// root tables and the multiply's scratch).  ctw_prp_mul_noalloc gives them the
// engine's multiply without any allocation: the scratch, the root tables of
// every supported degree, the per-lane parameters and the status word live in
// the file-scope __device__ arrays below, which every GPU that loads the
// library holds until the process exits (about 4.8 MiB in total).
#include <cstring>
#include <mutex>

#include <cuda_runtime.h>

#include "../../include/ctwin_gb300.h"
#include "prp_arith.cuh"
#include "prp_kernels.cuh"

namespace ctw {
int fail(int code, const char *fmt, ...);
}

using namespace ctw;

namespace {

constexpr int NA_MIN_LN = 8, NA_MAX_LN = 14;
constexpr size_t NA_SCRATCH_BYTES = size_t(4) << 20;   // transform of the second operand
constexpr int NA_MAX_LANES = 1024;
// forward + inverse roots, [G][3][M] = 3*D words each, for every degree 2^8..2^14
constexpr size_t NA_TABLE_WORDS = 6 * ((size_t(1) << (NA_MAX_LN + 1)) - (size_t(1) << NA_MIN_LN));
constexpr int NA_MAX_DEVICES = 64;

static __device__ __align__(256) uint32_t g_na_scratch[NA_SCRATCH_BYTES / 4];
static __device__ __align__(256) uint32_t g_na_tables[NA_TABLE_WORDS];
static __device__ __align__(256) uint32_t g_na_laneb[NA_MAX_LANES * 4];
static __device__ __align__(256) uint32_t g_na_status[64];

struct NaDevice {
	bool ready = false;
	uint32_t *scratch = nullptr, *tables = nullptr, *laneb = nullptr, *status = nullptr;
	PrpKernelArgs proto[NA_MAX_LN + 1];
};
NaDevice g_na_dev[NA_MAX_DEVICES];
std::mutex g_na_mu;
uint32_t g_na_host_tables[NA_TABLE_WORDS];     // host staging for the one-time set-up

size_t na_table_offset(int ln)
{
	size_t off = 0;
	for (int k = NA_MIN_LN; k < ln; ++k) off += 6 * (size_t(1) << k);
	return off;
}

uint32_t na_mulmod(uint32_t a, uint32_t b, uint32_t q) { return (uint32_t)(((uint64_t)a * b) % q); }
uint32_t na_pow(uint32_t a, uint64_t e, uint32_t q)
{
	uint32_t r = 1 % q;
	while (e) { if (e & 1) r = na_mulmod(r, a, q); a = na_mulmod(a, a, q); e >>= 1; }
	return r;
}
uint32_t na_inv(uint32_t a, uint32_t q) { return na_pow(a, q - 2, q); }
uint32_t na_mont(uint32_t a, uint32_t q) { return (uint32_t)(((uint64_t)a << 32) % q); }
size_t na_bitrev(size_t j, size_t s)
{
	size_t r = 0;
	for (size_t k = s; k > 1; k >>= 1, j >>= 1) r = (r << 1) | (j & 1);
	return r;
}

// Roots of X^D - X^{D/2} + 1 for one degree, written into the host staging
// area, and the per-degree launch constants.  Same ring decomposition as the
// handle-based engine: level s, block j uses r_{6s}^{3*bitrev(j,s)+1+floor(2j/s)}.
void na_build_degree(int ln, PrpKernelArgs &proto)
{
	static const uint32_t kQ[3] = { Q0, Q1, Q2 };
	static const uint32_t kG[3] = { QGEN0, QGEN1, QGEN2 };
	const size_t D = size_t(1) << ln;
	const int lg = ln > 12 ? (ln - 12 < MAX_LG ? ln - 12 : MAX_LG) : 0;
	const size_t G = size_t(1) << lg, M = D / G;
	const int lm = ln - lg;
	uint32_t *tf = g_na_host_tables + na_table_offset(ln), *ti = tf + 3 * D;
	memset(tf, 0, 6 * D * sizeof(uint32_t));
	memset(&proto, 0, sizeof(proto));
	for (int pi = 0; pi < 3; ++pi)
	{
		const uint32_t q = kQ[pi];
		auto W = [&](size_t idx) -> uint32_t {   // root w[idx], idx = s + j
			size_t s = 1;
			while (s * 2 <= idx) s *= 2;
			const size_t j = idx - s;
			const uint32_t rs = na_pow(kG[pi], (q - 1) / (6 * (uint64_t)s), q);
			return na_pow(rs, 3 * na_bitrev(j, s) + 1 + (2 * j) / s, q);
		};
		for (size_t g = 0; g < G; ++g)
			for (int l = 0; l < lm; ++l)
				for (size_t jp = 0; jp < (size_t(1) << l); ++jp)
				{
					const uint32_t w = W((G << l) + (g << l) + jp);
					tf[(g * 3 + pi) * M + (size_t(1) << l) + jp] = na_mont(w, q);
					ti[(g * 3 + pi) * M + (size_t(1) << l) + jp] = na_mont(na_inv(w, q), q);
				}
		for (size_t k = 1; k < G; ++k)
		{
			proto.tcf[pi][k] = na_mont(W(k), q);
			proto.tci[pi][k] = na_mont(na_inv(W(k), q), q);
		}
		const uint32_t w1 = W(1);
		const uint32_t S = na_mulmod((uint32_t)(((uint64_t)1 << 32) % q), na_mulmod(2, na_inv((uint32_t)(D % q), q), q), q);
		const uint32_t K1 = na_mulmod(S, na_inv((na_mulmod(2, w1, q) + q - 1) % q, q), q);
		proto.omega[pi] = na_mont(w1, q);
		proto.sc[pi] = na_mont(S, q);
		proto.k1[pi] = na_mont(K1, q);
	}
	proto.ginv[0] = na_mont(na_inv(Q2 % Q1, Q1), Q1);
	proto.ginv[1] = na_mont(na_inv(Q2 % Q0, Q0), Q0);
	proto.ginv[2] = na_mont(na_inv(Q1 % Q0, Q0), Q0);
	proto.lm = lm;
}

// One-time set-up of the current device: device addresses of the file-scope
// arrays (the names are only host-side stand-ins) and the root tables.
int na_setup(int dev)
{
	NaDevice &d = g_na_dev[dev];
	if (d.ready) return CTW_OK;
	cudaError_t e;
	if ((e = cudaGetSymbolAddress((void **)&d.scratch, g_na_scratch)) != cudaSuccess ||
	    (e = cudaGetSymbolAddress((void **)&d.tables, g_na_tables)) != cudaSuccess ||
	    (e = cudaGetSymbolAddress((void **)&d.laneb, g_na_laneb)) != cudaSuccess ||
	    (e = cudaGetSymbolAddress((void **)&d.status, g_na_status)) != cudaSuccess)
		return fail(CTW_E_CUDA, "no-alloc set-up: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
	for (int ln = NA_MIN_LN; ln <= NA_MAX_LN; ++ln) na_build_degree(ln, d.proto[ln]);
	if ((e = cudaMemcpy(d.tables, g_na_host_tables, sizeof(g_na_host_tables), cudaMemcpyHostToDevice)) != cudaSuccess)
		return fail(CTW_E_CUDA, "no-alloc set-up: table upload: %s", cudaGetErrorString(e));
	d.ready = true;
	return CTW_OK;
}

}  // namespace

extern "C" int ctw_prp_mul_noalloc(int log2_degree, int lanes, const uint32_t *b, const int32_t *x_dev,
                                   const int32_t *y_dev, int32_t *z_dev, int csize, void *stream)
{
	if (log2_degree < NA_MIN_LN || log2_degree > NA_MAX_LN)
		return fail(CTW_E_ARG, "ctw_prp_mul_noalloc: log2_degree %d outside [%d, %d]", log2_degree, NA_MIN_LN, NA_MAX_LN);
	const size_t D = size_t(1) << log2_degree;
	if (lanes < 1 || lanes > NA_MAX_LANES || (size_t)lanes * 3 * D * sizeof(uint32_t) > NA_SCRATCH_BYTES)
		return fail(CTW_E_ARG, "ctw_prp_mul_noalloc: %d lanes of degree 2^%d exceed the fixed scratch "
		            "(lanes * 12 * D bytes <= %zu, lanes <= %d)", lanes, log2_degree, NA_SCRATCH_BYTES, NA_MAX_LANES);
	if (csize != 8 && csize != 16 && csize != 32 && csize != 64) return fail(CTW_E_ARG, "csize %d not in {8,16,32,64}", csize);
	if (!b || !x_dev || !y_dev || !z_dev) return fail(CTW_E_ARG, "ctw_prp_mul_noalloc: null pointer");
	uint32_t lb[NA_MAX_LANES * 4];
	for (int l = 0; l < lanes; ++l)
	{
		if (b[l] < 64 || b[l] >= 0x80000000u) return fail(CTW_E_ARG, "b = %u outside [64, 2^31)", b[l]);
		const int s = (31 - __builtin_clz(b[l])) - 1;
		lb[4 * l + 0] = b[l];
		lb[4 * l + 1] = (uint32_t)(((uint64_t)1 << (s + 32)) / b[l]);
		lb[4 * l + 2] = (uint32_t)s;
		lb[4 * l + 3] = 0;
	}
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES)
		return fail(CTW_E_CUDA, "ctw_prp_mul_noalloc: no current CUDA device");
	NaDevice *d;
	{
		std::lock_guard<std::mutex> g(g_na_mu);
		if (int rc = na_setup(dev)) return rc;
		d = &g_na_dev[dev];
	}
	cudaStream_t st = (cudaStream_t)stream;
	const PrpKernelArgs &proto = d->proto[log2_degree];
	const int lg = log2_degree - proto.lm;
	if ((size_t)csize * 2 > (D >> lg)) return fail(CTW_E_ARG, "csize too large for this degree");
	PrpKernelArgs a = proto;
	a.tf = d->tables + na_table_offset(log2_degree);
	a.ti = a.tf + 3 * D;
	a.lane_b = d->laneb;
	a.status = d->status;
	a.scratch = d->scratch;
	a.csize = csize;
	a.mult = 2;
	a.tw_smem = prp_smem_bytes(proto.lm, 1) <= 227 * 1024 ? 1 : 0;
	a.op = OP_MUL;
	a.reg_in = x_dev;
	a.reg_y = y_dev;
	a.reg_out = z_dev;
	a.count = 1;
	cudaError_t e;
	// the shared status word must start at zero for every call
	if ((e = cudaMemcpyAsync(d->laneb, lb, (size_t)lanes * 4 * sizeof(uint32_t), cudaMemcpyHostToDevice, st)) != cudaSuccess ||
	    (e = cudaMemsetAsync(d->status, 0, sizeof(uint32_t), st)) != cudaSuccess)
		return fail(CTW_E_CUDA, "ctw_prp_mul_noalloc: %s", cudaGetErrorString(e));
	if ((e = prp_launch(a, lg, lanes, st)) != cudaSuccess)
		return fail(CTW_E_CUDA, "ctw_prp_mul_noalloc launch: %s", cudaGetErrorString(e));
	uint32_t status = 0;
	if ((e = cudaMemcpyAsync(&status, d->status, sizeof(status), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
	    (e = cudaStreamSynchronize(st)) != cudaSuccess)
		return fail(CTW_E_CUDA, "ctw_prp_mul_noalloc: %s", cudaGetErrorString(e));
	if (status) return fail(CTW_E_COMPUTE, "ctw_prp_mul_noalloc: device range check failed (0x%x)", status);
	return CTW_OK;
}
