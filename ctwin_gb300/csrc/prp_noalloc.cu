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
// library holds until the process exits (about 4.9 MiB in total).
#include <cstring>
#include <mutex>

#include <cuda_runtime.h>

#include "../../include/ctwin_gb300.h"
#include "prp_arith.cuh"
#include "prp_kernels.cuh"
#include "prp_tables.h"

namespace ctw {
int fail(int code, const char *fmt, ...);
}

using namespace ctw;

namespace {

constexpr int NA_MIN_LN = 8, NA_MAX_LN = 14;
constexpr size_t NA_SCRATCH_BYTES = size_t(4) << 20;   // transform of the second operand
constexpr int NA_MAX_LANES = 1024;
// forward + inverse roots, [G][3][M] = 3*D words each, for every degree 2^8..2^14,
// then the Shoup tables [G][3][256][2] of both directions for degrees 2^12..2^14
constexpr size_t NA_MAIN_WORDS = 6 * ((size_t(1) << (NA_MAX_LN + 1)) - (size_t(1) << NA_MIN_LN));
constexpr size_t NA_SHOUP_WORDS = (1 + 2 + 4) * 2 * 3 * 256 * 2;
constexpr size_t NA_TABLE_WORDS = NA_MAIN_WORDS + NA_SHOUP_WORDS;
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

// Shoup tables of degree 2^ln (12 <= ln <= 14): forward at the offset, inverse after it.
size_t na_shoup_offset(int ln)
{
	size_t off = NA_MAIN_WORDS;
	for (int k = 12; k < ln; ++k) off += (size_t(1) << (k - 12)) * 2 * 3 * 256 * 2;
	return off;
}

// One-time set-up of the current device: device addresses of the file-scope
// arrays (the names are only host-side stand-ins) and the root tables, uploaded
// on the caller's stream (no device-wide synchronisation) and waited for there.
int na_setup(int dev, cudaStream_t st)
{
	NaDevice &d = g_na_dev[dev];
	if (d.ready) return CTW_OK;
	cudaError_t e;
	if ((e = cudaGetSymbolAddress((void **)&d.scratch, g_na_scratch)) != cudaSuccess ||
	    (e = cudaGetSymbolAddress((void **)&d.tables, g_na_tables)) != cudaSuccess ||
	    (e = cudaGetSymbolAddress((void **)&d.laneb, g_na_laneb)) != cudaSuccess ||
	    (e = cudaGetSymbolAddress((void **)&d.status, g_na_status)) != cudaSuccess)
		return fail(CTW_E_CUDA, "no-alloc set-up: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
	for (int ln = NA_MIN_LN; ln <= NA_MAX_LN; ++ln)
	{
		uint32_t *tf = g_na_host_tables + na_table_offset(ln);
		memset(&d.proto[ln], 0, sizeof(PrpKernelArgs));
		uint32_t *tfs = nullptr, *tis = nullptr;
		if (ln >= 12)
		{
			const size_t G = size_t(1) << (ln - 12);
			tfs = g_na_host_tables + na_shoup_offset(ln);
			tis = tfs + G * 3 * 256 * 2;
		}
		prp_build_tables(ln, prp_lg_for(ln), tf, tf + 3 * (size_t(1) << ln), d.proto[ln], tfs, tis);
	}
	if ((e = cudaMemcpyAsync(d.tables, g_na_host_tables, sizeof(g_na_host_tables), cudaMemcpyHostToDevice, st)) !=
	        cudaSuccess ||
	    (e = cudaStreamSynchronize(st)) != cudaSuccess)
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
	{
		// the call copies from this stack frame and synchronises its stream: it
		// cannot be recorded into a graph
		cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
		const cudaError_t e = cudaStreamIsCapturing((cudaStream_t)stream, &cs);
		if (e != cudaSuccess)
		{
			cudaGetLastError();
			return fail(CTW_E_ARG, "ctw_prp_mul_noalloc: capture status of the stream: %s", cudaGetErrorString(e));
		}
		if (cs != cudaStreamCaptureStatusNone)
			return fail(CTW_E_ARG, "ctw_prp_mul_noalloc: the stream is being captured (the call synchronises it)");
	}
	uint32_t lb[NA_MAX_LANES * 4];
	uint32_t bmax = 0;
	for (int l = 0; l < lanes; ++l)
	{
		if (b[l] > bmax) bmax = b[l];
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
		if (int rc = na_setup(dev, (cudaStream_t)stream)) return rc;
		d = &g_na_dev[dev];
	}
	cudaStream_t st = (cudaStream_t)stream;
	const PrpKernelArgs &proto = d->proto[log2_degree];
	const int lg = log2_degree - proto.lm;
	if ((size_t)csize * 2 > (D >> lg)) return fail(CTW_E_ARG, "csize too large for this degree");
	PrpKernelArgs a = proto;
	a.tf = d->tables + na_table_offset(log2_degree);
	a.ti = a.tf + 3 * D;
	if (log2_degree >= 12)
	{
		a.tfs = d->tables + na_shoup_offset(log2_degree);
		a.tis = a.tfs + ((size_t)1 << (log2_degree - 12)) * 3 * 256 * 2;
	}
	a.lane_b = d->laneb;
	a.status = d->status;
	a.scratch = d->scratch;
	a.csize = csize;
	a.mult = 2;
	a.tw_smem = prp_smem_bytes(proto.lm, lg, 1) <= 227 * 1024 ? 1 : 0;
	a.narrow = (8.0 * (double)D * (double)bmax * (double)bmax < 4.611686018427388e18) ? 1 : 0;
	a.nprime = (prp_two_prime_split(proto.lm, lg) && prp_two_primes_exact(1.5 * (double)D, bmax)) ? 2 : 3;
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
