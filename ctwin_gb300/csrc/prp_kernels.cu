// PRP squaring kernels for sm_103a.
//
// One candidate ("lane") is a degree-D polynomial of base-b digits, x in
// Z[X]/(X^D - X^{D/2} + 1) evaluated at X = b.  A launch keeps the candidate
// resident in shared memory for `count` squarings:
//   digits -> residues mod 3 primes -> forward NTT -> pointwise square ->
//   inverse NTT -> Garner CRT -> carry in chunks of CSIZE (normalize1) ->
//   chunk carries with the wrap x^D = x^{D/2} - 1 (normalize2) -> digits.
// The digit vector after every step equals the reference engine's register
// contents for the same CSIZE (cyclo/ocl/kernel.cl:1029-1081): the products
// are exact integers, and the carry follows the reference's rules.
//
// D <= 2^12: one CTA per lane (G = 1).  Larger D: a thread-block cluster of
// G = 2..16 CTAs per lane, each owning a contiguous block of M = D/G
// coefficients.  The first log2(G) NTT levels pair coefficients of different
// CTAs: each CTA pulls its column block from every peer into a local stage with
// 16-byte distributed-shared-memory loads, runs radix-G butterflies there and
// pushes the results back (the forward direction pulls only the digit plane;
// the inverse fuses Garner before the push).  All other levels are local
// radix-16/8/4/2 passes in registers over XOR-swizzled shared-memory planes
// that keep every pass and the carry loops free of bank conflicts; the
// 4096-coefficient block (D = 2^12..2^16) has its own path with compile-time
// addressing.
//
// Residues are kept lazily reduced (q < 2^30, so 4q < 2^32): forward levels
// take and give values in [0, 4q), inverse levels in [0, 2q), and the last
// inverse level (the w1 split) reduces fully before Garner.
#include "prp_kernel_impl.cuh"

namespace ctw {

size_t prp_smem_bytes(int lm, int lg, int tw_smem, int np)
{
	if (lg > 0 && lm <= 13) return (cols_words(lm, lg, tw_smem, np) + prp_shoup_words(lm, np)) * 4;
	const size_t M = size_t(1) << lm;
	const int MG = (int)(M >> lg);
	const int cap = lm <= 13 ? 256 : 128;
	const int scols = MG < cap ? MG : cap;
	size_t words = np * M + smem_stage_words(lm, lg, scols) + 8;
	if (tw_smem) words += 2 * np * M;
	return (words + prp_shoup_words(lm, np)) * 4;
}

int prp_threads(int lm, int np, int lg)
{
	if (lm == 12) return np * 256;  // one thread per (prime, radix-16 group)
	const int M = 1 << lm;
	int nt = np * M / 16;
	const int cap = (np == 2 && lg == 0) ? 256 : NT_MAX;   // the two-prime one-CTA build is bounded to 256 threads
	if (nt > cap) nt = cap;
	if (nt < 64) nt = 64;
	return (nt + 31) / 32 * 32;
}

// Cluster splits with a kernel: one CTA for M = 2^8..2^14 (the 4096-coefficient
// path for M = 2^12); column-layout clusters of 2..16 CTAs for M = 2^8..2^13
// with runs of at least 32 columns (M / G >= 32, so the swizzle stays inside a
// run); staged cross levels for M = 2^14 on 16 CTAs.  The default split of each
// degree is prp_lg_for (prp_tables.h); the others are autotuning choices.
bool prp_split_supported(int lm, int lg)
{
	if (lm < 8 || lm > 14 || lg < 0 || lg > MAX_LG) return false;
	if (lg == 0) return true;
	if (lm <= 13) return lm - lg >= 5;
	return lg == 4;
}

// SM count of the current device (cached per device).
int prp_device_sms()
{
	static int cache[16] = {};
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess) return 0;
	if (dev < 0 || dev >= 16) return 0;
	if (!cache[dev]) cudaDeviceGetAttribute(&cache[dev], cudaDevAttrMultiProcessorCount, dev);
	return cache[dev];
}

bool prp_two_prime_split(int lm, int lg)
{
	return prp_split_supported(lm, lg) && (lm == 12 || lg == 0 || (lm == 13 && lg == 4));
}

cudaError_t prp_launch(const PrpKernelArgs &a, int lg, int lanes, cudaStream_t stream)
{
	if (!prp_split_supported(a.lm, lg)) return cudaErrorInvalidValue;
	if (a.nprime == 2) return prp_launch_np2(a, lg, lanes, stream);
	if (a.lm == 12 && (a.dense > 0 || (a.dense == 0 && (lanes << lg) >= prp_device_sms())))
	{
		// dense: two CTAs of 384 threads per SM, roots and Shoup tables from L1 / L2
		PrpKernelArgs a3 = a;
		a3.tw_smem = 0;
		switch (lg)
		{
		case 0: return launch_lg<0, true, false, 3, true>(a3, lanes, stream);
		case 1: return launch_lg<1, true, true, 3, true>(a3, lanes, stream);
		case 2: return launch_lg<2, true, true, 3, true>(a3, lanes, stream);
		case 3: return launch_lg<3, true, true, 3, true>(a3, lanes, stream);
		default: return launch_lg<4, true, true, 3, true>(a3, lanes, stream);
		}
	}
	if (a.lm == 12)
	{
		switch (lg)
		{
		case 0: return launch_lg<0, true, false, 3>(a, lanes, stream);
		case 1: return launch_lg<1, true, true, 3>(a, lanes, stream);
		case 2: return launch_lg<2, true, true, 3>(a, lanes, stream);
		case 3: return launch_lg<3, true, true, 3>(a, lanes, stream);
		default: return launch_lg<4, true, true, 3>(a, lanes, stream);
		}
	}
	if (lg == 0) return launch_lg<0, false, false, 3>(a, lanes, stream);
	if (a.lm == 14) return launch_lg<4, false, false, 3>(a, lanes, stream);
	switch (lg)
	{
	case 1: return launch_lg<1, false, true, 3>(a, lanes, stream);
	case 2: return launch_lg<2, false, true, 3>(a, lanes, stream);
	case 3: return launch_lg<3, false, true, 3>(a, lanes, stream);
	default: return launch_lg<4, false, true, 3>(a, lanes, stream);
	}
}

// Per-lane register moves of a pool tick (PrpLaneAux::ops), in bit order:
// bit 0 r0 = r1 = arg; bit 1 r3 = r1; bit 2 r2 = r0; bit 3 r4 = r1;
// bit 4 r0 = arg; bit 5 r1 = r3; bit 6 r0 = r1; bit 7 r5 = r0.
// (arg is the value 1 of the reference's engine::set.)  Registers are planes
// of `stride` words; lane l's register r starts at regs + r * stride + l * D.
__global__ void prp_aux_kernel(const PrpLaneAux *aux, int32_t *regs, long long stride, int D)
{
	const int lane = blockIdx.y;
	const PrpLaneAux c = aux[lane];
	if (c.ops == 0) return;
	int32_t *r[6];
#pragma unroll
	for (int k = 0; k < 6; ++k) r[k] = regs + k * stride + (size_t)lane * D;
	for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < D; j += gridDim.x * blockDim.x)
	{
		const int32_t v = (j == 0) ? (int32_t)c.arg : 0;
		int32_t x0 = r[0][j], x1 = r[1][j], x3 = r[3][j];
		if (c.ops & 1) { x0 = v; x1 = v; r[0][j] = v; r[1][j] = v; }
		if (c.ops & 2) { x3 = x1; r[3][j] = x1; }
		if (c.ops & 4) r[2][j] = x0;
		if (c.ops & 8) r[4][j] = x1;
		if (c.ops & 16) { x0 = v; r[0][j] = v; }
		if (c.ops & 32) { x1 = x3; r[1][j] = x3; }
		if (c.ops & 64) { x0 = x1; r[0][j] = x1; }
		if (c.ops & 128) r[5][j] = x0;
	}
}

cudaError_t prp_aux_launch(const PrpLaneAux *aux, int32_t *regs, long long reg_stride, int ln, int lanes,
                           cudaStream_t stream)
{
	const int D = 1 << ln, threads = 256;
	const int gx = D / (threads * 4) > 0 ? D / (threads * 4) : 1;
	prp_aux_kernel<<<dim3(gx, lanes), threads, 0, stream>>>(aux, regs, reg_stride, D);
	return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Roofline probe: independent 32-bit multiply-add chains.
// ---------------------------------------------------------------------------
__global__ void imad_probe_kernel(uint32_t *out, int iters)
{
	uint32_t v[8];
#pragma unroll
	for (int j = 0; j < 8; ++j) v[j] = threadIdx.x * 7u + j * 13u + blockIdx.x;
	for (int i = 0; i < iters; ++i)
	{
#pragma unroll
		for (int j = 0; j < 8; ++j) v[j] = v[j] * v[j] + 0x9E3779B9u;
	}
	uint32_t s = 0;
#pragma unroll
	for (int j = 0; j < 8; ++j) s ^= v[j];
	if (s == 0x2545F491u) out[0] = s;
}

// Modular-product probes: independent chains of the two products the
// transforms are built from, on the first NTT prime.  KIND 0: Montgomery
// (mlazy: one wide product, a low product by q^-1, a high product by q);
// KIND 1: Shoup with a precomputed quotient (one high, two low products).
template <int KIND>
__global__ void modmul_probe_kernel(uint32_t *out, int iters)
{
	constexpr int C = 8;
	uint32_t v[C], w[C], wq[C];
#pragma unroll
	for (int j = 0; j < C; ++j)
	{
		v[j] = threadIdx.x * 7u + j * 13u + blockIdx.x;
		w[j] = (0x9E3779B9u * (j + 1) + blockIdx.x) % Q0;
		wq[j] = (uint32_t)(((uint64_t)w[j] << 32) / Q0);
	}
	for (int i = 0; i < iters; ++i)
	{
#pragma unroll
		for (int j = 0; j < C; ++j)
			v[j] = KIND == 0 ? mlazy(v[j], w[j], Q0, QI0) : shoup(v[j], w[j], wq[j], Q0);
	}
	uint32_t s = 0;
#pragma unroll
	for (int j = 0; j < C; ++j) s ^= v[j];
	if (s == 0x2545F491u) out[0] = s;
}

template <class Launch>
static double probe_rate(int device, double per_thread_iter, Launch launch)
{
	int sms = 0;
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
	uint32_t *out = nullptr;
	if (cudaMalloc(&out, 64) != cudaSuccess) return 0.0;
	const int grid = sms * 8, block = 256, iters = 16384;
	cudaEvent_t e0, e1;
	cudaEventCreate(&e0);
	cudaEventCreate(&e1);
	launch(grid, block, out, 256);
	float best = 1e30f;
	for (int rep = 0; rep < 3; ++rep)
	{
		cudaEventRecord(e0);
		launch(grid, block, out, iters);
		cudaEventRecord(e1);
		cudaEventSynchronize(e1);
		float ms = 0;
		cudaEventElapsedTime(&ms, e0, e1);
		if (ms < best) best = ms;
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	cudaFree(out);
	return double(grid) * block * per_thread_iter * iters / (best * 1e-3);
}

double modmul_peak(int device, int kind)
{
	if (kind == 0)
		return probe_rate(device, 8, [](int g, int b, uint32_t *o, int it) { modmul_probe_kernel<0><<<g, b>>>(o, it); });
	return probe_rate(device, 8, [](int g, int b, uint32_t *o, int it) { modmul_probe_kernel<1><<<g, b>>>(o, it); });
}

double imad_peak(int device)
{
	int sms = 0;
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
	uint32_t *out = nullptr;
	if (cudaMalloc(&out, 64) != cudaSuccess) return 0.0;
	const int grid = sms * 8, block = 256, iters = 16384;
	cudaEvent_t e0, e1;
	cudaEventCreate(&e0);
	cudaEventCreate(&e1);
	imad_probe_kernel<<<grid, block>>>(out, 256);
	float best = 1e30f;
	for (int rep = 0; rep < 3; ++rep)
	{
		cudaEventRecord(e0);
		imad_probe_kernel<<<grid, block>>>(out, iters);
		cudaEventRecord(e1);
		cudaEventSynchronize(e1);
		float ms = 0;
		cudaEventElapsedTime(&ms, e0, e1);
		if (ms < best) best = ms;
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	cudaFree(out);
	return double(grid) * block * 8 * iters / (best * 1e-3);
}

}  // namespace ctw
