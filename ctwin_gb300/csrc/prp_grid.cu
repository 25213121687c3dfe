// Grid kernel: one candidate of degree D = G * M spread over G = 2^LG CTAs of
// M = 2^LM coefficients in one cooperative launch (the defaults: 64 CTAs of
// 1024 for D = 2^16, 64 of 2048 for 2^17, 128 of 2048 for 2^18), more SMs than
// a thread-block cluster (at most 16) can give one candidate.
//
// The residue rests in shared memory in the column layout of the cluster
// kernel: CTA g keeps, for every row block h < G, the run of coefficients
// [h*M + g*MG, h*M + (g+1)*MG), MG = M/G.  Per squaring:
//   digits -> residues; the LG cross levels of every column (radix-8/4 passes
//   in shared memory); publish the columns to L2; grid barrier A; gather row
//   block g (16-byte loads that bypass L1); the M-coefficient local
//   transform, pointwise square and inverse; publish the row; grid barrier B;
//   gather the columns; inverse cross levels; Garner; carry over the runs;
//   publish the run-end carries; wait for those of the preceding CTA only;
//   chunk carries.
// Registers after every squaring equal the cluster kernel's (and the
// reference's) for the same CSIZE: the same transform, carry and wrap rules.
//
// Grid barriers are counters in global memory (zeroed by the host before each
// launch).  The cooperative launch guarantees that all CTAs are resident; every
// wait is still bounded by a %globaltimer budget, after which the CTA records
// ST_GRID_WAIT and stops waiting, so a launch always ends.
#include "prp_device.cuh"

namespace ctw {

namespace {

constexpr unsigned long long GRID_WAIT_NS = 50ull * 1000 * 1000;   // 50 ms per barrier

__device__ __forceinline__ unsigned long long grid_timer()
{
#if defined(CTW_EMU)
	return emu_timer_ns();
#elif defined(__CUDA_ARCH__)
	unsigned long long t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
#else
	return 0;
#endif
}

__device__ __forceinline__ unsigned grid_load_acquire(const unsigned *p)
{
#if defined(CTW_EMU)
	return __atomic_load_n(p, __ATOMIC_ACQUIRE);
#elif defined(__CUDA_ARCH__)
	unsigned v;
	asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
	return v;
#else
	return *p;
#endif
}

// 16-byte global load / store at L2 (not L1: another CTA rewrites these words
// every squaring).
__device__ __forceinline__ uint4 ld_l2(const uint32_t *p)
{
#if !defined(CTW_EMU)
	return __ldcg(reinterpret_cast<const uint4 *>(p));
#else
	return *reinterpret_cast<const uint4 *>(p);
#endif
}
__device__ __forceinline__ void st_l2(uint32_t *p, uint4 v)
{
#if !defined(CTW_EMU)
	__stcg(reinterpret_cast<uint4 *>(p), v);
#else
	*reinterpret_cast<uint4 *>(p) = v;
#endif
}
__device__ __forceinline__ long long ld_l2_ll(const long long *p)
{
#if !defined(CTW_EMU)
	return __ldcg(p);
#else
	return *p;
#endif
}

// Barrier k of the launch over the G CTAs of one lane, in two halves: arrive
// (after every thread's global writes), then wait until k * G arrivals.  A CTA
// whose wait ran out (*dead) no longer waits.  The same pair on a per-CTA count
// (target k) waits for the k-th publication of one other CTA.
__device__ __forceinline__ void grid_arrive(unsigned *cnt)
{
	__syncthreads();
	if (threadIdx.x == 0)
	{
		__threadfence();
		atomicAdd(cnt, 1u);
	}
}
__device__ __forceinline__ void grid_wait(unsigned *cnt, unsigned target, uint32_t &err, int *dead)
{
	if (threadIdx.x == 0)
	{
		if (!*dead)
		{
			const unsigned long long t0 = grid_timer();
			while ((int)(grid_load_acquire(cnt) - target) < 0)
				if (grid_timer() - t0 > GRID_WAIT_NS)
				{
					err |= ST_GRID_WAIT;
					*dead = 1;
					break;
				}
		}
		__threadfence();
	}
	__syncthreads();
}

// Radix-R pass over cross levels [l0, l0 + log2 R) of the G-point transform of
// every (prime, column) of this CTA; items (prime, group, column) with the
// column fastest, so that a warp touches consecutive words of a row.  The
// roots XRT[pi][dir][k] (Montgomery form) of level L, block j sit at k = 2^L + j.
// Swizzle selector of a grid shape: the one-CTA / cluster choice, or 20 (no
// bit-4 term, so a 16-column run stays in place) when the runs are 16 words.
template <int LG, int LM> struct GridSwz {
	static constexpr int v = LM == 12 ? 3 : (((1 << LM) >> LG) >= 32 ? (LM == 11 ? 2 : 1) : 20);
};

template <int LG, int LM, int R, int NP>
__device__ __forceinline__ void cross_pass(uint32_t *XC, const uint32_t *XRT, int l0, int dir, int cb,
                                           const PrpKernelArgs &a, int tid, int nt)
{
	constexpr int G = 1 << LG, M = 1 << LM, MG = M >> LG, r = Log2<R>::v, NGR = G >> r, SB = GridSwz<LG, LM>::v;
	const int lsh = LG - l0 - r, stride = 1 << lsh;
	for (int it = tid; it < NP * NGR * MG; it += nt)
	{
		const int pi = it / (NGR * MG);
		const int rem = it - pi * NGR * MG;
		const int gam = rem / MG, tt = rem - gam * MG;
		const int jblk = gam >> lsh, i = gam & (stride - 1);
		const int hbase = (jblk << (LG - l0)) + i;
		const uint32_t q = qv(pi), qi = qiv(pi);
		uint32_t *S = XC + pi * M + (swz(cb + tt, SB) - cb);
		const uint32_t *tw = XRT + (pi * 2 + dir) * G;
		auto idx = [&](int t, int kk) { return (1 << (l0 + t)) + (jblk << t) + kk; };
		uint32_t u[R];
#pragma unroll
		for (int k = 0; k < R; ++k) u[k] = S[(hbase + k * stride) * MG];
		if (dir == 0) group_fwd<R>(u, tw, idx, q, qi, l0 == 0, a.omega[pi]);
		else group_inv<R>(u, tw, idx, q, qi, l0 == 0, a.omega[pi], a.k1[pi], a.sc[pi]);
#pragma unroll
		for (int k = 0; k < R; ++k) S[(hbase + k * stride) * MG] = u[k];
	}
}

// The LG cross levels as passes of at most 3 levels, larger first: pass P
// covers levels [l0, l0 + r).
template <int LG, int P> struct XPass {
	static constexpr int np = (LG + 2) / 3, base = LG / np, extra = LG % np;
	static constexpr int r = base + (P < extra ? 1 : 0);
	static constexpr int l0 = P * base + (P < extra ? P : extra);
	static constexpr int R = 1 << r;
};

template <int LG, int LM, int NP, int P>
__device__ __forceinline__ void cross_one(uint32_t *XC, const uint32_t *XRT, int dir, int cb, const PrpKernelArgs &a,
                                          int tid, int nt)
{
	if constexpr (P < XPass<LG, 0>::np)
	{
		cross_pass<LG, LM, XPass<LG, P>::R, NP>(XC, XRT, XPass<LG, P>::l0, dir, cb, a, tid, nt);
		__syncthreads();
	}
}

template <int LG, int LM, int NP>
__device__ __forceinline__ void cross_all(uint32_t *XC, const uint32_t *XRT, int dir, int cb, const PrpKernelArgs &a,
                                          int tid, int nt)
{
	static_assert(XPass<LG, 0>::np <= 3, "at most three cross passes");
	if (dir == 0)
	{
		cross_one<LG, LM, NP, 0>(XC, XRT, 0, cb, a, tid, nt);
		cross_one<LG, LM, NP, 1>(XC, XRT, 0, cb, a, tid, nt);
		cross_one<LG, LM, NP, 2>(XC, XRT, 0, cb, a, tid, nt);
	}
	else
	{
		cross_one<LG, LM, NP, 2>(XC, XRT, 1, cb, a, tid, nt);
		cross_one<LG, LM, NP, 1>(XC, XRT, 1, cb, a, tid, nt);
		cross_one<LG, LM, NP, 0>(XC, XRT, 1, cb, a, tid, nt);
	}
}

}  // namespace

__host__ __device__ __forceinline__ size_t grid_words(int lg, int lm, int tw_smem, int np)
{
	const size_t M = (size_t)1 << lm, G = (size_t)1 << lg;
	return 2 * np * M + M / 4 + 2 * G + 2 * np * G + (tw_smem ? 2 * np * M : 0) + (lm == 12 ? 2 * (size_t)np * 512 : 0);
}

// LM: 12 (4096 coefficients per CTA, the dedicated radix-16 path), 11 or 10
// (2048 / 1024, the generic passes); column runs of 16 words take the swizzle
// without its bit-4 term (GridSwz).
template <int LG, int NP, int LM>
__global__ void __launch_bounds__(prp_grid_threads(LM, NP), 1) prp_kernel_grid(const PrpKernelArgs a, const PrpGridArgs ga)
{
	static_assert(LG >= 1 && LG <= 7 && LM >= 10 && LM <= 12 && ((1 << LM) >> LG) >= (LM == 12 ? 32 : 16),
	              "grid shape");
	constexpr int G = 1 << LG, M = 1 << LM, MG = M >> LG, D = M * G, sb = GridSwz<LG, LM>::v;
	extern __shared__ __align__(16) uint32_t sm[];
	__shared__ int dead;
	const int tid = threadIdx.x, nt = blockDim.x;
	const int lane = blockIdx.x / G, g = blockIdx.x % G;
	const int csz = a.csize, runc = MG / csz, ncl = G * runc, cb = g * MG;

	uint32_t *XC = sm;                                          // [NP][G][MG] column runs
	uint32_t *XR = sm + NP * M;                                 // [NP][M] row block g
	int64_t *fch = reinterpret_cast<int64_t *>(sm + 2 * NP * M);   // [M/8] chunk carries
	int64_t *xch = fch + M / 8;                                 // [G] run-end carries
	uint32_t *XRT = reinterpret_cast<uint32_t *>(xch + G);      // [NP][2][G] cross-level roots
	uint32_t *TF = XRT + NP * 2 * G;                            // [NP][M] roots of row block g
	uint32_t *TI = TF + NP * M;
	if (tid == 0) dead = 0;

	const uint32_t b = a.lane_b[4 * lane + 0], b_inv = a.lane_b[4 * lane + 1];
	const int b_s = (int)a.lane_b[4 * lane + 2];
	const bool narrow = NP == 2 || (a.narrow | (int)a.lane_b[4 * lane + 3]) != 0;
	uint32_t err = 0;

	const uint32_t *tfg = a.tf + (size_t)g * 3 * M, *tig = a.ti + (size_t)g * 3 * M;
	if (a.tw_smem)
	{
		for (int i = tid; i < NP * M; i += nt) { TF[i] = tfg[i]; TI[i] = tig[i]; }
	}
	const uint32_t *TFl = a.tw_smem ? TF : tfg;
	const uint32_t *TIl = a.tw_smem ? TI : tig;
	uint32_t *SF = a.tw_smem ? TI + NP * M : TF, *SI = SF + NP * 256 * 2;   // Shoup roots of levels 0..7 (LM 12)
	if constexpr (LM == 12)
	{
		const uint32_t *sfg = a.tfs + (size_t)g * 3 * 256 * 2, *sig = a.tis + (size_t)g * 3 * 256 * 2;
		for (int i = tid; i < NP * 256 * 2; i += nt) { SF[i] = sfg[i]; SI[i] = sig[i]; }
	}
	for (int i = tid; i < NP * 2 * G; i += nt) XRT[i] = ga.xr[(i / G) * 128 + i % G];

	uint32_t *gx = ga.gx + (size_t)lane * G * 3 * M;             // [G][3][M]: CTA c's column planes at c*3M
	uint32_t *gr = ga.gr + (size_t)lane * G * 3 * M;             // [G][3][M]: CTA h's row planes at h*3M
	long long *gc = ga.gc + (size_t)lane * G * G;                // [G][G]: run-end carries of CTA c at c*G
	unsigned *bar = ga.bar + (size_t)lane * GRID_BAR_WORDS;
	unsigned *cpub = bar + 32;                                  // [G] carry publications of each CTA
	unsigned nbar = 0, ncar = 0;
	auto garrive = [&]() {
		++nbar;
		grid_arrive(bar);
	};
	auto gwait = [&]() { grid_wait(bar, nbar * (unsigned)G, err, &dead); };
	auto gsync = [&]() {
		garrive();
		gwait();
	};
	uint32_t *scr = a.scratch ? a.scratch + ((size_t)lane * G + g) * 3 * M : nullptr;
	const size_t lane_base = (size_t)lane * D;
	constexpr int MG4 = MG / 4, M4 = M / 4;

	auto pc = [&](int h, int tt) { return h * MG + (swz(cb + tt, sb) - cb); };
	auto load_digits = [&](const int32_t *src) {
		for (int e = tid; e < M; e += nt)
		{
			const int h = e / MG, tt = e - h * MG;
			XC[pc(h, tt)] = (uint32_t)src[lane_base + (size_t)h * M + cb + tt];
		}
	};

	// The transposes: block c of prime plane pi comes from CTA c's published
	// planes (src + c*3M + pi*M + g*MG) to dst + pi*M + c*MG.  Each thread
	// issues up to GB = 4 16-byte L2 loads before it stores them, so that their
	// round trips overlap (2^16 on 64 CTAs: 74.8 k -> 77.9 k squarings/s).
	auto gather = [&](uint32_t *dst, const uint32_t *src) {
		constexpr int NV = NP * G * MG4, GB = 4;
		for (int v0 = tid; v0 < NV; v0 += GB * nt)
		{
			uint4 t[GB] = {};
#pragma unroll
			for (int k = 0; k < GB; ++k)
			{
				const int v = v0 + k * nt;
				if (v < NV)
				{
					const int bx = v / MG4, o = (v - bx * MG4) * 4, pi = bx / G, c = bx - pi * G;
					t[k] = ld_l2(src + (size_t)c * 3 * M + pi * M + g * MG + o);
				}
			}
#pragma unroll
			for (int k = 0; k < GB; ++k)
			{
				const int v = v0 + k * nt;
				if (v < NV)
				{
					const int bx = v / MG4, o = (v - bx * MG4) * 4, pi = bx / G, c = bx - pi * G;
					*reinterpret_cast<uint4 *>(dst + pi * M + c * MG + o) = t[k];
				}
			}
		}
	};

	auto transform_and_normalize = [&](int mode, int mult) {
		__syncthreads();
		for (int e = tid; e < M; e += nt)
		{
			const int p = (e / MG) * MG + (swz(cb + e % MG, sb) - cb);
			to_residues<NP>(XC, M, p, (int32_t)XC[p]);
		}
		__syncthreads();
		cross_all<LG, LM, NP>(XC, XRT, 0, cb, a, tid, nt);
		// publish the columns, gather row block g
		for (int v = tid; v < NP * M4; v += nt)
			st_l2(gx + (size_t)g * 3 * M + 4 * v, *reinterpret_cast<const uint4 *>(XC + 4 * v));
		gsync();
		gather(XR, gx);
		__syncthreads();
		if constexpr (LM == 12) local_transform12<NP>(XR, TFl, TIl, SF, SI, mode, false, a, scr, scr, tid, nt);
		else local_transform<NP>(XR, TFl, TIl, M, LM, mode, false, a, scr, scr, tid, nt);
		if (mode == LM_FWD_ONLY) return;
		// publish the row, gather the columns
		for (int v = tid; v < NP * M4; v += nt)
			st_l2(gr + (size_t)g * 3 * M + 4 * v, *reinterpret_cast<const uint4 *>(XR + 4 * v));
		gsync();
		gather(XC, gr);
		__syncthreads();
		cross_all<LG, LM, NP>(XC, XRT, 1, cb, a, tid, nt);
		for (int e = tid; e < M; e += nt) garner_at<NP>(XC, M, (e / MG) * MG + (swz(cb + e % MG, sb) - cb), a, narrow);
		__syncthreads();
		// normalize1 over the runs; the last chunk of run h publishes its carry
		for (int c = tid; c < ncl; c += nt)
		{
			const int h = c / runc, j = c - h * runc;
			uint32_t *Xh = XC + h * MG;
			const int base = cb + j * csz;
			int64_t acc_f = 0;
			if (narrow)
			{
				int64_t acc = 0;
				for (int i = 0; i < csz; ++i)
				{
					const int p = swz(base + i, sb) - cb;
					acc += load64(Xh, M, p) * (int64_t)mult;
					Xh[p] = (uint32_t)reduce_b<int64_t>(acc, b, b_inv, b_s, err);
				}
				acc_f = acc;
			}
			else if constexpr (NP == 3)
			{
				i128 acc = 0;
				for (int i = 0; i < csz; ++i)
				{
					const int p = swz(base + i, sb) - cb;
					acc += load96(Xh, M, p) * (i128)mult;
					Xh[p] = (uint32_t)reduce_b<i128>(acc, b, b_inv, b_s, err);
				}
				acc_f = (int64_t)acc;
				if ((i128)acc_f != acc) err |= ST_DIGIT_RANGE;
			}
			fch[c] = acc_f;
			if (j == runc - 1) xch[h] = acc_f;
		}
		__syncthreads();
		for (int h = tid; h < G; h += nt) gc[(size_t)g * G + h] = xch[h];
		// normalize2: chunk j of run (h, g) takes the carry of the chunk before it
		// in natural order; -f of the last chunk goes to coefficient 0, +f to D/2.
		// Chunks j > 0 need only this CTA's carries; the first chunk of each run
		// needs the run-end carries of CTA g - 1 (CTA 0: of CTA G - 1), so CTA g
		// publishes its own and waits for that one CTA's publication only.  The
		// words of gc are rewritten one squaring later, after two grid barriers
		// that the reader reaches only after it has read them.
		auto carry_in = [&](int h, int j, int64_t acc) {
			// a chunk carry plus digits: 64-bit arithmetic is exact
			uint32_t *Xh = XC + h * MG;
			const int base = cb + j * csz;
			int i = 0;
			bool done = false;
			for (; i < csz - 1; ++i)
			{
				const int p = swz(base + i, sb) - cb;
				acc += (int32_t)Xh[p];
				Xh[p] = (uint32_t)reduce_b<int64_t>(acc, b, b_inv, b_s, err);
				if (acc == 0) { done = true; break; }
			}
			if (!done)
			{
				const int p = swz(base + csz - 1, sb) - cb;
				const int64_t s = (int64_t)(int32_t)Xh[p] + (int64_t)(int32_t)(int64_t)acc;
				if (s != (int32_t)s) err |= ST_DIGIT_RANGE;
				Xh[p] = (uint32_t)(int32_t)s;
			}
		};
		++ncar;
		grid_arrive(cpub + g);
		for (int k = tid; k < ncl - G; k += nt)
		{
			const int h = k / (runc - 1), j = k - h * (runc - 1) + 1;
			carry_in(h, j, fch[h * runc + j - 1]);
		}
		grid_wait(cpub + (g + G - 1) % G, ncar, err, &dead);
		for (int h = tid; h < G; h += nt)
		{
			int64_t acc;
			if (g > 0) acc = ld_l2_ll(gc + (size_t)(g - 1) * G + h);
			else
			{
				const int64_t last = ld_l2_ll(gc + (size_t)(G - 1) * G + (G - 1));
				if (h == 0) acc = -last;
				else
				{
					acc = ld_l2_ll(gc + (size_t)(G - 1) * G + (h - 1));
					if (h == G / 2) acc += last;
				}
			}
			carry_in(h, 0, acc);
		}
		__syncthreads();
	};

	if (a.op == OP_MUL)
	{
		load_digits(a.reg_y);
		transform_and_normalize(LM_FWD_ONLY, 1);
		gsync();              // every CTA has gathered y's row block before the columns are rewritten
		load_digits(a.reg_in);
		transform_and_normalize(LM_MUL, 1);
	}
	else
	{
		load_digits(a.reg_in);
		for (int it = 0; it < a.count; ++it)
		{
			const long long i = a.i_hi - it;
			int bit = 0;
			if (a.use_dupmask) bit = (int)((a.dupmask[lane >> 6] >> (lane & 63)) & 1);
			else if (i >= 0 && (i >> 5) < a.nwords) bit = (a.bits[(size_t)lane * a.nwords + (i >> 5)] >> (i & 31)) & 1;
			transform_and_normalize(LM_SQUARE, bit ? a.mult : 1);
		}
	}
	__syncthreads();
	for (int e = tid; e < M; e += nt)
	{
		const int h = e / MG, tt = e - h * MG;
		a.reg_out[lane_base + (size_t)h * M + cb + tt] = (int32_t)XC[pc(h, tt)];
	}
	if (err) atomicOr(a.status, err);
}

// Shared memory a grid CTA asks for: at least 116 KB, so that an SM holds one
// CTA and the grid spreads over 2^lg SMs.
constexpr size_t GRID_SMEM_MIN = 116 * 1024;
size_t prp_grid_smem_bytes(int lg, int lm, int tw_smem, int np)
{
	const size_t b = grid_words(lg, lm, tw_smem, np) * 4;
	return b > GRID_SMEM_MIN ? b : GRID_SMEM_MIN;
}

template <int LG, int NP, int LM>
static cudaError_t grid_launch_t(const PrpKernelArgs &a, const PrpGridArgs &ga, int lanes, cudaStream_t stream)
{
	void (*kern)(const PrpKernelArgs, const PrpGridArgs) = prp_kernel_grid<LG, NP, LM>;
	PrpKernelArgs a2 = a;
	a2.tw_smem = prp_grid_smem_bytes(LG, LM, 1, NP) <= 227 * 1024 ? 1 : 0;
	a2.swz_b = GridSwz<LG, LM>::v;          // the generic local passes read it
	const size_t smem = prp_grid_smem_bytes(LG, LM, a2.tw_smem, NP);
	cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e != cudaSuccess) return e;
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3(lanes << LG);
	cfg.blockDim = dim3(prp_grid_threads(LM, NP));
	cfg.dynamicSmemBytes = smem;
	cfg.stream = stream;
	cudaLaunchAttribute at[1];
	at[0].id = cudaLaunchAttributeCooperative;   // all CTAs resident: the grid barriers can complete
	at[0].val.cooperative = 1;
	cfg.attrs = at;
	cfg.numAttrs = 1;
	return cudaLaunchKernelEx(&cfg, kern, a2, ga);
}

typedef cudaError_t (*GridLaunch)(const PrpKernelArgs &, const PrpGridArgs &, int, cudaStream_t);
typedef void (*GridKernel)(const PrpKernelArgs, const PrpGridArgs);

// Instances: 2^17 / 2^18 on 32 / 64 CTAs of 4096, 2^16 / 2^17 / 2^18 on 32 / 64 / 128 CTAs of 2048,
// 2^16 on 64 CTAs of 1024.
static bool grid_pick(int lg, int lm, int np, GridLaunch *launch, GridKernel *kern)
{
	const bool two = np == 2;
#define CTW_GRID_CASE(LG_, LM_)                                                                                  \
	if (lg == LG_ && lm == LM_)                                                                                  \
	{                                                                                                          \
		if (launch) *launch = two ? grid_launch_t<LG_, 2, LM_> : grid_launch_t<LG_, 3, LM_>;                     \
		if (kern) *kern = two ? prp_kernel_grid<LG_, 2, LM_> : prp_kernel_grid<LG_, 3, LM_>;                     \
		return true;                                                                                           \
	}
	CTW_GRID_CASE(5, 12)
	CTW_GRID_CASE(6, 12)
	CTW_GRID_CASE(5, 11)
	CTW_GRID_CASE(6, 11)
	CTW_GRID_CASE(7, 11)
	CTW_GRID_CASE(6, 10)
#undef CTW_GRID_CASE
	return false;
}

bool prp_grid_supported(int lg, int lm) { return grid_pick(lg, lm, 3, nullptr, nullptr); }

cudaError_t prp_grid_launch(const PrpKernelArgs &a, const PrpGridArgs &ga, int lg, int lanes, cudaStream_t stream)
{
	GridLaunch launch = nullptr;
	if (!grid_pick(lg, a.lm, a.nprime == 2 ? 2 : 3, &launch, nullptr)) return cudaErrorInvalidValue;
	if (a.csize > ((1 << a.lm) >> lg)) return cudaErrorInvalidValue;
	return launch(a, ga, lanes, stream);
}

int prp_grid_max_lanes(int lg, int lm, int np)
{
	GridKernel kern = nullptr;
	if (!grid_pick(lg, lm, np, nullptr, &kern)) return 0;
	const int tw = prp_grid_smem_bytes(lg, lm, 1, np) <= 227 * 1024 ? 1 : 0;
	const size_t smem = prp_grid_smem_bytes(lg, lm, tw, np);
	if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 0;
	int per_sm = 0, dev = 0, sms = 0;
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, prp_grid_threads(lm, np), smem) != cudaSuccess)
		return 0;
	if (cudaGetDevice(&dev) != cudaSuccess) return 0;
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	return (per_sm * sms) >> lg;
}

}  // namespace ctw
