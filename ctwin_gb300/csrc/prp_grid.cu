// Grid kernel: one candidate of degree D = G * M spread over G = 2^LG CTAs of
// M = 2^LM coefficients in one cooperative launch (the defaults: 64 CTAs of
// 1024 for D = 2^16, 64 of 2048 for 2^17, 128 of 2048 for 2^18), more SMs than
// a thread-block cluster (at most 16) can give one candidate.
//
// The residue rests in shared memory in the column layout of the cluster
// kernel: CTA g keeps, for every row block h < G, the run of coefficients
// [h*M + g*MG, h*M + (g+1)*MG), MG = M/G.  Per squaring:
//   digits -> residues; the LG cross levels of every column (radix-8/4 passes
//   in shared memory); publish the columns to L2; gather row block g (loads
//   that bypass L1); the M-coefficient local transform, pointwise square and
//   inverse; publish the row; gather the columns; inverse cross levels;
//   Garner; carry over the runs; chunk carries.
// Registers after every squaring equal the cluster kernel's (and the
// reference's) for the same CSIZE: the same transform, carry and wrap rules.
//
// prp_kernel_grid (CTAs of 4096) orders the exchanges with grid barriers and a
// per-CTA carry count, counters in global memory zeroed by the host before each
// launch; prp_kernel_grid2 (CTAs of 1024 / 2048) needs no barrier in a
// squaring: its published words carry a parity bit that the readers poll (see
// the comment at st_pub_u1).  The cooperative launch guarantees that all CTAs
// are resident; every wait is still bounded by a %globaltimer budget, after
// which the CTA records ST_GRID_WAIT and stops waiting, so a launch always ends.
#include <type_traits>

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

// Release increment (red.release.gpu): the CTA's writes, ordered before it by
// the __syncthreads of grid_arrive, become visible to a CTA whose acquire load
// reads the new count.
__device__ __forceinline__ void grid_add_release(unsigned *p)
{
#if defined(CTW_EMU)
	__atomic_fetch_add(p, 1u, __ATOMIC_RELEASE);
#elif defined(__CUDA_ARCH__)
	asm volatile("red.release.gpu.global.add.u32 [%0], 1;" :: "l"(p) : "memory");
#else
	++*p;
#endif
}

// Barrier k of the launch over the G CTAs of one lane, in two halves: arrive
// (after every thread's global writes), then wait until k * G arrivals.  A CTA
// whose wait ran out (*dead) no longer waits.  The same pair on a per-CTA count
// (target k) waits for the k-th publication of one other CTA.  Thread 0's
// release increment and acquire load pair up across CTAs, the __syncthreads on
// either side carry the order to the other threads of each CTA (the PTX
// memory model's causality order is transitive through bar.sync), so neither
// half needs a full fence.
__device__ __forceinline__ void grid_arrive(unsigned *cnt)
{
	__syncthreads();
	if (threadIdx.x == 0) grid_add_release(cnt);
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
	const uint64_t b_m = ~0ull / b;                             // reciprocal of the one-step carry division
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
					Xh[p] = (uint32_t)reduce_b64(acc, b, b_m);
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
				Xh[p] = (uint32_t)reduce_b64(acc, b, b_m);
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

// ---------------------------------------------------------------------------
// Grid kernel with warp-local sub-transforms (CTAs of M = 1024 or 2048
// coefficients): the same squaring as prp_kernel_grid (registers equal), with
// fewer CTA-wide steps per squaring:
//   X1  digits -> residues fused into the first forward cross pass
//   X3  the last forward cross pass stores straight to L2 (no shared copy),
//       each word with its publication's parity bit
//   A   gather of row block g, polling each word for the parity of this
//       publication (no grid barrier), fused with local levels 0 .. C-1
//       (radix 2^C, C = LM - 8) across the CTA
//   W   local levels C .. LM-1, the pointwise step and their inverse on
//       sub-blocks of 256 coefficients, one warp each: three register passes
//       (radix 8, 8, 4) with warp-synchronous exchanges through shared memory;
//       local roots as Shoup pairs (one high and two low products each)
//   A'  inverse local levels C-1 .. 0 fused with the publication of the row
//   Y1  gather of the columns (polling, as A) fused with the first inverse
//       cross pass
//   Y2  the last inverse cross pass (with the final scale) fused with Garner,
//       one item per column group holding every prime
//   N   normalize1 with the chunk loaded ahead of its carry chain; each CTA
//       also gathers and transforms the last chunk of its left neighbour's
//       runs and takes that chunk's carry itself, so the carries need no
//       exchange between CTAs (when that chunk is at most half a run; else
//       the neighbour publishes its run-end carries).
// A squaring has no grid barrier: a multiply keeps one between the transform
// of y and that of x.
// Shared memory: XC [NP][G][MG] column runs (natural order, Garner words in
// place), XR [NP][M] row block (sub-block swizzle sbx), XD [M] digits at rest
// (column-run order), chunk carries and the left neighbour's run-end carries,
// cross and local roots, XN the neighbour's last chunk of every run.
// ---------------------------------------------------------------------------

// word of position p (0..255) inside a sub-block: 4-word groups XOR-permuted
// by the 32-word row, so that the three register layouts of a warp (p = lane +
// 32 k, 32 c + r + 4 k, 8 lane + k) and the pair stores of A are free of bank
// conflicts, and aligned quads stay aligned
__device__ __forceinline__ int sbx(int p) { return p ^ (((p >> 5) & 7) << 2); }

__device__ __forceinline__ uint2 ld_l2_u2(const uint32_t *p)
{
#if !defined(CTW_EMU)
	return __ldcg(reinterpret_cast<const uint2 *>(p));
#else
	return *reinterpret_cast<const uint2 *>(p);
#endif
}
__device__ __forceinline__ void st_l2_u2(uint32_t *p, uint2 v)
{
#if !defined(CTW_EMU)
	__stcg(reinterpret_cast<uint2 *>(p), v);
#else
	*reinterpret_cast<uint2 *>(p) = v;
#endif
}
__device__ __forceinline__ uint32_t ld_l2_u1(const uint32_t *p)
{
#if !defined(CTW_EMU)
	return __ldcg(p);
#else
	return *p;
#endif
}
__device__ __forceinline__ void st_l2_u1(uint32_t *p, uint32_t v)
{
#if !defined(CTW_EMU)
	__stcg(p, v);
#else
	*p = v;
#endif
}

// Published words (the columns of X3, the rows of A'): a residue below 2^31
// (in [0, 2q)) with bit 31 holding the parity of its publication within the
// launch.  The buffers are zeroed before every launch and publication k = 1,
// 2, ... of a buffer sets parity k & 1; every publication rewrites every word
// of its buffer for the launch's primes, so a word that shows the expected
// parity is this publication's, never the one before.  A reader therefore
// needs no grid barrier: it polls the words it gathers.  Stores and loads are
// relaxed at GPU scope, so each 32-bit word is single-copy atomic.
// Overwriting is safe without a barrier too: a CTA publishes a buffer again
// only after it has gathered the other buffer's next publication from every
// CTA, which each of them makes after its own gather of this one.
constexpr uint32_t PUB_BIT = 0x80000000u;
__device__ __forceinline__ void st_pub_u1(uint32_t *p, uint32_t v)
{
#if defined(CTW_EMU)
	__atomic_store_n(p, v, __ATOMIC_RELAXED);
#elif defined(__CUDA_ARCH__)
	asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
#else
	*p = v;
#endif
}
__device__ __forceinline__ void st_pub_u2(uint32_t *p, uint2 v)
{
#if defined(CTW_EMU)
	__atomic_store_n(p, v.x, __ATOMIC_RELAXED);
	__atomic_store_n(p + 1, v.y, __ATOMIC_RELAXED);
#elif defined(__CUDA_ARCH__)
	asm volatile("st.relaxed.gpu.global.v2.u32 [%0], {%1, %2};" :: "l"(p), "r"(v.x), "r"(v.y) : "memory");
#else
	p[0] = v.x;
	p[1] = v.y;
#endif
}
__device__ __forceinline__ uint2 ld_pub_u2(const uint32_t *p)
{
	uint2 v;
#if defined(CTW_EMU)
	v.x = __atomic_load_n(p, __ATOMIC_RELAXED);
	v.y = __atomic_load_n(p + 1, __ATOMIC_RELAXED);
#elif defined(__CUDA_ARCH__)
	asm volatile("ld.relaxed.gpu.global.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
#else
	v = *reinterpret_cast<const uint2 *>(p);
#endif
	return v;
}
__device__ __forceinline__ void grid_pause()
{
#if defined(CTW_EMU)
	emu_yield();
#endif
}

// Gather K published pairs (addr(k)), polling each until both words carry the
// parity bit `want` (PUB_BIT or 0), and strip the bit.  A wait that runs out
// (GRID_WAIT_NS of %globaltimer) marks the launch (ST_GRID_WAIT) and ends every
// later wait of the CTA (*dead).
template <int K, class Addr>
__device__ __forceinline__ void pub_gather(uint2 (&w)[K], Addr addr, uint32_t want, uint32_t &err,
                                           volatile int *dead)
{
#pragma unroll
	for (int k = 0; k < K; ++k) w[k] = ld_pub_u2(addr(k));
	auto stale = [&](int k) { return ((w[k].x ^ want) | (w[k].y ^ want)) & PUB_BIT; };
	uint32_t bad = 0;
#pragma unroll
	for (int k = 0; k < K; ++k) bad |= stale(k);
	if (bad && !*dead)
	{
		const unsigned long long t0 = grid_timer();
		for (;;)
		{
			grid_pause();
			// every stale pair is loaded again before any result is looked at,
			// so that one round costs one L2 round trip
#pragma unroll
			for (int k = 0; k < K; ++k)
				if (stale(k)) w[k] = ld_pub_u2(addr(k));
			bad = 0;
#pragma unroll
			for (int k = 0; k < K; ++k) bad |= stale(k);
			if (!bad || *dead) break;
			if (grid_timer() - t0 > GRID_WAIT_NS)
			{
				err |= ST_GRID_WAIT;
				*dead = 1;
				break;
			}
		}
	}
#pragma unroll
	for (int k = 0; k < K; ++k)
	{
		w[k].x &= ~PUB_BIT;
		w[k].y &= ~PUB_BIT;
	}
}
__device__ __forceinline__ void warp_sync()
{
#if defined(CTW_EMU)
	emu_syncwarp();
#else
	__syncwarp();
#endif
}

// Pad words of a column plane: when a row is 16 words, 16 words after every
// 2^r rows, r the radix exponent of the last cross pass (the rows that one
// half-warp of that pass covers: 8 for 64 CTAs, 4 for 128), so that the
// half-warps of a cross pass fall in different banks; none otherwise.
__host__ __device__ constexpr int grid2_pad_words(int lg, int lm)
{
	return ((1 << lm) >> lg) == 16
	           ? ((1 << lg) >> (lg / ((lg + 2) / 3) + ((lg + 2) / 3 - 1 < lg % ((lg + 2) / 3) ? 1 : 0))) * 16
	           : 0;
}

__host__ __device__ __forceinline__ size_t grid2_words(int lg, int lm, int np)
{
	const size_t M = (size_t)1 << lm, G = (size_t)1 << lg;
	// XC (with its pads), XR, XD, chunk carries (M/8 int64), the left
	// neighbour's carries (G int64), cross roots, TF + TI (pairs), XN, XDN
	return 2 * np * M + np * (size_t)grid2_pad_words(lg, lm) + M + M / 4 + 2 * G + 2 * np * G + 4 * np * M + np * M + M;
}

// Normalize1 of one chunk of CSZ Garner words (64-bit, two primes or narrow
// three primes): the words are loaded first, then the carry chain runs on
// registers.  Returns the chunk's carry.
// W0, W1 and XDo are 16-byte aligned: the words move in 16-byte pieces.
template <int CSZ>
__device__ __forceinline__ int64_t norm1_chunk64(const uint32_t *W0, const uint32_t *W1, int32_t *XDo, int mult,
                                                  uint32_t b, uint64_t b_m)
{
	uint32_t lo[CSZ], hi[CSZ];
#pragma unroll
	for (int i = 0; i < CSZ; i += 4)
	{
		const uint4 a0 = *reinterpret_cast<const uint4 *>(W0 + i), a1 = *reinterpret_cast<const uint4 *>(W1 + i);
		lo[i] = a0.x; lo[i + 1] = a0.y; lo[i + 2] = a0.z; lo[i + 3] = a0.w;
		hi[i] = a1.x; hi[i + 1] = a1.y; hi[i + 2] = a1.z; hi[i + 3] = a1.w;
	}
	int32_t d[CSZ];
	int64_t acc = 0;
#pragma unroll
	for (int i = 0; i < CSZ; ++i)
	{
		acc += (int64_t)((uint64_t)lo[i] | ((uint64_t)hi[i] << 32)) * (int64_t)mult;
		d[i] = reduce_b64(acc, b, b_m);
	}
#pragma unroll
	for (int i = 0; i < CSZ; i += 4) *reinterpret_cast<int4 *>(XDo + i) = make_int4(d[i], d[i + 1], d[i + 2], d[i + 3]);
	return acc;
}

template <int LG, int NP, int LM>
__global__ void __launch_bounds__(prp_grid_threads(LM, NP), 1) prp_kernel_grid2(const PrpKernelArgs a, const PrpGridArgs ga)
{
	static_assert(LM == 10 || LM == 11, "CTAs of 1024 or 2048 coefficients");
	static_assert(LG >= 4 && LG <= 7, "grid shape");
	constexpr int G = 1 << LG, M = 1 << LM, MG = M >> LG, D = M * G, C = LM - 8, NSB = 1 << C;
	constexpr int NPASS = XPass<LG, 0>::np, PL = NPASS - 1;
	static_assert(NPASS >= 2 && NPASS <= 3, "two or three cross passes");
	extern __shared__ __align__(16) uint32_t sm[];
	__shared__ int dead;
	const int tid = threadIdx.x, nt = blockDim.x, warp = tid >> 5, lane32 = tid & 31, nwarps = nt >> 5;
	const int lane = blockIdx.x / G, g = blockIdx.x % G;
	const int csz = a.csize, runc = MG / csz, ncl = G * runc, cb = g * MG;

	uint32_t *XC = sm;                                          // [NP][G][MG]
	// column planes of MP words: row h at h * MG, plus the pads of
	// grid2_pad_words (after every 2^PADSH rows when a row is 16 words)
	constexpr int MP = M + grid2_pad_words(LG, LM), PADSH = XPass<LG, PL>::r;
	static_assert(MG != 16 || (G >> PADSH) * 16 == MP - M, "pad layout");
	auto xcp = [](int h, int tt) { return h * MG + (MG == 16 ? (h >> PADSH) * 16 : 0) + tt; };
	uint32_t *XR = XC + NP * MP;                                // [NP][M] (sub-block swizzle)
	int32_t *XD = reinterpret_cast<int32_t *>(XR + NP * M);     // [G][MG] digits
	int64_t *fch = reinterpret_cast<int64_t *>(XD + M);         // [M/8]
	int64_t *xch = fch + M / 8;                                 // [G]
	uint32_t *XRT = reinterpret_cast<uint32_t *>(xch + G);      // [NP][2][G]
	uint32_t *TF = XRT + NP * 2 * G;                            // [NP][M][2] Shoup pairs
	uint32_t *TI = TF + NP * 2 * M;
	uint32_t *XN = TI + NP * 2 * M;                             // [NP][G][MG] the left neighbour's last chunk
	int32_t *XDN = reinterpret_cast<int32_t *>(XN + NP * M);   // [G][MG] its digits (discarded)
	const int gl = (g + G - 1) % G;                             // the left neighbour in natural order
	if (tid == 0) dead = 0;

	const uint32_t b = a.lane_b[4 * lane + 0], b_inv = a.lane_b[4 * lane + 1];
	const int b_s = (int)a.lane_b[4 * lane + 2];
	const uint64_t b_m = ~0ull / b;                             // reciprocal of the one-step carry division
	const bool narrow = NP == 2 || (a.narrow | (int)a.lane_b[4 * lane + 3]) != 0;
	uint32_t err = 0;

	{
		const uint32_t *tfg = a.tf + (size_t)g * 3 * 2 * M, *tig = a.ti + (size_t)g * 3 * 2 * M;
		for (int i = tid; i < NP * 2 * M; i += nt) { TF[i] = tfg[i]; TI[i] = tig[i]; }
		for (int i = tid; i < NP * 2 * G; i += nt) XRT[i] = ga.xr[(i / G) * 128 + i % G];
	}

	uint32_t *gx = ga.gx + (size_t)lane * G * 3 * M;
	uint32_t *gr = ga.gr + (size_t)lane * G * 3 * M;
	long long *gc = ga.gc + (size_t)lane * G * G;                // [G][G]: run-end carries of CTA c at c*G
	unsigned *bar = ga.bar + (size_t)lane * GRID_BAR_WORDS;
	unsigned *cpub = bar + 32;                                  // [G] carry publications of each CTA
	unsigned nbar = 0, ncar = 0;
	unsigned npx = 0, npr = 0;                                  // publications of gx / gr in this launch
	volatile int *vdead = &dead;
	// on two primes the left neighbour's last chunk is recomputed here when it
	// is at most half a run; otherwise (three primes, whose Garner step costs
	// more than the wait, or a chunk of more than half a run) the neighbour
	// publishes its run-end carries and this CTA waits for them
	const bool nbr = NP == 2 && 2 * csz <= MG;
	auto gsync = [&]() {
		++nbar;
		grid_arrive(bar);
		grid_wait(bar, nbar * (unsigned)G, err, &dead);
	};
	uint32_t *scr = a.scratch ? a.scratch + ((size_t)lane * G + g) * 3 * M : nullptr;
	const size_t lane_base = (size_t)lane * D;

	auto load_digits = [&](const int32_t *src) {
		for (int e = tid; e < M; e += nt)
		{
			const int h = e / MG, tt = e - h * MG;
			XD[e] = src[lane_base + (size_t)h * M + cb + tt];
		}
	};

	// cross pass P over XC (or from the digits / to L2), direction dir
	// columns tt < MG are this CTA's (XC), MG <= tt < ncols the left neighbour's
	// last chunk (XN)
	auto xpass = [&](auto PC, int dir, int ncols, auto load, auto store) {
		constexpr int P = decltype(PC)::value;
		constexpr int R = XPass<LG, P>::R, r = Log2<R>::v, l0 = XPass<LG, P>::l0, NGR = G >> r;
		constexpr int lsh = LG - l0 - r, stride = 1 << lsh;
		for (int it = tid; it < NP * NGR * ncols; it += nt)
		{
			const int pi = it / (NGR * ncols);
			const int rem = it - pi * NGR * ncols;
			const int gam = rem / ncols, tt = rem - gam * ncols;
			const int jblk = gam >> lsh, i = gam & (stride - 1);
			const int hbase = (jblk << (LG - l0)) + i;
			const uint32_t q = qv(pi), qi = qiv(pi);
			const uint32_t *tw = XRT + (pi * 2 + dir) * G;
			auto idx = [&](int t, int kk) { return (1 << (l0 + t)) + (jblk << t) + kk; };
			uint32_t u[R];
#pragma unroll
			for (int k = 0; k < R; ++k) u[k] = load(pi, hbase + k * stride, tt, q);
			if (dir == 0) group_fwd<R>(u, tw, idx, q, qi, l0 == 0, a.omega[pi]);
			else group_inv<R>(u, tw, idx, q, qi, l0 == 0, a.omega[pi], a.k1[pi], a.sc[pi]);
#pragma unroll
			for (int k = 0; k < R; ++k) store(pi, hbase + k * stride, tt, u[k]);
		}
	};
	auto xw = [&](int pi, int h, int tt) -> uint32_t & {
		return tt < MG ? XC[pi * MP + xcp(h, tt)] : XN[pi * M + h * MG + (tt - MG)];
	};
	auto ld_xc = [&](int pi, int h, int tt, uint32_t) { return xw(pi, h, tt); };
	auto st_xc = [&](int pi, int h, int tt, uint32_t v) { xw(pi, h, tt) = v; };

	// W: local levels C .. LM-1 of sub-block (pi, sb), pointwise, inverse
	auto wphase = [&](int pi, int sb, int mode) {
		const uint32_t q = qv(pi), qi = qiv(pi);
		uint32_t *S = XR + pi * M + sb * 256;
		const uint2 *tf = reinterpret_cast<const uint2 *>(TF) + pi * M + sb * 256;
		const uint2 *ti = reinterpret_cast<const uint2 *>(TI) + pi * M + sb * 256;
		const int l = lane32, c4 = l >> 2, r4 = l & 3;
		uint32_t u[8];
		// W1: p = l + 32 k, levels C .. C+2
#pragma unroll
		for (int k = 0; k < 8; ++k) u[k] = S[sbx(l + 32 * k)];
		group_fwd_s<8>(u, tf, [&](int t, int kk) { return (1 << t) + kk; }, q);
#pragma unroll
		for (int k = 0; k < 8; ++k) S[sbx(l + 32 * k)] = u[k];
		warp_sync();
		// W2: p = 32 c + r + 4 k, levels C+3 .. C+5
#pragma unroll
		for (int k = 0; k < 8; ++k) u[k] = S[sbx(32 * c4 + r4 + 4 * k)];
		group_fwd_s<8>(u, tf, [&](int t, int kk) { return (8 << t) + (c4 << t) + kk; }, q);
#pragma unroll
		for (int k = 0; k < 8; ++k) S[sbx(32 * c4 + r4 + 4 * k)] = u[k];
		warp_sync();
		// W3: p = 8 l + k, levels C+6, C+7 as two radix-4 groups, pointwise, inverse
		{
			const uint4 lo = *reinterpret_cast<const uint4 *>(S + sbx(8 * l));
			const uint4 hi = *reinterpret_cast<const uint4 *>(S + sbx(8 * l + 4));
			u[0] = lo.x; u[1] = lo.y; u[2] = lo.z; u[3] = lo.w;
			u[4] = hi.x; u[5] = hi.y; u[6] = hi.z; u[7] = hi.w;
		}
#pragma unroll
		for (int e = 0; e < 2; ++e)
		{
			uint32_t *v = u + 4 * e;
			const uint2 w6 = tf[64 + 32 * e + l], w7a = tf[128 + 32 * (2 * e) + l], w7b = tf[128 + 32 * (2 * e + 1) + l];
			bf_fwd_s(v[0], v[2], w6.x, w6.y, q);
			bf_fwd_s(v[1], v[3], w6.x, w6.y, q);
			bf_fwd_s(v[0], v[1], w7a.x, w7a.y, q);
			bf_fwd_s(v[2], v[3], w7b.x, w7b.y, q);
		}
		uint32_t *Y = scr + pi * M + sb * 256 + 8 * l;          // the transform of y, logical order
		if (mode == LM_FWD_ONLY)
		{
			uint32_t o[8];
#pragma unroll
			for (int k = 0; k < 8; ++k) o[k] = red(u[k], 2 * q);
			*reinterpret_cast<uint4 *>(Y) = make_uint4(o[0], o[1], o[2], o[3]);
			*reinterpret_cast<uint4 *>(Y + 4) = make_uint4(o[4], o[5], o[6], o[7]);
			return;
		}
		if (mode == LM_SQUARE)
		{
#pragma unroll
			for (int k = 0; k < 8; ++k) { const uint32_t v = red(u[k], 2 * q); u[k] = mlazy(v, v, q, qi); }
		}
		else
		{
			const uint4 ylo = *reinterpret_cast<const uint4 *>(Y), yhi = *reinterpret_cast<const uint4 *>(Y + 4);
			const uint32_t y[8] = { ylo.x, ylo.y, ylo.z, ylo.w, yhi.x, yhi.y, yhi.z, yhi.w };
#pragma unroll
			for (int k = 0; k < 8; ++k) u[k] = mlazy(red(u[k], 2 * q), y[k], q, qi);
		}
#pragma unroll
		for (int e = 0; e < 2; ++e)
		{
			uint32_t *v = u + 4 * e;
			const uint2 w6 = ti[64 + 32 * e + l], w7a = ti[128 + 32 * (2 * e) + l], w7b = ti[128 + 32 * (2 * e + 1) + l];
			bf_inv_s(v[0], v[1], w7a.x, w7a.y, q);
			bf_inv_s(v[2], v[3], w7b.x, w7b.y, q);
			bf_inv_s(v[0], v[2], w6.x, w6.y, q);
			bf_inv_s(v[1], v[3], w6.x, w6.y, q);
		}
		*reinterpret_cast<uint4 *>(S + sbx(8 * l)) = make_uint4(u[0], u[1], u[2], u[3]);
		*reinterpret_cast<uint4 *>(S + sbx(8 * l + 4)) = make_uint4(u[4], u[5], u[6], u[7]);
		warp_sync();
#pragma unroll
		for (int k = 0; k < 8; ++k) u[k] = S[sbx(32 * c4 + r4 + 4 * k)];
		group_inv_s<8>(u, ti, [&](int t, int kk) { return (8 << t) + (c4 << t) + kk; }, q);
#pragma unroll
		for (int k = 0; k < 8; ++k) S[sbx(32 * c4 + r4 + 4 * k)] = u[k];
		warp_sync();
#pragma unroll
		for (int k = 0; k < 8; ++k) u[k] = S[sbx(l + 32 * k)];
		group_inv_s<8>(u, ti, [&](int t, int kk) { return (1 << t) + kk; }, q);
#pragma unroll
		for (int k = 0; k < 8; ++k) S[sbx(l + 32 * k)] = u[k];
	};

	// a roots index of the local levels L < C, block J: word 256 (2^L + J)
	auto aidx = [&](int t, int kk) { return ((1 << t) + kk) * 256; };

	auto transform_and_normalize = [&](int mode, int mult) {
		__syncthreads();
		// X1: digits -> residues, first forward cross pass
		xpass(std::integral_constant<int, 0>{}, 0, MG,
		      [&](int, int h, int tt, uint32_t q) { return modq_i32(XD[h * MG + tt], q); }, st_xc);
		__syncthreads();
		if constexpr (NPASS == 3)
		{
			xpass(std::integral_constant<int, 1>{}, 0, MG, ld_xc, st_xc);
			__syncthreads();
		}
		// X3: last forward cross pass, columns published to L2 (reduced to
		// [0, 2q), with the parity bit)
		const uint32_t bx = (++npx & 1) ? PUB_BIT : 0u;
		const bool pub = ga.test_mute != g + 1 || npx > 1;       // testing: one CTA skips its first publication
		xpass(std::integral_constant<int, PL>{}, 0, MG, ld_xc, [&](int pi, int h, int tt, uint32_t v) {
			if (pub) st_pub_u1(gx + (size_t)g * 3 * M + pi * M + h * MG + tt, red(v, 2 * qv(pi)) | bx);
		});
		// A: gather row block g (pairs of coefficients m0, m0 + 1 of every sub-block j),
		// local levels 0 .. C-1
		for (int it = tid; it < NP * 128; it += nt)
		{
			const int pi = it >> 7, m0 = 2 * (it & 127);
			const uint32_t q = qv(pi);
			uint32_t v0[NSB], v1[NSB];
			uint2 w[NSB];
			pub_gather<NSB>(w, [&](int j) {
				const int m = j * 256 + m0, c = m / MG, tt = m - c * MG;
				return gx + (size_t)c * 3 * M + pi * M + g * MG + tt;
			}, bx, err, vdead);
#pragma unroll
			for (int j = 0; j < NSB; ++j)
			{
				v0[j] = w[j].x;
				v1[j] = w[j].y;
			}
			group_fwd_s<NSB>(v0, reinterpret_cast<const uint2 *>(TF) + pi * M, aidx, q);
			group_fwd_s<NSB>(v1, reinterpret_cast<const uint2 *>(TF) + pi * M, aidx, q);
#pragma unroll
			for (int j = 0; j < NSB; ++j)
				*reinterpret_cast<uint2 *>(XR + pi * M + j * 256 + sbx(m0)) = make_uint2(v0[j], v1[j]);
		}
		__syncthreads();
		// W: one warp per sub-block
		for (int wt = warp; wt < NP * NSB; wt += nwarps) wphase(wt / NSB, wt % NSB, mode);
		if (mode == LM_FWD_ONLY) return;
		__syncthreads();
		// A': inverse local levels C-1 .. 0, row published to L2 (natural order,
		// values in [0, 2q), with the parity bit)
		const uint32_t br = (++npr & 1) ? PUB_BIT : 0u;
		for (int it = tid; it < NP * 128; it += nt)
		{
			const int pi = it >> 7, m0 = 2 * (it & 127);
			const uint32_t q = qv(pi);
			uint32_t v0[NSB], v1[NSB];
#pragma unroll
			for (int j = 0; j < NSB; ++j)
			{
				const uint2 w = *reinterpret_cast<const uint2 *>(XR + pi * M + j * 256 + sbx(m0));
				v0[j] = w.x;
				v1[j] = w.y;
			}
			group_inv_s<NSB>(v0, reinterpret_cast<const uint2 *>(TI) + pi * M, aidx, q);
			group_inv_s<NSB>(v1, reinterpret_cast<const uint2 *>(TI) + pi * M, aidx, q);
#pragma unroll
			for (int j = 0; j < NSB; ++j)
				st_pub_u2(gr + (size_t)g * 3 * M + pi * M + j * 256 + m0, make_uint2(v0[j] | br, v1[j] | br));
		}
		// Y1: gather the columns — this CTA's and the left neighbour's last chunk —
		// in pairs, first inverse cross pass
		const int ncols = nbr ? MG + csz : MG;
		{
			constexpr int R = XPass<LG, PL>::R, r = Log2<R>::v, l0 = XPass<LG, PL>::l0, NGR = G >> r;
			constexpr int lsh = LG - l0 - r, stride = 1 << lsh;
			const int ncp = ncols / 2;
			for (int it = tid; it < NP * NGR * ncp; it += nt)
			{
				const int pi = it / (NGR * ncp);
				const int rem = it - pi * NGR * ncp;
				const int gam = rem / ncp, tt = 2 * (rem - gam * ncp);
				const int jblk = gam >> lsh, i = gam & (stride - 1);
				const int hbase = (jblk << (LG - l0)) + i;
				const uint32_t q = qv(pi), qi = qiv(pi);
				const uint32_t *tw = XRT + (pi * 2 + 1) * G;
				auto idx = [&](int t, int kk) { return (1 << (l0 + t)) + (jblk << t) + kk; };
				const uint32_t *src = gr + pi * M + (tt < MG ? g * MG + tt : gl * MG + (MG - csz) + (tt - MG));
				uint32_t u0[R], u1[R];
				uint2 w[R];
				pub_gather<R>(w, [&](int k) { return src + (size_t)(hbase + k * stride) * 3 * M; }, br, err, vdead);
#pragma unroll
				for (int k = 0; k < R; ++k)
				{
					u0[k] = w[k].x;
					u1[k] = w[k].y;
				}
				group_inv<R>(u0, tw, idx, q, qi, l0 == 0, a.omega[pi], a.k1[pi], a.sc[pi]);
				group_inv<R>(u1, tw, idx, q, qi, l0 == 0, a.omega[pi], a.k1[pi], a.sc[pi]);
#pragma unroll
				for (int k = 0; k < R; ++k)
				{
					xw(pi, hbase + k * stride, tt) = u0[k];
					xw(pi, hbase + k * stride, tt + 1) = u1[k];
				}
			}
		}
		__syncthreads();
		if constexpr (NPASS == 3)
		{
			xpass(std::integral_constant<int, 1>{}, 1, ncols, ld_xc, st_xc);
			__syncthreads();
		}
		// Y2: last inverse cross pass (levels of pass 0, with the final scale) and
		// Garner, one item per (column, row group) holding every prime
		{
			constexpr int R = XPass<LG, 0>::R, r = Log2<R>::v, NGR = G >> r, lsh = LG - r, stride = 1 << lsh;
			for (int it = tid; it < NGR * ncols; it += nt)
			{
				const int gam = it / ncols, tt = it - gam * ncols;
				const int hbase = gam;                          // pass 0: jblk = 0, i = gam
				uint32_t u[NP][R];
#pragma unroll
				for (int pi = 0; pi < NP; ++pi)
				{
					const uint32_t q = qv(pi), qi = qiv(pi);
#pragma unroll
					for (int k = 0; k < R; ++k) u[pi][k] = xw(pi, hbase + k * stride, tt);
					group_inv<R>(u[pi], XRT + (pi * 2 + 1) * G, [&](int t, int kk) { return (1 << t) + kk; }, q, qi,
					             true, a.omega[pi], a.k1[pi], a.sc[pi]);
				}
#pragma unroll
				for (int k = 0; k < R; ++k)
				{
					const int h = hbase + k * stride;
					uint32_t w0, w1;
					if constexpr (NP == 3)
					{
						uint32_t w2;
						garner3(u[0][k], u[1][k], u[2][k], a, narrow, w0, w1, w2);
						xw(2, h, tt) = w2;
					}
					else garner2(u[0][k], u[1][k], a, w0, w1);
					xw(0, h, tt) = w0;
					xw(1, h, tt) = w1;
				}
			}
		}
		__syncthreads();
		// N: normalize1 over this CTA's chunks and, per row, over the left
		// neighbour's last chunk, whose carry is the run-end carry that
		// neighbour computes for itself (normalize1 of a chunk starts from zero,
		// so it needs that chunk's Garner words only)
		auto norm1 = [&](const uint32_t *W, int stride_pl, int32_t *XDo) -> int64_t {
			if (narrow && csz == 8) return norm1_chunk64<8>(W, W + stride_pl, XDo, mult, b, b_m);
			if (narrow && csz == 16) return norm1_chunk64<16>(W, W + stride_pl, XDo, mult, b, b_m);
			if (narrow)
			{
				int64_t acc = 0;
				for (int i = 0; i < csz; ++i)
				{
					acc += load64(W, stride_pl, i) * (int64_t)mult;
					XDo[i] = reduce_b64(acc, b, b_m);
				}
				return acc;
			}
			i128 acc = 0;
			if constexpr (NP == 3)
			{
				for (int i = 0; i < csz; ++i)
				{
					acc += load96(W, stride_pl, i) * (i128)mult;
					XDo[i] = reduce_b<i128>(acc, b, b_inv, b_s, err);
				}
			}
			int64_t carry = static_cast<int64_t>(acc);
			if (static_cast<i128>(carry) != acc) err |= ST_DIGIT_RANGE;
			return carry;
		};
		for (int c = tid; c < ncl + (nbr ? G : 0); c += nt)
		{
			if (c < ncl)
			{
				const int h = c / runc, j = c - h * runc;
				const int64_t f = norm1(XC + xcp(h, j * csz), MP, XD + h * MG + j * csz);
				fch[c] = f;
				if (!nbr && j == runc - 1) xch[h] = f;
			}
			else
			{
				const int h = c - ncl;
				xch[h] = norm1(XN + h * MG, M, XDN + h * MG);
			}
		}
		__syncthreads();
		// normalize2: chunk j of run (h, g) takes the carry of the chunk before it
		// in natural order — for j = 0 the left neighbour's run-end carry, from
		// the row before for CTA 0, whose run 0 takes -f and run G/2 +f of the
		// last run (X^D = X^{D/2} - 1).  A chunk carry plus digits: 64-bit
		// arithmetic is exact.
		auto carry_in = [&](int h, int j, int64_t acc) {
			int32_t *Xh = XD + h * MG + j * csz;
			int i = 0;
			bool done = false;
			for (; i < csz - 1; ++i)
			{
				acc += Xh[i];
				Xh[i] = reduce_b64(acc, b, b_m);
				if (acc == 0) { done = true; break; }
			}
			if (!done)
			{
				const int64_t s = (int64_t)Xh[csz - 1] + (int64_t)(int32_t)(int64_t)acc;
				if (s != (int32_t)s) err |= ST_DIGIT_RANGE;
				Xh[csz - 1] = (int32_t)s;
			}
		};
		auto first_carry = [&](int h, auto run_end) -> int64_t {
			if (g > 0) return run_end(h);
			const int64_t last = run_end(G - 1);
			if (h == 0) return -last;
			return h == G / 2 ? run_end(h - 1) + last : run_end(h - 1);
		};
		if (nbr)
		{
			for (int c = tid; c < ncl; c += nt)
			{
				const int h = c / runc, j = c - h * runc;
				carry_in(h, j, j > 0 ? fch[c - 1] : first_carry(h, [&](int hh) { return xch[hh]; }));
			}
			return;
		}
		// the run-end carries are published (the last thread releases the count)
		// while threads 0 .. ncl - G - 1 carry into the chunks j > 0, which need
		// no remote carry; then the chunks j = 0 wait for the left neighbour's
		for (int h = tid; h < G; h += nt) gc[(size_t)g * G + h] = xch[h];
		++ncar;
		__syncthreads();
		if (tid == nt - 1) grid_add_release(cpub + g);
		const int nin = ncl - G;                                 // chunks j > 0
		const int nw = nin < nt - 1 ? nin : nt - 1;              // threads that carry (not the publisher)
		for (int k = tid; k < nin && tid < nw; k += nw)
		{
			const int h = k / (runc - 1), j = k - h * (runc - 1) + 1;
			carry_in(h, j, fch[h * runc + j - 1]);
		}
		grid_wait(cpub + gl, ncar, err, &dead);
		for (int h = tid; h < G; h += nt)
			carry_in(h, 0, first_carry(h, [&](int hh) { return (int64_t)ld_l2_ll(gc + (size_t)gl * G + hh); }));
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
		a.reg_out[lane_base + (size_t)h * M + cb + tt] = XD[e];
	}
	if (err) atomicOr(a.status, err);
}

// Shared memory a grid CTA asks for: at least 116 KB, so that an SM holds one
// CTA and the grid spreads over 2^lg SMs.
constexpr size_t GRID_SMEM_MIN = 116 * 1024;
size_t prp_grid_smem_bytes(int lg, int lm, int tw_smem, int np)
{
	const size_t b = (lm == 12 ? grid_words(lg, lm, tw_smem, np) : grid2_words(lg, lm, np)) * 4;
	return b > GRID_SMEM_MIN ? b : GRID_SMEM_MIN;
}

// The kernel of a grid shape: the warp-local kernel for CTAs of 1024 and 2048
// coefficients, the radix-16 kernel for 4096.
template <int LG, int NP, int LM> struct GridKern {
	typedef void (*Fn)(const PrpKernelArgs, const PrpGridArgs);
	static Fn fn()
	{
		if constexpr (LM == 12) return prp_kernel_grid<LG, NP, LM>;
		else return prp_kernel_grid2<LG, NP, LM>;
	}
};

template <int LG, int NP, int LM>
static cudaError_t grid_launch_t(const PrpKernelArgs &a, const PrpGridArgs &ga, int lanes, cudaStream_t stream)
{
	void (*kern)(const PrpKernelArgs, const PrpGridArgs) = GridKern<LG, NP, LM>::fn();
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
	at[0].id = cudaLaunchAttributeCooperative;   // all CTAs resident: every wait for another CTA can end
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
		if (kern) *kern = two ? GridKern<LG_, 2, LM_>::fn() : GridKern<LG_, 3, LM_>::fn();                       \
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
