// PRP kernel templates (one CTA and column-layout clusters) and their launch
// helper, shared by the translation units that instantiate them: prp_kernels.cu
// (three primes) and prp_kernels_np2.cu (two primes).
#pragma once
#include "prp_device.cuh"

namespace ctw {


// Shared memory (words): planes [3][M], stage (cross levels) or chunk carries,
// carry exchange, then the CTA's roots [3][M] forward and inverse when they fit.
__host__ __device__ __forceinline__ size_t smem_stage_words(int lm, int lg, int scols)
{
	const size_t stage = lg > 0 ? (size_t)4 * ((size_t)1 << lg) * scols : 0;
	const size_t fch = ((size_t)1 << lm) / 4;     // M/8 int64 chunk carries (CSIZE >= 8)
	return stage > fch ? stage : fch;
}

// Occupancy of the one-CTA builds: two primes run 2 CTAs per SM on the
// 4096-coefficient path (512 threads, 64 registers) and 3 on the generic path
// (at most 256 threads, 80 registers); the DENSE three-prime build of the
// 4096-coefficient path runs 2 CTAs per SM of 384 threads (80 registers).
template <bool M12, int NP, int LG, bool DENSE> struct PrpBounds {
	static constexpr int threads =
	    M12 ? ((DENSE && NP == 3) ? 384 : NP * 256) : ((NP == 2 && LG == 0) ? 256 : NT_MAX);
	static constexpr int blocks = DENSE ? 2 : ((NP == 2 && LG == 0) ? (M12 ? 2 : 3) : 1);
};

// DENSE (M12, three primes): launched with the root tables and the Shoup
// tables in global memory, so that two CTAs fit an SM; for pools whose lanes
// fill the GPU.
// The body of prp_kernel for lane `lane`, CTA g of its cluster (0 for one
// CTA); shared by the kernel below and the batch kernel (prp_batch.cu).
template <int LG, bool M12, int NP, bool DENSE = false>
__device__ __forceinline__ void prp_body(const PrpKernelArgs &a, uint32_t *sm, const int lane, const int g)
{
	constexpr int G = 1 << LG;
	static_assert(NP == 3 || LG == 0, "two-prime launches use one CTA or the column layout");
	const int lm = M12 ? 12 : a.lm, M = 1 << lm, D = M * G;   // compile-time sizes on the 4096 path
	const int tid = threadIdx.x, nt = blockDim.x;
	const int ncl = M / a.csize, sb = M12 ? 3 : a.swz_b;

	uint32_t *X = sm;                                           // [NP][M] swizzled planes
	uint32_t *ST = sm + NP * M;                                 // stage / chunk carries
	int64_t *fch = reinterpret_cast<int64_t *>(ST);             // [M/8]
	const size_t sw = smem_stage_words(lm, LG, a.scols);
	int64_t *xch = reinterpret_cast<int64_t *>(ST + sw);        // [2] carry out of this CTA's last chunk
	uint32_t *TF = ST + sw + 8;                                 // [NP][M] forward roots of this CTA
	uint32_t *TI = TF + NP * M;                                 // [NP][M] inverse roots

	const uint32_t b = a.lane_b[4 * lane + 0], b_inv = a.lane_b[4 * lane + 1];
	const int b_s = (int)a.lane_b[4 * lane + 2];
	const uint64_t b_m = ~0ull / b;                 // reciprocal of the one-step carry division
	// 64-bit carries: always with two primes, else launch-wide or per lane
	const bool narrow = NP == 2 || (a.narrow | (int)a.lane_b[4 * lane + 3]) != 0;
	uint32_t err = 0;

	// Root tables are laid out [G][3][M]: the slice of CTA g is contiguous,
	// and a two-prime launch uses the first two primes of it.
	const uint32_t *tfg = a.tf + (size_t)g * 3 * M, *tig = a.ti + (size_t)g * 3 * M;
	if (a.tw_smem)
	{
		for (int i = tid; i < NP * M; i += nt) { TF[i] = tfg[i]; TI[i] = tig[i]; }
	}
	const uint32_t *TFl = a.tw_smem ? TF : tfg;
	const uint32_t *TIl = a.tw_smem ? TI : tig;
	// Shoup roots of levels 0..7 (M12): in shared memory, or read through L1 by
	// the dense three-prime build, which has no room for them
	uint32_t *SFs = a.tw_smem ? TI + NP * M : TF, *SIs = SFs + NP * 256 * 2;
	const uint32_t *SF = SFs, *SI = SIs;
	if constexpr (M12)
	{
		const uint32_t *sfg = a.tfs + (size_t)g * 3 * 256 * 2, *sig = a.tis + (size_t)g * 3 * 256 * 2;
		if constexpr (DENSE && NP == 3)
		{
			SF = sfg;
			SI = sig;
		}
		else
			for (int i = tid; i < NP * 256 * 2; i += nt) { SFs[i] = sfg[i]; SIs[i] = sig[i]; }
	}

	const size_t lane_off = (size_t)lane * D + (size_t)g * M;
	uint32_t *scr = a.scratch ? a.scratch + ((size_t)lane * G + g) * 3 * M : nullptr;
	const bool sp_local = (LG == 0);

	// state between squarings: plane 0 holds the digits (int32)
	auto load_digits = [&](const int32_t *src) {
		for (int t = tid; t < M; t += nt) X[swz(t, sb)] = (uint32_t)src[lane_off + t];
	};

	auto transform_and_normalize = [&](int mode, int mult) {
		if constexpr (LG > 0)
		{
			csync<LG>();
			cross_levels<LG>(X, ST, M, g, 0, a, narrow, tid, nt);
			csync<LG>();
		}
		else
		{
			__syncthreads();
			for (int t = tid; t < M; t += nt)
			{
				const int p = swz(t, sb);
				to_residues<NP>(X, M, p, (int32_t)X[p]);
			}
			__syncthreads();
		}
		if constexpr (M12) local_transform12<NP>(X, TFl, TIl, SF, SI, mode, sp_local, a, scr, scr, tid, nt);
		else local_transform<NP>(X, TFl, TIl, M, lm, mode, sp_local, a, scr, scr, tid, nt);
		if (mode == LM_FWD_ONLY) return;
		if constexpr (LG > 0)
		{
			csync<LG>();
			cross_levels<LG>(X, ST, M, g, 1, a, narrow, tid, nt);   // includes Garner
			csync<LG>();
		}
		else
		{
			for (int t = tid; t < M; t += nt) garner_at<NP>(X, M, swz(t, sb), a, narrow);
			__syncthreads();
		}
		// N- = b^Dn - b^{Dn/2} - 1 (one CTA, M = 2 Dn): the transform gave the
		// exact product c_0..c_{2Dn-2}; fold it with X^Dn = X^{Dn/2} + 1:
		// j < Dn/2: c_j + c_{j+Dn} + c_{j+3Dn/2}; j >= Dn/2: c_j + c_{j+Dn/2} + 2 c_{j+Dn}
		int ncu = ncl;                                   // chunks carried
		if constexpr (LG == 0)
		{
			if (a.minus)
			{
				const int Dh = M / 2, Dq = M / 4;
				for (int j = tid; j < Dh; j += nt)
				{
					if constexpr (NP == 3)
					{
						i128 v = load96(X, M, swz(j, sb)) + load96(X, M, swz(j + Dh, sb));
						if (j < Dq) v += load96(X, M, swz(j + Dh + Dq, sb));
						else v += load96(X, M, swz(j + Dq, sb)) + load96(X, M, swz(j + Dh, sb));
						store96(X, M, swz(j, sb), v);
					}
					else
					{
						// |c| < q0 q1 / 2 < 2^59: the sum of four stays in 64 bits
						int64_t v = load64(X, M, swz(j, sb)) + load64(X, M, swz(j + Dh, sb));
						if (j < Dq) v += load64(X, M, swz(j + Dh + Dq, sb));
						else v += load64(X, M, swz(j + Dq, sb)) + load64(X, M, swz(j + Dh, sb));
						store64(X, M, swz(j, sb), v);
					}
				}
				ncu = ncl / 2;
				__syncthreads();
			}
		}
		// normalize1: one thread per chunk
		for (int c = tid; c < ncu; c += nt)
		{
			int64_t f;
			if constexpr (NP == 2) f = carry_chunk64(X, M, c, a.csize, sb, mult, b, b_m);
			else f = narrow ? carry_chunk64(X, M, c, a.csize, sb, mult, b, b_m)
			                : carry_chunk<i128>(X, M, c, a.csize, sb, mult, b, b_inv, b_s, err);
			fch[c] = f;
			if (c == ncu - 1) xch[0] = f;
		}
		csync<LG>();
		// normalize2: carry into chunk c from chunk c-1, wrap -f -> 0, +f -> D/2
		// (N-: +f -> 0 and +f -> Dn/2)
		for (int c = tid; c < ncu; c += nt)
		{
			int64_t acc;                  // a chunk carry plus digits: 64-bit arithmetic is exact
			if (c > 0)
			{
				acc = fch[c - 1];
				if (LG == 0 && c == ncu / 2) acc += fch[ncu - 1];
			}
			else if constexpr (LG > 0)
			{
				cg::cluster_group cl = cg::this_cluster();
				const int gp = (g + G - 1) % G;
				acc = *cl.map_shared_rank(xch, gp);
				if (g == 0) acc = -acc;
				else if (g == G / 2) acc += *cl.map_shared_rank(xch, G - 1);
			}
			else
			{
				acc = a.minus ? fch[ncu - 1] : -fch[ncu - 1];
			}
			int i = 0;
			bool done = false;
			for (; i < a.csize - 1; ++i)
			{
				const int p = swz(c * a.csize + i, sb);
				acc += (int32_t)X[p];
				X[p] = (uint32_t)reduce_b64(acc, b, b_m);
				if (acc == 0) { done = true; break; }
			}
			if (!done)
			{
				const int p = swz(c * a.csize + a.csize - 1, sb);
				const int64_t s = (int64_t)(int32_t)X[p] + (int64_t)(int32_t)(int64_t)acc;
				if (s != (int32_t)s) err |= ST_DIGIT_RANGE;
				X[p] = (uint32_t)(int32_t)s;
			}
		}
		if (ncu < ncl)
			for (int t = ncu * a.csize + tid; t < M; t += nt) X[swz(t, sb)] = 0;   // N-: upper half stays 0
		__syncthreads();
	};

	if (a.op == OP_MUL)
	{
		load_digits(a.reg_y);
		transform_and_normalize(LM_FWD_ONLY, 1);
		__syncthreads();
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
	// digits -> global
	for (int t = tid; t < M; t += nt) a.reg_out[lane_off + t] = (int32_t)X[swz(t, sb)];
	if (err) atomicOr(a.status, err);
	// No CTA may leave while another can still read its shared memory.
	csync<LG>();
}

template <int LG, bool M12, int NP, bool DENSE = false>
__global__ void __launch_bounds__(PrpBounds<M12, NP, LG, DENSE>::threads, PrpBounds<M12, NP, LG, DENSE>::blocks)
    prp_kernel(const PrpKernelArgs a)
{
	extern __shared__ __align__(16) uint32_t sm[];
	int g = 0;
	if constexpr (LG > 0) g = (int)cg::this_cluster().block_rank();
	prp_body<LG, M12, NP, DENSE>(a, sm, (int)blockIdx.x >> LG, g);
}

// ---------------------------------------------------------------------------
// Cluster kernel with the residue at rest in column layout (G > 1, M <= 8192).
// CTA g holds, for every row block h, the run of coefficients
// [h*M + g*MG, h*M + (g+1)*MG) (MG = M/G), in the same swizzled physical order
// as those words have in row block h.  Per squaring:
//   digits -> residues; the log2(G) cross levels, local to each column;
//   cluster barrier; pull row block g from every CTA (16-byte DSMEM loads);
//   local forward passes, pointwise, local inverse passes on the row block;
//   cluster barrier; pull the columns back; inverse cross levels and Garner,
//   local again; carry over the runs (run-end carries through DSMEM); cluster
//   barrier; chunk carries.  Three cluster barriers and two transposes.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ size_t cols_words(int lm, int lg, int tw_smem, int np)
{
	const size_t M = (size_t)1 << lm, G = (size_t)1 << lg;
	return 2 * np * M + M / 4 + 2 * G + 8 + (tw_smem ? 2 * np * M : 0);
}

// DENSE: compiled for two CTAs per SM (64 registers) and launched with the
// root tables in global memory, for pools whose many lanes fill the GPU.
// The body of prp_kernel_cols for lane `lane` on the CTAs of cluster ranks
// rbase .. rbase + G - 1, this CTA being the g-th of them; shared by the
// kernel below (rbase 0) and the batch kernel (prp_batch.cu), whose clusters
// hold several lanes.  Cluster barriers span the whole cluster: every lane of
// a cluster runs the same number of squarings.
template <int LG, bool M12, int NP, bool DENSE = false>
__device__ __forceinline__ void cols_body(const PrpKernelArgs &a, uint32_t *sm, const int lane, const int g,
                                          const int rbase)
{
	constexpr int G = 1 << LG;
	const int lm = M12 ? 12 : a.lm, M = 1 << lm, D = M * G, MG = M >> LG;   // compile-time on the 4096 path
	const int tid = threadIdx.x, nt = blockDim.x;
	cg::cluster_group cl = cg::this_cluster();
	const int csz = a.csize, sb = M12 ? 3 : a.swz_b;
	const int runc = MG / csz;                                  // chunks per run
	const int ncl = G * runc;                                   // chunks held by this CTA
	const int cb = g * MG;                                      // first column of this CTA

	uint32_t *XC = sm;                                          // [NP][G][MG] column runs
	uint32_t *XR = sm + NP * M;                                 // [NP][M] row block g
	int64_t *fch = reinterpret_cast<int64_t *>(sm + 2 * NP * M);   // [M/8] chunk carries
	int64_t *xch = fch + M / 8;                                 // [G] run-end carries
	uint32_t *TF = reinterpret_cast<uint32_t *>(xch + G) + 8;   // [NP][M] roots of row block g
	uint32_t *TI = TF + NP * M;

	const uint32_t b = a.lane_b[4 * lane + 0], b_inv = a.lane_b[4 * lane + 1];
	const int b_s = (int)a.lane_b[4 * lane + 2];
	const uint64_t b_m = ~0ull / b;                 // reciprocal of the one-step carry division
	// 64-bit carries: always with two primes, else launch-wide or per lane
	const bool narrow = NP == 2 || (a.narrow | (int)a.lane_b[4 * lane + 3]) != 0;
	uint32_t err = 0;

	const uint32_t *tfg = a.tf + (size_t)g * 3 * M, *tig = a.ti + (size_t)g * 3 * M;
	if (a.tw_smem)
	{
		for (int i = tid; i < NP * M; i += nt) { TF[i] = tfg[i]; TI[i] = tig[i]; }
	}
	const uint32_t *TFl = a.tw_smem ? TF : tfg;
	const uint32_t *TIl = a.tw_smem ? TI : tig;
	// Shoup roots of levels 0..7 (M12): in shared memory, or read through L1 by
	// the dense three-prime build, which has no room for them
	uint32_t *SFs = a.tw_smem ? TI + NP * M : TF, *SIs = SFs + NP * 256 * 2;
	const uint32_t *SF = SFs, *SI = SIs;
	if constexpr (M12)
	{
		const uint32_t *sfg = a.tfs + (size_t)g * 3 * 256 * 2, *sig = a.tis + (size_t)g * 3 * 256 * 2;
		if constexpr (DENSE && NP == 3)
		{
			SF = sfg;
			SI = sig;
		}
		else
			for (int i = tid; i < NP * 256 * 2; i += nt) { SFs[i] = sfg[i]; SIs[i] = sig[i]; }
	}
	uint32_t *scr = a.scratch ? a.scratch + ((size_t)lane * G + g) * 3 * M : nullptr;
	const size_t lane_base = (size_t)lane * D;

	// physical word of (row h, column cb + tt) in a column plane
	auto pc = [&](int h, int tt) { return h * MG + (swz(cb + tt, sb) - cb); };

	auto load_digits = [&](const int32_t *src) {
		for (int e = tid; e < M; e += nt)
		{
			const int h = e / MG, tt = e - h * MG;
			XC[pc(h, tt)] = (uint32_t)src[lane_base + (size_t)h * M + cb + tt];
		}
	};

	auto transform_and_normalize = [&](int mode, int mult) {
		__syncthreads();
		// one (prime, column) item per thread: read the digits straight into the
		// item's registers (no separate digit -> residue pass)
		const bool fused = M12 && NP * MG <= nt;
		if (!fused)
		{
			for (int e = tid; e < M; e += nt)
			{
				const int p = (e / MG) * MG + (swz(cb + e % MG, sb) - cb);
				to_residues<NP>(XC, M, p, (int32_t)XC[p]);
			}
			__syncthreads();
		}
		uint32_t vf[G];
		if (fused)
		{
			if (tid < NP * MG)
			{
				const int pi = tid / MG, tt = tid - pi * MG;
				const uint32_t *S0 = XC + (swz(cb + tt, sb) - cb);
#pragma unroll
				for (int h = 0; h < G; ++h) vf[h] = modq_i32((int32_t)S0[h * MG], qv(pi));
			}
			__syncthreads();              // every digit read before any residue plane is written
		}
		// forward cross levels, one radix-G transform per (prime, column)
		for (int it = tid; it < NP * MG; it += nt)
		{
			const int pi = it / MG, tt = it - pi * MG;
			const int p0 = swz(cb + tt, sb) - cb;
			const uint32_t q = qv(pi), qi = qiv(pi);
			uint32_t *S = XC + pi * M + p0;
			uint32_t v[G];
#pragma unroll
			for (int h = 0; h < G; ++h) v[h] = fused ? vf[h] : S[h * MG];
#pragma unroll
			for (int L = 0; L < LG; ++L)
			{
				const int half = G >> (L + 1);
#pragma unroll
				for (int h = 0; h < G; ++h)
				{
					if (h & half) continue;
					if (L == 0) bf_fwd0(v[h], v[h + half], a.omega[pi], q, qi);
					else
					{
						const int k = (1 << L) + (h >> (LG - L));
						bf_fwd_s(v[h], v[h + half], a.tcf[pi][k], a.tcfq[pi][k], q);
					}
				}
			}
#pragma unroll
			for (int h = 0; h < G; ++h) S[h * MG] = v[h];
		}
		cl.sync();
		// row block g: XR[pi][c*MG + p] <- XC_c[pi][g*MG + p]
		{
			const int MG4 = MG >> 2;
			for (int v = tid; v < NP * G * MG4; v += nt)
			{
				const int pc_ = v / MG4, o = (v - pc_ * MG4) * 4;
				const int pi = pc_ / G, c = pc_ - pi * G;
				const uint4 val = *reinterpret_cast<const uint4 *>(cl.map_shared_rank(XC + pi * M + g * MG + o, rbase + c));
				*reinterpret_cast<uint4 *>(XR + pi * M + c * MG + o) = val;
			}
		}
		__syncthreads();
		if constexpr (M12) local_transform12<NP>(XR, TFl, TIl, SF, SI, mode, false, a, scr, scr, tid, nt);
		else local_transform<NP>(XR, TFl, TIl, M, lm, mode, false, a, scr, scr, tid, nt);
		if (mode == LM_FWD_ONLY) return;
		cl.sync();
		// columns back: XC[pi][h*MG + p] <- XR_h[pi][g*MG + p]
		{
			const int MG4 = MG >> 2;
			for (int v = tid; v < NP * G * MG4; v += nt)
			{
				const int ph = v / MG4, o = (v - ph * MG4) * 4;
				const int pi = ph / G, h = ph - pi * G;
				const uint4 val = *reinterpret_cast<const uint4 *>(cl.map_shared_rank(XR + pi * M + g * MG + o, rbase + h));
				*reinterpret_cast<uint4 *>(XC + pi * M + h * MG + o) = val;
			}
		}
		__syncthreads();
		// inverse cross levels
		for (int it = tid; it < NP * MG; it += nt)
		{
			const int pi = it / MG, tt = it - pi * MG;
			const int p0 = swz(cb + tt, sb) - cb;
			const uint32_t q = qv(pi), qi = qiv(pi);
			uint32_t *S = XC + pi * M + p0;
			uint32_t v[G];
#pragma unroll
			for (int h = 0; h < G; ++h) v[h] = S[h * MG];
#pragma unroll
			for (int L = LG - 1; L >= 0; --L)
			{
				const int half = G >> (L + 1);
#pragma unroll
				for (int h = 0; h < G; ++h)
				{
					if (h & half) continue;
					if (L == 0) bf_inv0(v[h], v[h + half], a.omega[pi], a.k1[pi], a.sc[pi], q, qi);
					else
					{
						const int k = (1 << L) + (h >> (LG - L));
						bf_inv_s(v[h], v[h + half], a.tci[pi][k], a.tciq[pi][k], q);
					}
				}
			}
#pragma unroll
			for (int h = 0; h < G; ++h) S[h * MG] = v[h];
		}
		__syncthreads();
		for (int e = tid; e < M; e += nt)
			garner_at<NP>(XC, M, (e / MG) * MG + (swz(cb + e % MG, sb) - cb), a, narrow);
		__syncthreads();
		// N- (G >= 4, rows of M coefficients, Dn = G/2 rows): fold rows G/2..G-1
		// into rows 0..G/2-1 of each column (all in this CTA):
		// h < G/4: v_h + v_{h+G/2} + v_{h+3G/4}; h >= G/4: v_h + v_{h+G/4} + 2 v_{h+G/2}
		int ncu = ncl;
		if (a.minus)
		{
			const int H2 = G / 2, H4 = G / 4;
			for (int it = tid; it < H2 * MG; it += nt)
			{
				const int h = it / MG, tt = it - h * MG;
				const int p = swz(cb + tt, sb) - cb;
				if constexpr (NP == 3)
				{
					i128 v = load96(XC + h * MG, M, p) + load96(XC + (h + H2) * MG, M, p);
					if (h < H4) v += load96(XC + (h + H2 + H4) * MG, M, p);
					else v += load96(XC + (h + H4) * MG, M, p) + load96(XC + (h + H2) * MG, M, p);
					store96(XC + h * MG, M, p, v);
				}
				else
				{
					int64_t v = load64(XC + h * MG, M, p) + load64(XC + (h + H2) * MG, M, p);
					if (h < H4) v += load64(XC + (h + H2 + H4) * MG, M, p);
					else v += load64(XC + (h + H4) * MG, M, p) + load64(XC + (h + H2) * MG, M, p);
					store64(XC + h * MG, M, p, v);
				}
			}
			ncu = H2 * runc;
			__syncthreads();
		}
		// normalize1 over the runs; the last chunk of run h publishes its carry
		for (int c = tid; c < ncu; c += nt)
		{
			const int h = c / runc, j = c - h * runc;
			int64_t acc_f = 0;
			{
				uint32_t *Xh = XC + h * MG;
				const int base = cb + j * csz;
				if (NP == 2 || narrow)
				{
					int64_t acc = 0;
					auto step = [&](int i) {
						const int p = swz(base + i, sb) - cb;
						acc += load64(Xh, M, p) * (int64_t)mult;
						Xh[p] = (uint32_t)reduce_b64(acc, b, b_m);
					};
					if (csz == 8)
					{
#pragma unroll
						for (int i = 0; i < 8; ++i) step(i);
					}
					else
						for (int i = 0; i < csz; ++i) step(i);
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
			}
			fch[c] = acc_f;
			if (j == runc - 1) xch[h] = acc_f;
		}
		cl.sync();
		// normalize2: chunk j of run (h, g) takes the carry of the chunk before it
		// in natural order; -f of the last chunk goes to coefficient 0, +f to D/2
		// (N-: the last of the Dn = G/2 rows; +f to 0 and +f to Dn/2)
		const int hl = a.minus ? G / 2 - 1 : G - 1, hw = a.minus ? G / 4 : G / 2;
		for (int c = tid; c < ncu; c += nt)
		{
			const int h = c / runc, j = c - h * runc;
			// a chunk carry plus digits: |acc| < 2^62, 64-bit arithmetic is exact
			int64_t acc;
			if (j > 0) acc = fch[c - 1];
			else if (g > 0) acc = *cl.map_shared_rank(xch + h, rbase + g - 1);
			else
			{
				const int64_t last = *cl.map_shared_rank(xch + hl, rbase + G - 1);
				if (h == 0) acc = a.minus ? last : -last;
				else
				{
					acc = *cl.map_shared_rank(xch + (h - 1), rbase + G - 1);
					if (h == hw) acc += last;
				}
			}
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
		}
		if (ncu < ncl)
			for (int e = (G / 2) * MG + tid; e < M; e += nt) XC[e] = 0;   // N-: rows G/2..G-1 stay 0
		__syncthreads();
	};

	if (a.op == OP_MUL)
	{
		load_digits(a.reg_y);
		transform_and_normalize(LM_FWD_ONLY, 1);
		cl.sync();                // peers may still be pulling y's columns
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
	for (int e = tid; e < M; e += nt)
	{
		const int h = e / MG, tt = e - h * MG;
		a.reg_out[lane_base + (size_t)h * M + cb + tt] = (int32_t)XC[pc(h, tt)];
	}
	if (err) atomicOr(a.status, err);
	cl.sync();                    // peers may still read this CTA's carries
}

template <int LG, bool M12, int NP, bool DENSE = false>
__global__ void __launch_bounds__(M12 ? ((DENSE && NP == 3) ? 384 : NP * 256) : NT_MAX, DENSE ? 2 : 1)
    prp_kernel_cols(const PrpKernelArgs a)
{
	extern __shared__ __align__(16) uint32_t sm[];
	cols_body<LG, M12, NP, DENSE>(a, sm, (int)blockIdx.x >> LG, (int)cg::this_cluster().block_rank(), 0);
}

template <int LG, bool M12, bool COLS, int NP, bool DENSE = false>
static cudaError_t launch_lg(const PrpKernelArgs &a, int lanes, cudaStream_t stream)
{
	constexpr int G = 1 << LG;
	void (*kern)(const PrpKernelArgs);
	if constexpr (COLS) kern = prp_kernel_cols<LG, M12, NP, DENSE>;
	else kern = prp_kernel<LG, M12, NP, DENSE>;
	constexpr bool SHOUP_L2 = M12 && DENSE && NP == 3;     // Shoup tables read from global memory
	const size_t smem = prp_smem_bytes(a.lm, LG, a.tw_smem, NP) - (SHOUP_L2 ? prp_shoup_words(12, 3) * 4 : 0);
	cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e != cudaSuccess) return e;
	if (G > 8)
	{
		e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
		if (e != cudaSuccess) return e;
	}
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3(lanes * G);
	cfg.blockDim = dim3(SHOUP_L2 ? 384 : prp_threads(a.lm, NP, LG));
	cfg.dynamicSmemBytes = smem;
	cfg.stream = stream;
	cudaLaunchAttribute at[1];
	at[0].id = cudaLaunchAttributeClusterDimension;
	at[0].val.clusterDim.x = G;
	at[0].val.clusterDim.y = 1;
	at[0].val.clusterDim.z = 1;
	cfg.attrs = at;
	cfg.numAttrs = 1;
	return cudaLaunchKernelEx(&cfg, kern, a);
}

}  // namespace ctw
