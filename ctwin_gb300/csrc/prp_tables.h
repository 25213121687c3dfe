// Host-side construction of the PRP kernel's root tables and launch constants.
// Used by the handle-based engine and by the allocation-free multiply so that
// both feed the kernel the same layout.
#pragma once
#include <cstdint>
#include <cstring>
#include <vector>

#include "prp_arith.cuh"
#include "prp_kernels.cuh"

namespace ctw {

namespace tables_detail {
inline uint32_t mulmod(uint32_t a, uint32_t b, uint32_t q) { return (uint32_t)(((uint64_t)a * b) % q); }
inline uint32_t powmod(uint32_t a, uint64_t e, uint32_t q)
{
	uint32_t r = 1 % q;
	while (e) { if (e & 1) r = mulmod(r, a, q); a = mulmod(a, a, q); e >>= 1; }
	return r;
}
inline uint32_t invmod(uint32_t a, uint32_t q) { return powmod(a, q - 2, q); }
inline uint32_t mont(uint32_t a, uint32_t q) { return (uint32_t)((((uint64_t)a) << 32) % q); }
inline size_t bitrev(size_t j, size_t s)
{
	size_t r = 0;
	for (size_t k = s; k > 1; k >>= 1, j >>= 1) r = (r << 1) | (j & 1);
	return r;
}
}  // namespace tables_detail

// Cluster split of a degree: G = 2^lg CTAs per lane, M = D/G coefficients each.
inline int prp_lg_for(int ln) { return ln > 12 ? (ln - 12 < MAX_LG ? ln - 12 : MAX_LG) : 0; }

// XOR-swizzle selector of the shared-memory planes for M = 2^lm (the bit of the
// row index that flips bank half); chosen so that every radix pass and the
// CSIZE 8/16 carry loops are free of bank conflicts (one 2-way pass remains
// for lm = 9, 10, 13, 14).
inline int prp_swizzle_bit(int lm)
{
	switch (lm)
	{
	case 11: return 2;
	case 12: return 3;
	case 8: return 0;
	default: return 1;
	}
}

// Columns per staging round of the cross-CTA levels.
inline int prp_stage_cols(int lm, int lg)
{
	const int MG = (1 << lm) >> lg;
	const int cap = lm <= 13 ? 256 : 128;
	return MG < cap ? MG : cap;
}

// Roots of X^D - X^{D/2} + 1 in the reference's ordering
// (cyclo/src/transform.h:336-368): level s (s blocks), block j uses
// r_{6s}^{3*bitrev(j,s) + 1 + floor(2j/s)}, r_{6s} a primitive 6s-th root.
// tf/ti ([G][3][M] words, Montgomery form) hold, for CTA g and local level l,
// the root of global block g*2^l + j at index 2^l + j; the levels of the last
// local pass are stored transposed (index 2^l0 * (2^t + k) + jblk) so that
// consecutive threads read consecutive words.
// tfs/tis (lm == 12 only, else may be null): [G][3][256][2] Shoup pairs
// (w, floor(w 2^32 / q)) of the plain roots at indices 1..255 (local levels 0..7).
// lg is the cluster split (2^lg CTAs per candidate; prp_lg_for(ln) by default).
// xr (optional, [3][2][128] words): the cross-level roots in Montgomery form,
// forward then inverse, for the grid kernel (2^lg <= 128).
inline void prp_build_tables(int ln, int lg, uint32_t *tf, uint32_t *ti, PrpKernelArgs &proto, uint32_t *tfs = nullptr,
                             uint32_t *tis = nullptr, uint32_t *xr = nullptr)
{
	using namespace tables_detail;
	static const uint32_t kQ[3] = { Q0, Q1, Q2 };
	static const uint32_t kG[3] = { QGEN0, QGEN1, QGEN2 };
	const int lm = ln - lg;
	const size_t D = size_t(1) << ln, G = size_t(1) << lg, M = D / G;
	// last local pass (same split as the kernel: passes of <= 4 levels, larger first)
	const int np = (lm + 3) / 4, base = lm / np, extra = lm % np;
	int l0_last = 0;
	for (int k = 0; k < np - 1; ++k) l0_last += base + (k < extra ? 1 : 0);
	memset(tf, 0, G * 3 * M * sizeof(uint32_t));
	memset(ti, 0, G * 3 * M * sizeof(uint32_t));
	if (lm == 12 && tfs && tis)
	{
		memset(tfs, 0, G * 3 * 256 * 2 * sizeof(uint32_t));
		memset(tis, 0, G * 3 * 256 * 2 * sizeof(uint32_t));
	}
	for (int pi = 0; pi < 3; ++pi)
	{
		const uint32_t q = kQ[pi];
		std::vector<uint32_t> W(D, 0);
		for (size_t s = 1; s < D; s *= 2)
		{
			const uint32_t rs = powmod(kG[pi], (q - 1) / (6 * (uint64_t)s), q);
			for (size_t j = 0; j < s; ++j) W[s + j] = powmod(rs, 3 * bitrev(j, s) + 1 + (2 * j) / s, q);
		}
		for (size_t g = 0; g < G; ++g)
			for (int l = 0; l < lm; ++l)
				for (size_t jp = 0; jp < ((size_t)1 << l); ++jp)
				{
					const uint32_t w = W[(G << l) + (g << l) + jp];
					size_t idx = ((size_t)1 << l) + jp;
					if (l >= l0_last)
					{
						const int t = l - l0_last;
						const size_t jblk = jp >> t, kk = jp & (((size_t)1 << t) - 1);
						idx = ((size_t)1 << l0_last) * (((size_t)1 << t) + kk) + jblk;
					}
					const uint32_t wi = invmod(w, q);
					tf[(g * 3 + pi) * M + idx] = mont(w, q);
					ti[(g * 3 + pi) * M + idx] = mont(wi, q);
					if (lm == 12 && l < 8 && tfs && tis)
					{
						const size_t s = ((g * 3 + pi) * 256 + ((size_t)1 << l) + jp) * 2;
						tfs[s] = w;
						tfs[s + 1] = (uint32_t)(((uint64_t)w << 32) / q);
						tis[s] = wi;
						tis[s + 1] = (uint32_t)(((uint64_t)wi << 32) / q);
					}
				}
		for (size_t k = 1; k < G && k < (size_t)MAX_G; ++k)
		{
			const uint32_t w = W[k], wi = invmod(W[k], q);
			proto.tcf[pi][k] = w;
			proto.tcfq[pi][k] = (uint32_t)(((uint64_t)w << 32) / q);
			proto.tci[pi][k] = wi;
			proto.tciq[pi][k] = (uint32_t)(((uint64_t)wi << 32) / q);
		}
		if (xr)
			for (size_t k = 0; k < 128; ++k)
			{
				const bool in = k >= 1 && k < G;
				xr[(pi * 2 + 0) * 128 + k] = in ? mont(W[k], q) : 0;
				xr[(pi * 2 + 1) * 128 + k] = in ? mont(invmod(W[k], q), q) : 0;
			}
		const uint32_t w1 = W[1];
		const uint32_t S = mulmod((uint32_t)(((uint64_t)1 << 32) % q), mulmod(2, invmod((uint32_t)(D % q), q), q), q);
		const uint32_t K1 = mulmod(S, invmod((mulmod(2, w1, q) + q - 1) % q, q), q);
		proto.omega[pi] = mont(w1, q);
		proto.sc[pi] = mont(S, q);
		proto.k1[pi] = mont(K1, q);
	}
	proto.ginv[0] = mont(invmod(Q2 % Q1, Q1), Q1);
	proto.ginv[1] = mont(invmod(Q2 % Q0, Q0), Q0);
	proto.ginv[2] = mont(invmod(Q1 % Q0, Q0), Q0);
	proto.lm = lm;
	proto.swz_b = prp_swizzle_bit(lm);
	proto.scols = prp_stage_cols(lm, lg);
}

// Root tables of the grid kernel with warp-local sub-transforms
// (prp_kernel_grid2: 2^lg CTAs of M = 2^lm coefficients, lm = 10 or 11): the
// first C = lm - 8 local levels run across the CTA (radix 2^C), the last 8 on
// sub-blocks of 256 coefficients, one warp each.  Per CTA g and prime, M
// Shoup pairs (w, floor(w 2^32 / q)) of plain roots, 2M words ([G][3][M][2]),
// forward in tf and inverse in ti: for sub-block sb, pairs [256 sb, 256 sb +
// 256) hold its roots of local level C + l at index 2^l + jj (jj the block
// within the sub-block; for l = 6 and 7, jj = 2 u + e and 4 u + e are stored
// at 2^l + 32 e + u, the order a warp reads them in); pair 256 j (j = 1 ..
// 2^C - 1, unused by the sub-blocks) holds the root of local level L < C,
// block J with 2^L + J = j.  The root of local level L, block J of CTA g is
// that of global block (G + g) 2^L + J, as in prp_build_tables.
inline void prp_build_grid2_tables(int ln, int lg, uint32_t *tf, uint32_t *ti)
{
	using namespace tables_detail;
	static const uint32_t kQ[3] = { Q0, Q1, Q2 };
	static const uint32_t kG[3] = { QGEN0, QGEN1, QGEN2 };
	const int lm = ln - lg, C = lm - 8;
	const size_t D = size_t(1) << ln, G = size_t(1) << lg, M = D / G;
	memset(tf, 0, G * 3 * 2 * M * sizeof(uint32_t));
	memset(ti, 0, G * 3 * 2 * M * sizeof(uint32_t));
	for (int pi = 0; pi < 3; ++pi)
	{
		const uint32_t q = kQ[pi];
		std::vector<uint32_t> W(D, 0);
		for (size_t s = 1; s < D; s *= 2)
		{
			const uint32_t rs = powmod(kG[pi], (q - 1) / (6 * (uint64_t)s), q);
			for (size_t j = 0; j < s; ++j) W[s + j] = powmod(rs, 3 * bitrev(j, s) + 1 + (2 * j) / s, q);
		}
		for (size_t g = 0; g < G; ++g)
		{
			uint32_t *f = tf + (g * 3 + pi) * 2 * M, *iv = ti + (g * 3 + pi) * 2 * M;
			auto put = [&](size_t idx, int L, size_t J) {
				const uint32_t w = W[((G + g) << L) + J], wi = invmod(w, q);
				f[2 * idx] = w;
				f[2 * idx + 1] = (uint32_t)(((uint64_t)w << 32) / q);
				iv[2 * idx] = wi;
				iv[2 * idx + 1] = (uint32_t)(((uint64_t)wi << 32) / q);
			};
			for (int L = 0; L < C; ++L)
				for (size_t J = 0; J < ((size_t)1 << L); ++J) put((((size_t)1 << L) + J) * 256, L, J);
			for (size_t sb = 0; sb < ((size_t)1 << C); ++sb)
				for (int l = 0; l < 8; ++l)
					for (size_t jj = 0; jj < ((size_t)1 << l); ++jj)
					{
						size_t pos = jj;
						if (l == 6) pos = (jj & 1) * 32 + (jj >> 1);
						if (l == 7) pos = (jj & 3) * 32 + (jj >> 2);
						put(sb * 256 + ((size_t)1 << l) + pos, C + l, (sb << l) + jj);
					}
		}
	}
}

}  // namespace ctw
