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
#include <cooperative_groups.h>
#include "prp_arith.cuh"
#include "prp_kernels.cuh"

namespace cg = cooperative_groups;

namespace ctw {

namespace {

constexpr int NT_MAX = 512;

__device__ __forceinline__ uint32_t qv(int pi) { return pi == 0 ? Q0 : (pi == 1 ? Q1 : Q2); }

constexpr uint32_t qinv_c(uint32_t q)
{
	uint32_t x = 1;
	for (int i = 0; i < 6; ++i) x *= 2 - q * x;
	return x;
}
constexpr uint32_t QI0 = qinv_c(Q0), QI1 = qinv_c(Q1), QI2 = qinv_c(Q2);
static_assert(Q0 * QI0 == 1u && Q1 * QI1 == 1u && Q2 * QI2 == 1u, "q^-1 mod 2^32");
__device__ __forceinline__ uint32_t qiv(int pi) { return pi == 0 ? QI0 : (pi == 1 ? QI1 : QI2); }

// ---- lazy modular arithmetic ----
// u*w/2^32 mod q in [0, 2q) for any u < 2^32 and w < q (or u, w < 2q).
__device__ __forceinline__ uint32_t mlazy(uint32_t u, uint32_t w, uint32_t q, uint32_t qi)
{
	const uint64_t p = (uint64_t)u * w;            // one wide product for lo and hi
	const uint32_t lo = (uint32_t)p, hi = (uint32_t)(p >> 32);
	const uint32_t mq = __umulhi(lo * qi, q);
	return hi - mq + q;
}
// [0, 2m) -> [0, m)
__device__ __forceinline__ uint32_t red(uint32_t x, uint32_t m) { return umin32(x, x - m); }

// Forward (Cooley-Tukey) butterfly: a in [0,4q), b any -> (a + b w, a - b w) in [0,4q).
__device__ __forceinline__ void bf_fwd(uint32_t &a, uint32_t &b, uint32_t w, uint32_t q, uint32_t qi)
{
	const uint32_t t = mlazy(b, w, q, qi);
	const uint32_t ar = red(a, 2 * q);
	b = ar - t + 2 * q;
	a = ar + t;
}
// Forward split by the 6th root w1: (a, b) -> (a + b w1, a + b - b w1), in [0,4q).
__device__ __forceinline__ void bf_fwd0(uint32_t &a, uint32_t &b, uint32_t w1, uint32_t q, uint32_t qi)
{
	const uint32_t t = mlazy(b, w1, q, qi);
	const uint32_t ar = red(a, 2 * q), s = red(ar + red(b, 2 * q), 2 * q);
	b = s - t + 2 * q;
	a = ar + t;
}
// Inverse (Gentleman-Sande) butterfly without halving: a, b in [0,2q) ->
// (a + b, (a - b) wi) in [0,2q).
__device__ __forceinline__ void bf_inv(uint32_t &a, uint32_t &b, uint32_t wi, uint32_t q, uint32_t qi)
{
	const uint32_t s = red(a + b, 2 * q);
	b = mlazy(a - b + 2 * q, wi, q, qi);
	a = s;
}
// Inverse of the w1 split with the final scale, fully reduced to [0, q):
// u1 = (a - b) k1, u0 = a S - u1 w1.
__device__ __forceinline__ void bf_inv0(uint32_t &a, uint32_t &b, uint32_t w1, uint32_t k1, uint32_t sc, uint32_t q,
                                        uint32_t qi)
{
	const uint32_t u1 = red(mlazy(a - b + 2 * q, k1, q, qi), q);
	const uint32_t u0 = mlazy(a, sc, q, qi) + 2 * q - mlazy(u1, w1, q, qi);   // (0, 4q)
	a = red(red(u0, 2 * q), q);
	b = u1;
}

// Shoup product u*w mod q in [0, 2q) for any u < 2^32, w < q, wq = floor(w 2^32 / q)
// (V. Shoup's precomputed-quotient multiplication).
__device__ __forceinline__ uint32_t shoup(uint32_t u, uint32_t w, uint32_t wq, uint32_t q)
{
	return u * w - __umulhi(u, wq) * q;
}
__device__ __forceinline__ void bf_fwd_s(uint32_t &a, uint32_t &b, uint32_t w, uint32_t wq, uint32_t q)
{
	const uint32_t t = shoup(b, w, wq, q);
	const uint32_t ar = red(a, 2 * q);
	b = ar - t + 2 * q;
	a = ar + t;
}
__device__ __forceinline__ void bf_inv_s(uint32_t &a, uint32_t &b, uint32_t w, uint32_t wq, uint32_t q)
{
	const uint32_t s = red(a + b, 2 * q);
	b = shoup(a - b + 2 * q, w, wq, q);
	a = s;
}

// Physical word of logical coefficient t in a plane (XOR within 32-word rows).
__device__ __forceinline__ int swz(int t, int b)
{
	const int x = t >> 5;
	return t ^ ((x & 15) | (((x >> b) & 1) << 4));
}

template <int R> struct Log2;
template <> struct Log2<2> { static constexpr int v = 1; };
template <> struct Log2<4> { static constexpr int v = 2; };
template <> struct Log2<8> { static constexpr int v = 3; };
template <> struct Log2<16> { static constexpr int v = 4; };

// ---------------------------------------------------------------------------
// Radix-R groups.  Forward level with s blocks: block j holds X^m - c_j and
// splits into X^{m/2} -+ w[s+j].  Global level 0 splits X^D - X^{D/2} + 1 =
// (X^{D/2} - w1)(X^{D/2} - w1^5), w1 a primitive 6th root.  The inverse levels
// skip the halving; the last one applies S = 2^32*2/D.
// idx(t, kk) gives the root of level l0+t for the pair whose high index bits
// (within the group) are kk.
// ---------------------------------------------------------------------------

template <int R, class Idx>
__device__ __forceinline__ void group_fwd(uint32_t (&u)[R], const uint32_t *__restrict__ tw, Idx idx, uint32_t q,
                                          uint32_t qi, bool special0, uint32_t omega)
{
	constexpr int r = Log2<R>::v;
#pragma unroll
	for (int t = 0; t < r; ++t)
	{
		const int half = R >> (t + 1);
#pragma unroll
		for (int k = 0; k < R; ++k)
		{
			if (k & half) continue;
			if (t == 0 && special0) bf_fwd0(u[k], u[k + half], omega, q, qi);
			else bf_fwd(u[k], u[k + half], tw[idx(t, k >> (r - t))], q, qi);
		}
	}
}

template <int R, class Idx>
__device__ __forceinline__ void group_inv(uint32_t (&u)[R], const uint32_t *__restrict__ ti, Idx idx, uint32_t q,
                                          uint32_t qi, bool special0, uint32_t omega, uint32_t k1, uint32_t sc)
{
	constexpr int r = Log2<R>::v;
#pragma unroll
	for (int t = r - 1; t >= 0; --t)
	{
		const int half = R >> (t + 1);
#pragma unroll
		for (int k = 0; k < R; ++k)
		{
			if (k & half) continue;
			if (t == 0 && special0) bf_inv0(u[k], u[k + half], omega, k1, sc, q, qi);
			else bf_inv(u[k], u[k + half], ti[idx(t, k >> (r - t))], q, qi);
		}
	}
}

// Pointwise step of the last pass: square, multiply by the stored transform
// of y, or store the transform (values leave in [0, 2q)).
enum LocalMode { LM_FWD_ONLY = 0, LM_SQUARE = 1, LM_MUL = 2 };

template <int R>
__device__ __forceinline__ bool pointwise(uint32_t (&u)[R], const int (&ph)[R], int mode, const uint32_t *Y,
                                          uint32_t *Ys, uint32_t q, uint32_t qi)
{
	if (mode == LM_SQUARE)
	{
#pragma unroll
		for (int k = 0; k < R; ++k) { const uint32_t v = red(u[k], 2 * q); u[k] = mlazy(v, v, q, qi); }
		return true;
	}
	if (mode == LM_MUL)
	{
#pragma unroll
		for (int k = 0; k < R; ++k) u[k] = mlazy(red(u[k], 2 * q), Y[ph[k]], q, qi);
		return true;
	}
#pragma unroll
	for (int k = 0; k < R; ++k) Ys[ph[k]] = red(u[k], 2 * q);
	return false;
}

struct Pass { int l0, r; };

__device__ __forceinline__ int pass_count(int lm) { return (lm + 3) / 4; }
// Passes of at most 4 levels, sizes as equal as possible, larger ones first.
__device__ __forceinline__ Pass pass_at(int lm, int i)
{
	const int np = pass_count(lm), base = lm / np, extra = lm % np;
	int l0 = 0;
	for (int k = 0; k < i; ++k) l0 += base + (k < extra ? 1 : 0);
	return Pass{ l0, base + (i < extra ? 1 : 0) };
}

// Generic radix-R pass over the CTA's M coefficients, one prime per item.
// dir: 0 forward, 1 inverse; LAST: fused forward + pointwise + inverse.
template <int R, bool LAST, int NP>
__device__ void run_pass(uint32_t *X, const uint32_t *TF, const uint32_t *TI, int M, int lm, int l0, int dir,
                         int mode, bool special_local0, const PrpKernelArgs &a, const uint32_t *ybase,
                         uint32_t *ystore, int tid, int nt)
{
	constexpr int r = Log2<R>::v;
	const int ng = M >> r, stride = M >> (l0 + r);
	const int lsh = lm - l0 - r, sb = a.swz_b;
	for (int it = tid; it < NP * ng; it += nt)
	{
		const int pi = it >> (lm - r);
		const int gam = it & (ng - 1);
		const int jblk = gam >> lsh, i = gam & (stride - 1);
		const int base = (jblk << (lm - l0)) + i;
		const uint32_t q = qv(pi), qi = qiv(pi);
		uint32_t *P = X + pi * M;
		const uint32_t *tf = TF + pi * M, *ti = TI + pi * M;
		const bool sp = special_local0 && (l0 == 0);
		auto idx = [&](int t, int kk) {
			if (LAST) return ((1 << t) + kk) * (1 << l0) + jblk;        // transposed last-pass table
			return (1 << (l0 + t)) + (jblk << t) + kk;
		};
		int ph[R];
		uint32_t u[R];
#pragma unroll
		for (int k = 0; k < R; ++k)
		{
			ph[k] = swz(base + k * stride, sb);
			u[k] = P[ph[k]];
		}
		if (dir == 0 || LAST) group_fwd<R>(u, tf, idx, q, qi, sp, a.omega[pi]);
		if (LAST && !pointwise<R>(u, ph, mode, ybase + pi * M, ystore + pi * M, q, qi)) continue;
		if (dir == 1 || LAST) group_inv<R>(u, ti, idx, q, qi, sp, a.omega[pi], a.k1[pi], a.sc[pi]);
#pragma unroll
		for (int k = 0; k < R; ++k) P[ph[k]] = u[k];
	}
}

template <bool LAST, int NP>
__device__ __forceinline__ void dispatch_pass(uint32_t *X, const uint32_t *TF, const uint32_t *TI, int M, int lm,
                                              Pass ps, int dir, int mode, bool sp, const PrpKernelArgs &a,
                                              const uint32_t *ybase, uint32_t *ystore, int tid, int nt)
{
	switch (ps.r)
	{
	case 1: run_pass<2, LAST, NP>(X, TF, TI, M, lm, ps.l0, dir, mode, sp, a, ybase, ystore, tid, nt); break;
	case 2: run_pass<4, LAST, NP>(X, TF, TI, M, lm, ps.l0, dir, mode, sp, a, ybase, ystore, tid, nt); break;
	case 3: run_pass<8, LAST, NP>(X, TF, TI, M, lm, ps.l0, dir, mode, sp, a, ybase, ystore, tid, nt); break;
	default: run_pass<16, LAST, NP>(X, TF, TI, M, lm, ps.l0, dir, mode, sp, a, ybase, ystore, tid, nt); break;
	}
}

// Generic local transform: forward passes, pointwise op, inverse passes.
template <int NP>
__device__ void local_transform(uint32_t *X, const uint32_t *TF, const uint32_t *TI, int M, int lm, int mode,
                                bool sp, const PrpKernelArgs &a, const uint32_t *ybase, uint32_t *ystore, int tid,
                                int nt)
{
	const int np = pass_count(lm);
	for (int i = 0; i < np - 1; ++i)
	{
		dispatch_pass<false, NP>(X, TF, TI, M, lm, pass_at(lm, i), 0, mode, sp, a, ybase, ystore, tid, nt);
		__syncthreads();
	}
	dispatch_pass<true, NP>(X, TF, TI, M, lm, pass_at(lm, np - 1), 0, mode, sp, a, ybase, ystore, tid, nt);
	__syncthreads();
	if (mode == LM_FWD_ONLY) return;
	for (int i = np - 2; i >= 0; --i)
	{
		dispatch_pass<false, NP>(X, TF, TI, M, lm, pass_at(lm, i), 1, mode, sp, a, ybase, ystore, tid, nt);
		__syncthreads();
	}
}

// ---------------------------------------------------------------------------
// 4096-coefficient block (passes of levels 0-3, 4-7, 8-11), one thread per
// (prime, radix-16 group).  With the swizzle bit 3 the physical
// addresses of a group are base registers combined with compile-time offsets:
//   pass A (stride 256): (g ^ g>>5 ^ 24*(k&1)) + 256k
//   pass B (stride 16):  (256*jb + (i ^ 24*(jb&1))) ^ ((16*(k&1) ^ k>>1) + 32*(k>>1))
//   pass C (stride 1):   swz(16 g) ^ k
// ---------------------------------------------------------------------------
constexpr int M12 = 4096;

__device__ __forceinline__ int kB(int k) { return ((16 * (k & 1)) ^ (k >> 1)) + 32 * (k >> 1); }

template <int PASS>
__device__ __forceinline__ void addr12(int g, int (&ph)[16])
{
	if (PASS == 0)
	{
		const int pe = g ^ (g >> 5), po = pe ^ 24;
#pragma unroll
		for (int k = 0; k < 16; ++k) ph[k] = ((k & 1) ? po : pe) + 256 * k;
	}
	else if (PASS == 1)
	{
		const int jb = g >> 4, i = g & 15;
		const int base = 256 * jb + (i ^ (24 * (jb & 1)));
#pragma unroll
		for (int k = 0; k < 16; ++k) ph[k] = base ^ kB(k);
	}
	else
	{
		const int x = (16 * g) >> 5;
		const int P0 = (16 * g) ^ ((x & 15) | (((x >> 3) & 1) << 4));
#pragma unroll
		for (int k = 0; k < 16; ++k) ph[k] = P0 ^ k;
	}
}

template <int PASS>
__device__ __forceinline__ void pass12(uint32_t *X, const uint32_t *TF, const uint32_t *TI, const uint32_t *SF,
                                       const uint32_t *SI, int dir, int mode, bool sp, const PrpKernelArgs &a,
                                       const uint32_t *ybase, uint32_t *ystore, int item)
{
	constexpr bool LAST = (PASS == 2);
	const int pi = item >> 8, g = item & 255;
	int ph[16];
	addr12<PASS>(g, ph);
	const int jb = g >> 4;
	auto idx = [&](int t, int kk) {
		if (PASS == 0) return (1 << t) + kk;
		if (PASS == 1) return (1 << (4 + t)) + (jb << t) + kk;
		return ((1 << t) + kk) * 256 + g;
	};
	const uint32_t q = qv(pi), qi = qiv(pi);
	uint32_t *P = X + pi * M12;
	uint32_t u[16];
#pragma unroll
	for (int k = 0; k < 16; ++k) u[k] = P[ph[k]];
	const bool spp = sp && PASS == 0;
	if (LAST)
	{
		group_fwd<16>(u, TF + pi * M12, idx, q, qi, false, 0);
		if (!pointwise<16>(u, ph, mode, ybase + pi * M12, ystore + pi * M12, q, qi)) return;
		group_inv<16>(u, TI + pi * M12, idx, q, qi, false, 0, 0, 0);
	}
	else
	{
		// levels 0..7: Shoup pairs (w, wq) from shared memory
		const uint2 *sf = reinterpret_cast<const uint2 *>(SF) + pi * 256;
		const uint2 *si = reinterpret_cast<const uint2 *>(SI) + pi * 256;
		if (dir == 0)
		{
#pragma unroll
			for (int t = 0; t < 4; ++t)
			{
				const int half = 16 >> (t + 1);
#pragma unroll
				for (int k = 0; k < 16; ++k)
				{
					if (k & half) continue;
					if (t == 0 && spp) bf_fwd0(u[k], u[k + half], a.omega[pi], q, qi);
					else
					{
						const uint2 w = sf[idx(t, k >> (4 - t))];
						bf_fwd_s(u[k], u[k + half], w.x, w.y, q);
					}
				}
			}
		}
		else
		{
#pragma unroll
			for (int t = 3; t >= 0; --t)
			{
				const int half = 16 >> (t + 1);
#pragma unroll
				for (int k = 0; k < 16; ++k)
				{
					if (k & half) continue;
					if (t == 0 && spp) bf_inv0(u[k], u[k + half], a.omega[pi], a.k1[pi], a.sc[pi], q, qi);
					else
					{
						const uint2 w = si[idx(t, k >> (4 - t))];
						bf_inv_s(u[k], u[k + half], w.x, w.y, q);
					}
				}
			}
		}
	}
#pragma unroll
	for (int k = 0; k < 16; ++k) P[ph[k]] = u[k];
}

// NP * 256 items per pass: (prime, radix-16 group).
template <int NP>
__device__ void local_transform12(uint32_t *X, const uint32_t *TF, const uint32_t *TI, const uint32_t *SF,
                                  const uint32_t *SI, int mode, bool sp, const PrpKernelArgs &a,
                                  const uint32_t *ybase, uint32_t *ystore, int tid, int nt)
{
	for (int it = tid; it < NP * 256; it += nt) pass12<0>(X, TF, TI, SF, SI, 0, mode, sp, a, ybase, ystore, it);
	__syncthreads();
	for (int it = tid; it < NP * 256; it += nt) pass12<1>(X, TF, TI, SF, SI, 0, mode, sp, a, ybase, ystore, it);
	__syncthreads();
	for (int it = tid; it < NP * 256; it += nt) pass12<2>(X, TF, TI, SF, SI, 0, mode, sp, a, ybase, ystore, it);
	__syncthreads();
	if (mode == LM_FWD_ONLY) return;
	for (int it = tid; it < NP * 256; it += nt) pass12<1>(X, TF, TI, SF, SI, 1, mode, sp, a, ybase, ystore, it);
	__syncthreads();
	for (int it = tid; it < NP * 256; it += nt) pass12<0>(X, TF, TI, SF, SI, 1, mode, sp, a, ybase, ystore, it);
	__syncthreads();
}

// ---------------------------------------------------------------------------
// Garner and carries
// ---------------------------------------------------------------------------

typedef __int128 i128;
typedef unsigned __int128 u128;

__device__ __forceinline__ uint32_t barrett(uint64_t a, uint32_t b, uint32_t b_inv, int b_s, uint32_t &d_out)
{
	const uint32_t d = __umulhi((uint32_t)(a >> b_s), b_inv);
	const uint32_t r = (uint32_t)a - d * b;
	const bool o = (r >= b);
	d_out = o ? d + 1 : d;
	return o ? r - b : r;
}

// Truncated division f = q*b + r (|r| < b, sign of f) in two 29-bit Barrett
// steps with a one-correction quotient (reduce96/reduce64 of
// cyclo/ocl/kernel.cl:480-510).  T is int64_t or __int128.
template <class T>
__device__ __forceinline__ int32_t reduce_b(T &f, uint32_t b, uint32_t b_inv, int b_s, uint32_t &err)
{
	const bool s = f < 0;
	const u128 t = s ? (u128)(-f) : (u128)f;
	const uint64_t t_h = (uint64_t)(t >> 29);
	if (((t >> 29) >> 64) != 0 || ((t_h >> b_s) >> 32) != 0) err |= ST_BARRETT_RANGE;
	const uint32_t t_l = (uint32_t)t & ((1u << 29) - 1);
	uint32_t d_h, d_l;
	const uint32_t r_h = barrett(t_h, b, b_inv, b_s, d_h);
	const uint32_t r_l = barrett(((uint64_t)r_h << 29) | t_l, b, b_inv, b_s, d_l);
	const uint64_t d = ((uint64_t)d_h << 29) | d_l;
	f = s ? -(T)d : (T)d;
	return s ? -(int32_t)r_l : (int32_t)r_l;
}

template <>
__device__ __forceinline__ int32_t reduce_b<int64_t>(int64_t &f, uint32_t b, uint32_t b_inv, int b_s, uint32_t &err)
{
	const bool s = f < 0;
	const uint64_t t = s ? (uint64_t)(-f) : (uint64_t)f;
	const uint64_t t_h = t >> 29;
	if ((t_h >> b_s) >> 32) err |= ST_BARRETT_RANGE;
	const uint32_t t_l = (uint32_t)t & ((1u << 29) - 1);
	uint32_t d_h, d_l;
	const uint32_t r_h = barrett(t_h, b, b_inv, b_s, d_h);
	const uint32_t r_l = barrett(((uint64_t)r_h << 29) | t_l, b, b_inv, b_s, d_l);
	const uint64_t d = ((uint64_t)d_h << 29) | d_l;
	f = s ? -(int64_t)d : (int64_t)d;
	return s ? -(int32_t)r_l : (int32_t)r_l;
}

constexpr uint64_t Q21 = (uint64_t)Q2 * Q1;

// Balanced CRT value of residues r0, r1, r2 (each in [0, q)) as 96-bit two's
// complement words.  x = a0 + q2 (a1 + q1 a2) is the mixed-radix form in [0, P);
// it exceeds P/2 iff a2 > (q0-1)/2, or a2 == (q0-1)/2 and 2(a0 + q2 a1) > q2 q1.
__device__ __forceinline__ void garner3(uint32_t r0, uint32_t r1, uint32_t r2, const PrpKernelArgs &a, bool narrow,
                                        uint32_t &w0, uint32_t &w1, uint32_t &w2)
{
	const uint32_t a0 = r2;                                                     // < Q2 < Q1 < Q0
	const uint32_t a1 = mmulq(subq(r1, a0, Q1), a.ginv[0], Q1, QI1);
	const uint32_t tt = mmulq(subq(r0, a0, Q0), a.ginv[1], Q0, QI0);
	const uint32_t a2 = mmulq(subq(tt, a1, Q0), a.ginv[2], Q0, QI0);
	const uint64_t low = (uint64_t)a0 + (uint64_t)Q2 * a1;                      // < q2 q1
	const bool neg = (a2 > (Q0 - 1) / 2) || (a2 == (Q0 - 1) / 2 && 2 * low > Q21);
	if (narrow)
	{
		const uint64_t P64 = Q21 * (uint64_t)Q0;                                 // P mod 2^64
		const uint64_t v = low + Q21 * a2 - (neg ? P64 : 0);
		w0 = (uint32_t)v;
		w1 = (uint32_t)(v >> 32);
		w2 = (uint32_t)((int64_t)v >> 63);
		return;
	}
	const u128 P = (u128)Q21 * Q0;
	const u128 x = (u128)low + (u128)Q21 * a2;
	const u128 uv = neg ? (u128)((i128)x - (i128)P) : x;
	w0 = (uint32_t)uv;
	w1 = (uint32_t)(uv >> 32);
	w2 = (uint32_t)(uv >> 64);
}

// Balanced CRT value of residues r0 mod q0 and r1 mod q1 as a 64-bit two's
// complement word (two-prime launches: every product coefficient lies in
// (-q0 q1 / 2, q0 q1 / 2)).  x = r1 + q1 a1, a1 = (r0 - r1) / q1 mod q0, in [0, q0 q1).
__device__ __forceinline__ void garner2(uint32_t r0, uint32_t r1, const PrpKernelArgs &a, uint32_t &w0, uint32_t &w1)
{
	constexpr uint64_t P2 = (uint64_t)Q0 * Q1;
	const uint32_t a1 = mmulq(subq(r0, r1, Q0), a.ginv[2], Q0, QI0);   // r1 < q1 < q0
	const uint64_t x = (uint64_t)r1 + (uint64_t)Q1 * a1;
	const uint64_t v = (2 * x > P2) ? x - P2 : x;
	w0 = (uint32_t)v;
	w1 = (uint32_t)(v >> 32);
}

__device__ __forceinline__ i128 load96(const uint32_t *X, int M, int p)
{
	const uint64_t lo = (uint64_t)X[p] | ((uint64_t)X[M + p] << 32);
	const int64_t hi = (int32_t)X[2 * M + p];
	return (i128)(((u128)(uint64_t)hi << 64) | lo);
}
__device__ __forceinline__ int64_t load64(const uint32_t *X, int M, int p)
{
	return (int64_t)((uint64_t)X[p] | ((uint64_t)X[M + p] << 32));
}
__device__ __forceinline__ void store96(uint32_t *X, int M, int p, i128 v)
{
	X[p] = (uint32_t)v;
	X[M + p] = (uint32_t)(v >> 32);
	X[2 * M + p] = (uint32_t)(v >> 64);
}
__device__ __forceinline__ void store64(uint32_t *X, int M, int p, int64_t v)
{
	X[p] = (uint32_t)v;
	X[M + p] = (uint32_t)((uint64_t)v >> 32);
}
// Garner on the NP planes at word p, the result as 96-bit (NP = 3) or 64-bit words.
template <int NP>
__device__ __forceinline__ void garner_at(uint32_t *X, int M, int p, const PrpKernelArgs &a, bool narrow)
{
	uint32_t w0, w1;
	if constexpr (NP == 3)
	{
		uint32_t w2;
		garner3(X[p], X[M + p], X[2 * M + p], a, narrow, w0, w1, w2);
		X[2 * M + p] = w2;
	}
	else garner2(X[p], X[M + p], a, w0, w1);
	X[p] = w0;
	X[M + p] = w1;
}
// Residues of a digit in the NP planes at word p.
template <int NP>
__device__ __forceinline__ void to_residues(uint32_t *X, int M, int p, int32_t d)
{
	X[p] = modq_i32(d, Q0);
	X[M + p] = modq_i32(d, Q1);
	if constexpr (NP == 3) X[2 * M + p] = modq_i32(d, Q2);
}

// ---------------------------------------------------------------------------
// Cross-CTA levels 0..LG-1 through a shared-memory stage.
// Forward: pull the digit plane of columns [gbase, gbase + SC) from every CTA,
// convert to residues, radix-G transform, push the three residue planes back.
// Inverse: pull the three planes, inverse radix-G, Garner, push the 96-bit words.
// ---------------------------------------------------------------------------

template <int LG>
__device__ void cross_levels(uint32_t *X, uint32_t *ST, int M, int g, int dir, const PrpKernelArgs &a, bool narrow,
                             int tid, int nt)
{
	constexpr int G = 1 << LG;
	cg::cluster_group cl = cg::this_cluster();
	const int MG = M >> LG, SC = a.scols, nr = MG / SC, sb = a.swz_b;
	const int SC4 = SC >> 2;
	uint32_t *SD = ST;                 // [G][SC] digits (forward)
	uint32_t *SR = ST + G * SC;        // [3][G][SC] residues
	for (int rnd = 0; rnd < nr; ++rnd)
	{
		const int gbase = g * MG + rnd * SC;   // multiple of 32: physical rows == logical rows
		if (dir == 0)
		{
			for (int v = tid; v < G * SC4; v += nt)
			{
				const int h = v / SC4, o = (v - h * SC4) * 4;
				const uint4 val = *reinterpret_cast<const uint4 *>(cl.map_shared_rank(X + gbase + o, h));
				*reinterpret_cast<uint4 *>(SD + h * SC + o) = val;
			}
		}
		else
		{
			for (int v = tid; v < 3 * G * SC4; v += nt)
			{
				const int ph = v / SC4, o = (v - ph * SC4) * 4;
				const int pi = ph / G, h = ph - pi * G;
				const uint4 val = *reinterpret_cast<const uint4 *>(cl.map_shared_rank(X + pi * M + gbase + o, h));
				*reinterpret_cast<uint4 *>(SR + ph * SC + o) = val;
			}
		}
		__syncthreads();
		for (int it = tid; it < 3 * SC; it += nt)
		{
			const int pi = it / SC, tt = it - pi * SC;
			const int po = swz(gbase + tt, sb) - gbase;
			const uint32_t q = qv(pi), qi = qiv(pi);
			uint32_t v[G];
			uint32_t *S = SR + pi * G * SC + po;
			if (dir == 0)
			{
#pragma unroll
				for (int h = 0; h < G; ++h) v[h] = modq_i32((int32_t)SD[h * SC + po], q);
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
			}
			else
			{
#pragma unroll
				for (int h = 0; h < G; ++h) v[h] = S[h * SC];
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
			}
#pragma unroll
			for (int h = 0; h < G; ++h) S[h * SC] = v[h];
		}
		__syncthreads();
		if (dir == 1)
		{
			// Garner on the stage: element (h, tt) has its three residues at [pi][h][po]
			for (int e = tid; e < G * SC; e += nt)
			{
				const int h = e / SC, tt = e - h * SC;
				const int po = swz(gbase + tt, sb) - gbase;
				uint32_t *S0 = SR + h * SC + po, *S1 = S0 + G * SC, *S2 = S1 + G * SC;
				uint32_t w0, w1, w2;
				garner3(*S0, *S1, *S2, a, narrow, w0, w1, w2);
				*S0 = w0;
				*S1 = w1;
				*S2 = w2;
			}
			__syncthreads();
		}
		for (int v = tid; v < 3 * G * SC4; v += nt)
		{
			const int ph = v / SC4, o = (v - ph * SC4) * 4;
			const int pi = ph / G, h = ph - pi * G;
			const uint4 val = *reinterpret_cast<const uint4 *>(SR + ph * SC + o);
			*reinterpret_cast<uint4 *>(cl.map_shared_rank(X + pi * M + gbase + o, h)) = val;
		}
		__syncthreads();
	}
}

template <int LG>
__device__ __forceinline__ void csync()
{
	if constexpr (LG > 0) cg::this_cluster().sync();
	else __syncthreads();
}

// normalize1 over chunk c: carry of the Garner integers (x mult) into digits.
template <class T>
__device__ __forceinline__ int64_t carry_chunk(uint32_t *X, int M, int c, int csize, int sb, int mult, uint32_t b,
                                               uint32_t b_inv, int b_s, uint32_t &err)
{
	T acc = 0;
	for (int i = 0; i < csize; ++i)
	{
		const int p = swz(c * csize + i, sb);
		T v;
		if constexpr (sizeof(T) == 8) v = load64(X, M, p);
		else v = load96(X, M, p);
		acc += v * (T)mult;
		X[p] = (uint32_t)reduce_b<T>(acc, b, b_inv, b_s, err);
	}
	const int64_t f = (int64_t)acc;
	if ((T)f != acc) err |= ST_DIGIT_RANGE;
	return f;
}

}  // namespace

// Shared memory (words): planes [3][M], stage (cross levels) or chunk carries,
// carry exchange, then the CTA's roots [3][M] forward and inverse when they fit.
__host__ __device__ __forceinline__ size_t smem_stage_words(int lm, int lg, int scols)
{
	const size_t stage = lg > 0 ? (size_t)4 * ((size_t)1 << lg) * scols : 0;
	const size_t fch = ((size_t)1 << lm) / 4;     // M/8 int64 chunk carries (CSIZE >= 8)
	return stage > fch ? stage : fch;
}

template <int LG, bool M12, int NP>
__global__ void __launch_bounds__(M12 ? NP * 256 : NT_MAX, 1) prp_kernel(const PrpKernelArgs a)
{
	constexpr int G = 1 << LG;
	static_assert(NP == 3 || LG == 0, "two-prime launches use one CTA or the column layout");
	extern __shared__ __align__(16) uint32_t sm[];
	const int lm = M12 ? 12 : a.lm, M = 1 << lm, D = M * G;   // compile-time sizes on the 4096 path
	const int tid = threadIdx.x, nt = blockDim.x;
	int g = 0;
	if constexpr (LG > 0) g = (int)cg::this_cluster().block_rank();
	const int lane = blockIdx.x / G;
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
	uint32_t *SF = a.tw_smem ? TI + NP * M : TF, *SI = SF + NP * 256 * 2;   // Shoup roots of levels 0..7 (M12)
	if constexpr (M12)
	{
		const uint32_t *sfg = a.tfs + (size_t)g * 3 * 256 * 2, *sig = a.tis + (size_t)g * 3 * 256 * 2;
		for (int i = tid; i < NP * 256 * 2; i += nt) { SF[i] = sfg[i]; SI[i] = sig[i]; }
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
			if constexpr (NP == 2) f = carry_chunk<int64_t>(X, M, c, a.csize, sb, mult, b, b_inv, b_s, err);
			else f = narrow ? carry_chunk<int64_t>(X, M, c, a.csize, sb, mult, b, b_inv, b_s, err)
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
				X[p] = (uint32_t)reduce_b<int64_t>(acc, b, b_inv, b_s, err);
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

template <int LG, bool M12, int NP>
__global__ void __launch_bounds__(M12 ? NP * 256 : NT_MAX, 1) prp_kernel_cols(const PrpKernelArgs a)
{
	constexpr int G = 1 << LG;
	extern __shared__ __align__(16) uint32_t sm[];
	const int lm = M12 ? 12 : a.lm, M = 1 << lm, D = M * G, MG = M >> LG;   // compile-time on the 4096 path
	const int tid = threadIdx.x, nt = blockDim.x;
	cg::cluster_group cl = cg::this_cluster();
	const int g = (int)cl.block_rank();
	const int lane = blockIdx.x / G;
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
	uint32_t *SF = a.tw_smem ? TI + NP * M : TF, *SI = SF + NP * 256 * 2;   // Shoup roots of levels 0..7 (M12)
	if constexpr (M12)
	{
		const uint32_t *sfg = a.tfs + (size_t)g * 3 * 256 * 2, *sig = a.tis + (size_t)g * 3 * 256 * 2;
		for (int i = tid; i < NP * 256 * 2; i += nt) { SF[i] = sfg[i]; SI[i] = sig[i]; }
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
				const uint4 val = *reinterpret_cast<const uint4 *>(cl.map_shared_rank(XC + pi * M + g * MG + o, c));
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
				const uint4 val = *reinterpret_cast<const uint4 *>(cl.map_shared_rank(XR + pi * M + g * MG + o, h));
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
						Xh[p] = (uint32_t)reduce_b<int64_t>(acc, b, b_inv, b_s, err);
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
			else if (g > 0) acc = *cl.map_shared_rank(xch + h, g - 1);
			else
			{
				const int64_t last = *cl.map_shared_rank(xch + hl, G - 1);
				if (h == 0) acc = a.minus ? last : -last;
				else
				{
					acc = *cl.map_shared_rank(xch + (h - 1), G - 1);
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

int prp_threads(int lm, int np)
{
	if (lm == 12) return np * 256;  // one thread per (prime, radix-16 group)
	const int M = 1 << lm;
	int nt = np * M / 16;
	if (nt > NT_MAX) nt = NT_MAX;
	if (nt < 64) nt = 64;
	return (nt + 31) / 32 * 32;
}

template <int LG, bool M12, bool COLS, int NP>
static cudaError_t launch_lg(const PrpKernelArgs &a, int lanes, cudaStream_t stream)
{
	constexpr int G = 1 << LG;
	void (*kern)(const PrpKernelArgs);
	if constexpr (COLS) kern = prp_kernel_cols<LG, M12, NP>;
	else kern = prp_kernel<LG, M12, NP>;
	const size_t smem = prp_smem_bytes(a.lm, LG, a.tw_smem, NP);
	cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e != cudaSuccess) return e;
	if (G > 8)
	{
		e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
		if (e != cudaSuccess) return e;
	}
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3(lanes * G);
	cfg.blockDim = dim3(prp_threads(a.lm, NP));
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

bool prp_two_prime_split(int lm, int lg)
{
	return prp_split_supported(lm, lg) && (lm == 12 || lg == 0);
}

cudaError_t prp_launch(const PrpKernelArgs &a, int lg, int lanes, cudaStream_t stream)
{
	if (!prp_split_supported(a.lm, lg)) return cudaErrorInvalidValue;
	if (a.nprime == 2)
	{
		if (!prp_two_prime_split(a.lm, lg)) return cudaErrorInvalidValue;
		PrpKernelArgs a2 = a;     // two planes of roots may fit where three do not
		a2.tw_smem = prp_smem_bytes(a.lm, lg, 1, 2) <= 227 * 1024 ? 1 : 0;
		if (a.lm != 12) return launch_lg<0, false, false, 2>(a2, lanes, stream);
		switch (lg)
		{
		case 0: return launch_lg<0, true, false, 2>(a2, lanes, stream);
		case 1: return launch_lg<1, true, true, 2>(a2, lanes, stream);
		case 2: return launch_lg<2, true, true, 2>(a2, lanes, stream);
		case 3: return launch_lg<3, true, true, 2>(a2, lanes, stream);
		default: return launch_lg<4, true, true, 2>(a2, lanes, stream);
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
