// Device-side building blocks of the PRP kernels (shared by prp_kernels.cu and
// prp_grid.cu): lazy modular arithmetic, radix groups and passes, the
// 4096-coefficient passes, Garner, carries and the cross-CTA stage.
#pragma once
#include <cooperative_groups.h>
#include "prp_arith.cuh"
#include "prp_kernels.cuh"

namespace ctw {

namespace cg = cooperative_groups;

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

// The same groups with Shoup pairs (w, floor(w 2^32 / q)) of plain roots.
template <int R, class Idx>
__device__ __forceinline__ void group_fwd_s(uint32_t (&u)[R], const uint2 *__restrict__ tw, Idx idx, uint32_t q)
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
			const uint2 w = tw[idx(t, k >> (r - t))];
			bf_fwd_s(u[k], u[k + half], w.x, w.y, q);
		}
	}
}
template <int R, class Idx>
__device__ __forceinline__ void group_inv_s(uint32_t (&u)[R], const uint2 *__restrict__ ti, Idx idx, uint32_t q)
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
			const uint2 w = ti[idx(t, k >> (r - t))];
			bf_inv_s(u[k], u[k + half], w.x, w.y, q);
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

// The same truncated division of a 64-bit f in one step, for the grid
// kernel's carry chains: with m = floor((2^64 - 1) / b), q = hi64(|f| m) is
// floor(|f| / b) or one less (|f| < 2^63) and the remainder fits 32 bits, so
// one correction ends it.  For b >= 64 and |f| < 2^63 the two Barrett steps of
// reduce_b<int64_t> are exact (the first step's estimate is low by less than
// 2^(2 - b_s) + 1/2 < 1, the second's by less than 1, and the range check
// needs |f| >= 2^(b_s + 61)), so both give the same quotient and remainder;
// this one has the shorter dependent chain.
__device__ __forceinline__ int32_t reduce_b64(int64_t &f, uint32_t b, uint64_t m)
{
	const bool s = f < 0;
	const uint64_t t = s ? 0 - (uint64_t)f : (uint64_t)f;
	uint64_t q = __umul64hi(t, m);
	uint32_t r = (uint32_t)t - (uint32_t)q * b;
	if (r >= b)
	{
		r -= b;
		++q;
	}
	f = s ? -(int64_t)q : (int64_t)q;
	return s ? -(int32_t)r : (int32_t)r;
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

// normalize1 over chunk c of 64-bit Garner integers (x mult): the one-step
// division of reduce_b64, b_m = floor((2^64 - 1) / b).
__device__ __forceinline__ int64_t carry_chunk64(uint32_t *X, int M, int c, int csize, int sb, int mult, uint32_t b,
                                                 uint64_t b_m)
{
	int64_t acc = 0;
	for (int i = 0; i < csize; ++i)
	{
		const int p = swz(c * csize + i, sb);
		acc += load64(X, M, p) * (int64_t)mult;
		X[p] = (uint32_t)reduce_b64(acc, b, b_m);
	}
	return acc;
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

}  // namespace ctw
