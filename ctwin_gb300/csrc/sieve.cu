// Modular-root sieve for b^{2^n} - b^{2^{n-1}} +- 1 on sm_103a.
//
// "+" form (sieve/GPU/ocl/kernel.cl:243-320, sieve/CPU/ctsieve.cpp:678-726):
//   p = 3k*2^n + 1.  A generator c = a^k of order 3*2^n gives the 2^n roots of
//   Phi_{3*2^n} mod p as c^j, j = 1, 5 (mod 6), j < 3*2^n; every b = root (mod p)
//   in [b_min, b_max] is struck.
// "-" form (sieve/GPU/ocl/kernel.cl:328-479, sieve/CPU/ctsieve.cpp:728-787):
//   p = 10k +- 1, x^2 - x - 1 = 0 has roots r = (1 -+ sqrt5)/2; b are the
//   2^{n-1}-th roots of r.
//
// The reference strikes, for every prime p in range, exactly the b with
// p | N(b); a composite p that passes its base-2 filter can only strike b that
// a smaller prime factor already struck.  So the kernels keep the reference's
// filters (small factors, base-2 Euler test, which also decide the last p it
// records) and then drop composites with a deterministic Miller-Rabin test.
//
// Kernels: (1) candidates -> compacted primes, (2) per-prime generator,
// (3) root chunks -> strikes (shared-memory bitmap when the b range fits,
// else atomics on the HBM bitmap), (4) "-" form: one thread per prime.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/ctwin_gb300.h"

namespace ctw {
int fail(int code, const char *fmt, ...);
}
using ctw::fail;

namespace {

#define SV_CUDA(call)                                                                                        \
	do {                                                                                                     \
		cudaError_t e_ = (call);                                                                             \
		if (e_ != cudaSuccess) return fail(CTW_E_CUDA, "%s: %s", #call, cudaGetErrorString(e_));            \
	} while (0)

// ---------------------------------------------------------------------------
// 64-bit Montgomery arithmetic (Montgomery 1985), residues in [0, p).
// ---------------------------------------------------------------------------
struct Mp {
	uint64_t p, q, one;
};

__device__ __forceinline__ uint64_t mp_mul(const Mp &m, uint64_t a, uint64_t b)
{
	const uint64_t lo = a * b, hi = __umul64hi(a, b);
	const uint64_t mq = __umul64hi(lo * m.q, m.p);
	const uint64_t r = hi - mq;
	return (hi < mq) ? r + m.p : r;
}
__device__ __forceinline__ uint64_t mp_add(const Mp &m, uint64_t a, uint64_t b)
{
	const uint64_t c = (a >= m.p - b) ? m.p : 0;
	return a + b - c;
}
__device__ __forceinline__ uint64_t mp_sub(const Mp &m, uint64_t a, uint64_t b)
{
	const uint64_t c = (a < b) ? m.p : 0;
	return a - b + c;
}
__device__ __forceinline__ uint64_t mp_half(const Mp &m, uint64_t a) { return (a & 1) ? (a >> 1) + (m.p >> 1) + 1 : a >> 1; }
__device__ __forceinline__ uint64_t mp_toint(const Mp &m, uint64_t r)
{
	const uint64_t mq = __umul64hi(r * m.q, m.p);
	return mq ? m.p - mq : 0;
}
__device__ __forceinline__ Mp mp_make(uint64_t p)
{
	Mp m;
	m.p = p;
	uint64_t x = p;                      // p*p = 1 mod 8: 3 bits
	for (int i = 0; i < 5; ++i) x *= 2 - p * x;
	m.q = x;
	m.one = (0 - p) % p;
	return m;
}
// The same Montgomery arithmetic for p < 2^32 on 32-bit words (values travel
// as uint64_t so that the root routines below serve both widths).
struct Mp32 {
	uint32_t p, q, one;
};
__host__ __device__ __forceinline__ Mp32 mp_make32(uint32_t p)
{
	Mp32 m;
	m.p = p;
	uint32_t x = p;                      // p*p = 1 mod 8: 3 bits
	for (int i = 0; i < 4; ++i) x *= 2 - p * x;
	m.q = x;
	m.one = (0u - p) % p;
	return m;
}
__host__ __device__ __forceinline__ uint64_t mp_mul(const Mp32 &m, uint64_t a, uint64_t b)
{
	const uint64_t ab = (uint64_t)(uint32_t)a * (uint32_t)b;
	const uint32_t lo = (uint32_t)ab, hi = (uint32_t)(ab >> 32);
	const uint32_t mq = (uint32_t)(((uint64_t)(lo * m.q) * m.p) >> 32);
	const uint32_t r = hi - mq;
	return (hi < mq) ? r + m.p : r;
}
__host__ __device__ __forceinline__ uint64_t mp_add(const Mp32 &m, uint64_t a, uint64_t b)
{
	const uint32_t x = (uint32_t)a, y = (uint32_t)b;
	const uint32_t c = (x >= m.p - y) ? m.p : 0;
	return (uint32_t)(x + y - c);
}
__host__ __device__ __forceinline__ uint64_t mp_sub(const Mp32 &m, uint64_t a, uint64_t b)
{
	const uint32_t x = (uint32_t)a, y = (uint32_t)b;
	const uint32_t c = (x < y) ? m.p : 0;
	return (uint32_t)(x - y + c);
}
__host__ __device__ __forceinline__ uint64_t mp_half(const Mp32 &m, uint64_t a)
{
	return (a & 1) ? (a >> 1) + (m.p >> 1) + 1 : a >> 1;
}
__host__ __device__ __forceinline__ uint64_t mp_toint(const Mp32 &m, uint64_t r)
{
	const uint32_t mq = (uint32_t)(((uint64_t)((uint32_t)r * m.q) * m.p) >> 32);
	return mq ? m.p - mq : 0;
}
template <class M> __device__ __forceinline__ M mp_make_t(uint64_t p);
template <> __device__ __forceinline__ Mp mp_make_t<Mp>(uint64_t p) { return mp_make(p); }
template <> __device__ __forceinline__ Mp32 mp_make_t<Mp32>(uint64_t p) { return mp_make32((uint32_t)p); }

template <class M>
__device__ __forceinline__ uint64_t mp_pow(const M &m, uint64_t a, uint64_t e)
{
	uint64_t r = m.one;
	if (e == 0) return r;
	const int top = 63 - __clzll(e);
	r = a;
	for (int bit = top - 1; bit >= 0; --bit)
	{
		r = mp_mul(m, r, r);
		if ((e >> bit) & 1) r = mp_mul(m, r, a);
	}
	return r;
}
// Montgomery form of a small integer by doubling/adding from one.
template <class M>
__device__ __forceinline__ uint64_t mp_small(const M &m, uint32_t v)
{
	uint64_t r = 0, t = m.one;
	while (v)
	{
		if (v & 1) r = mp_add(m, r, t);
		t = mp_add(m, t, t);
		v >>= 1;
	}
	return r;
}

// The reference's base-2 filter: 2^((p-1)/2) == +-1 (ctsieve.cpp:368-381).
template <class M>
__device__ __forceinline__ bool euler2(const M &m)
{
	const uint64_t e = (m.p - 1) >> 1;
	const uint64_t two = mp_add(m, m.one, m.one);
	const uint64_t r = mp_pow(m, two, e);
	return r == m.one || r == m.p - m.one;
}

// Strong probable-prime test to base a.
template <class M>
__device__ bool sprp(const M &m, uint32_t a)
{
	uint64_t d = m.p - 1;
	int s = 0;
	while (!(d & 1)) { d >>= 1; ++s; }
	const uint64_t am = mp_small(m, a);
	if (am == 0) return true;
	uint64_t x = mp_pow(m, am, d);
	const uint64_t mone = m.p - m.one;
	if (x == m.one || x == mone) return true;
	for (int i = 1; i < s; ++i)
	{
		x = mp_mul(m, x, x);
		if (x == mone) return true;
		if (x == m.one) return false;
	}
	return false;
}

// Deterministic Miller-Rabin: bases {2, 7, 61} for p < 4,759,123,141 (Jaeschke
// 1993), the primes up to 17 for p < 341,550,071,728,321 and up to 37 for
// p < 2^64 (Sorenson and Webster 2015).  p is odd; a base equal to p passes.
template <class M>
__device__ bool is_prime(const M &m)
{
	const uint64_t p = m.p;
	if (p < 2) return false;
	if (p < 38) return p == 2 || p == 3 || p == 5 || p == 7 || p == 11 || p == 13 || p == 17 || p == 19 ||
	                   p == 23 || p == 29 || p == 31 || p == 37;
	if (!(p & 1)) return false;
	if (p < 4759123141ull) return sprp(m, 2) && sprp(m, 7) && (p == 61 || sprp(m, 61));
	const uint32_t bases[12] = { 2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37 };
	const int nb = p < 341550071728321ull ? 7 : 12;
	for (int i = 0; i < nb; ++i)
		if (!sprp(m, bases[i])) return false;
	return true;
}

__device__ int jacobi32(uint32_t a, uint32_t n)
{
	int k = 1;
	a %= n;
	while (a != 0)
	{
		int tz = __ffs((int)a) - 1;
		a >>= tz;
		if ((tz & 1) && ((n & 7) == 3 || (n & 7) == 5)) k = -k;
		if ((a & 3) == 3 && (n & 3) == 3) k = -k;
		const uint32_t t = a; a = n; n = t;
		a %= n;
	}
	return (n == 1) ? k : 0;
}

__device__ int jacobi(uint64_t a, uint64_t n)
{
	if (n < (1ull << 32)) return jacobi32((uint32_t)(a % n), (uint32_t)n);   // 32-bit divisions
	int k = 1;
	a %= n;
	while (a != 0)
	{
		int tz = __ffsll((long long)a) - 1;
		a >>= tz;
		if ((tz & 1) && ((n & 7) == 3 || (n & 7) == 5)) k = -k;
		if ((a & 3) == 3 && (n & 3) == 3) k = -k;
		const uint64_t t = a; a = n; n = t;
		a %= n;
	}
	return (n == 1) ? k : 0;
}

// Square root of a quadratic residue am (Montgomery form); 0 if none found.
// p = 3 mod 4: am^((p+1)/4); p = 5 mod 8: Atkin; otherwise Tonelli-Shanks.
template <class M>
__device__ uint64_t mp_sqrt(const M &m, uint64_t am)
{
	const uint64_t p = m.p;
	if (am == 0 || am == m.one) return am;
	uint64_t x;
	if ((p & 3) == 3) x = mp_pow(m, am, (p + 1) >> 2);
	else if ((p & 7) == 5)
	{
		const uint64_t b2 = mp_add(m, am, am);
		const uint64_t v = mp_pow(m, b2, (p - 5) >> 3);
		const uint64_t i = mp_mul(m, b2, mp_mul(m, v, v));
		x = mp_mul(m, mp_mul(m, am, v), mp_sub(m, i, m.one));
	}
	else
	{
		uint64_t q = p - 1;
		int s = 0;
		while (!(q & 1)) { q >>= 1; ++s; }
		uint32_t z = 2;
		while (jacobi(z, p) != -1 && z < 1000000u) ++z;
		uint64_t c = mp_pow(m, mp_small(m, z), q);
		uint64_t t = mp_pow(m, am, q);
		x = mp_pow(m, am, (q + 1) >> 1);
		int Ms = s;
		for (int guard = 0; guard < 70 && t != m.one; ++guard)
		{
			int i = 0;
			uint64_t tt = t;
			while (tt != m.one && i < Ms) { tt = mp_mul(m, tt, tt); ++i; }
			if (i == Ms) return 0;
			uint64_t bb = c;
			for (int j = 0; j < Ms - i - 1; ++j) bb = mp_mul(m, bb, bb);
			Ms = i;
			c = mp_mul(m, bb, bb);
			t = mp_mul(m, t, c);
			x = mp_mul(m, x, bb);
		}
	}
	return (mp_mul(m, x, x) == am) ? x : 0;
}

// ---------------------------------------------------------------------------
// Strikes
// ---------------------------------------------------------------------------
struct StrikeTarget {
	uint32_t *gbits;        // HBM bitmap (1 = struck), bit i <-> b_min + i
	uint64_t b_min, b_max;
	int smem_words;         // > 0: strike into a shared copy of this many words
	// factor mode (gbits == null): append (p, b) pairs, as the reference's GPU
	// sieve does (push_factor, sieve/GPU/ocl/kernel.cl:233-240)
	unsigned long long *pairs;
	uint32_t *pair_count;
	uint32_t pair_cap;
	uint32_t *status;       // bit 4 set when the pair buffer overflows
};

__device__ __forceinline__ void strike_root(const StrikeTarget &T, uint32_t *sbits, uint64_t r, uint64_t p)
{
	if (T.pairs)
	{
		// factor mode: the root itself, as push_factor(b) / push_factor(p - b)
		if (r >= T.b_min && r <= T.b_max)
		{
			const uint32_t idx = atomicAdd(T.pair_count, 1u);
			if (idx < T.pair_cap)
			{
				T.pairs[2 * (size_t)idx] = p;
				T.pairs[2 * (size_t)idx + 1] = r;
			}
			else atomicOr(T.status, 16u);
		}
		return;
	}
	// smallest s >= b_min with s = r (mod p)
	uint64_t s = r;
	if (s < T.b_min)
	{
		const uint64_t k = (T.b_min - s + p - 1) / p;
		s += k * p;
	}
	for (; s <= T.b_max; s += p)
	{
		const uint64_t i = s - T.b_min;
		if (sbits) atomicOr(&sbits[i >> 5], 1u << (i & 31));
		else atomicOr(&T.gbits[i >> 5], 1u << (i & 31));
		if (s > ~0ull - p) break;
	}
}

__device__ __forceinline__ void flush_smem_bits(const StrikeTarget &T, uint32_t *sbits)
{
	__syncthreads();
	for (int w = threadIdx.x; w < T.smem_words; w += blockDim.x)
	{
		const uint32_t v = sbits[w];
		if (v) atomicOr(&T.gbits[w], v);
	}
}

// ---------------------------------------------------------------------------
// "+" form
// ---------------------------------------------------------------------------
struct PosPrime {
	uint64_t p, k;
};

// Generator of one prime: c (Montgomery form) and, in plain form with their
// Shoup quotients floor(w 2^64 / p), the steps c^2 and c^4 of the root walk.
struct PosGen {
	uint64_t c, c2, c2q, c4, c4q;
};

// x * w mod p for any x < 2^64, w < p < 2^62 and wq = floor(w 2^64 / p), in
// plain form (V. Shoup's precomputed-quotient multiplication: x w - q p < 2p).
__device__ __forceinline__ uint64_t shoup64(uint64_t x, uint64_t w, uint64_t wq, uint64_t p)
{
	const uint64_t q = __umul64hi(x, wq);
	const uint64_t r = x * w - q * p;
	return r >= p ? r - p : r;
}
__device__ __forceinline__ uint64_t shoup64_quot(uint64_t w, uint64_t p)
{
	return (uint64_t)(((unsigned __int128)w << 64) / p);
}

// k in [k0, k0 + nk): filters of ctsieve.cpp:683-701, compaction of primes.
// Candidates pass three filters of growing cost; the survivors of each are
// compacted in shared memory so that the next, more expensive test runs on
// full warps (a warp of raw candidates almost always holds a prime).
constexpr int CAND_THREADS = 256;

__global__ void __launch_bounds__(CAND_THREADS) pos_candidates(int n, uint64_t k0, uint64_t nk, PosPrime *out,
                                                               uint32_t *count, unsigned long long *p_last,
                                                               uint32_t cap)
{
	__shared__ uint64_t q1[CAND_THREADS], q2[CAND_THREADS];
	__shared__ uint32_t n1, n2;
	for (uint64_t base = blockIdx.x * (uint64_t)CAND_THREADS; base < nk; base += (uint64_t)gridDim.x * CAND_THREADS)
	{
		if (threadIdx.x == 0) { n1 = 0; n2 = 0; }
		__syncthreads();
		const uint64_t i = base + threadIdx.x;
		if (i < nk)
		{
			const uint64_t k = k0 + i;
			const uint64_t p = 3 * (k << n) + 1;
			if (!((p % 5 == 0) || (p % 7 == 0) || (p % 11 == 0) || (p % 13 == 0) || (p % 17 == 0) || (p % 19 == 0) ||
			      (p % 23 == 0) || (p % 29 == 0) || (p % 31 == 0)))
				q1[atomicAdd(&n1, 1u)] = k;
		}
		__syncthreads();
		for (uint32_t j = threadIdx.x; j < n1; j += CAND_THREADS)
		{
			const uint64_t k = q1[j], p = 3 * (k << n) + 1;
			if (!euler2(mp_make(p))) continue;
			atomicMax(p_last, (unsigned long long)p);
			q2[atomicAdd(&n2, 1u)] = k;
		}
		__syncthreads();
		for (uint32_t j = threadIdx.x; j < n2; j += CAND_THREADS)
		{
			const uint64_t k = q2[j], p = 3 * (k << n) + 1;
			if (!is_prime(mp_make(p))) continue;
			const uint32_t idx = atomicAdd(count, 1u);
			if (idx < cap) out[idx] = PosPrime{ p, k };
		}
		__syncthreads();
	}
}

// Generator c = a^k with c^(3*2^(n-1)) = -1 and c^(2^n) != 1, i.e. of order 3*2^n.
__global__ void pos_generators(int n, const PosPrime *pr, const uint32_t *count, uint32_t cap, PosGen *gen,
                               uint32_t *status)
{
	const uint32_t cnt = min(*count, cap);
	if (*count > cap && blockIdx.x == 0 && threadIdx.x == 0) atomicOr(status, 8u);
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x)
	{
		const uint64_t p = pr[i].p, k = pr[i].k;
		const Mp m = mp_make(p);
		const uint64_t mone = p - m.one;
		uint64_t c = 0;
		for (uint32_t a = 2; a < 4096u; ++a)
		{
			if (jacobi(a, p) != -1) continue;
			const uint64_t ck = mp_pow(m, mp_small(m, a), k);
			uint64_t x = ck;                                   // x = c^(2^(n-1)) = a^((p-1)/6)
			for (int s = 0; s < n - 1; ++s) x = mp_mul(m, x, x);
			if (x == mone) continue;                         // a is a cubic residue
			c = ck;
			break;
		}
		if (c == 0) atomicOr(status, 1u);
		PosGen gv{ c, 0, 0, 0, 0 };
		if (c)
		{
			const uint64_t c2m = mp_mul(m, c, c);
			gv.c2 = mp_toint(m, c2m);
			gv.c4 = mp_toint(m, mp_mul(m, c2m, c2m));
			gv.c2q = shoup64_quot(gv.c2, p);
			gv.c4q = shoup64_quot(gv.c4, p);
		}
		gen[i] = gv;
	}
}

// Root chunks: task = (prime, chunk of t), t in [0, 2^(n-2)), four roots per t:
// +-c^(6t+1), +-c^(6t+5).  The walk stays in plain form (two Shoup products by
// c^4 and c^2 per four roots), so no root leaves Montgomery form.
__global__ void pos_roots(int n, int lchunk, const PosPrime *pr, const uint32_t *count, uint32_t cap,
                          const PosGen *gen, StrikeTarget T)
{
	extern __shared__ uint32_t sbits[];
	uint32_t *sb = T.smem_words > 0 ? sbits : nullptr;
	if (sb)
	{
		for (int w = threadIdx.x; w < T.smem_words; w += blockDim.x) sbits[w] = 0;
		__syncthreads();
	}
	const uint32_t cnt = min(*count, cap);
	const int lt = n - 2;                                  // log2 of t values per prime
	const int lc = (lchunk < lt) ? lchunk : lt;            // log2 of t values per task
	const uint64_t tasks_per_prime = 1ull << (lt - lc);
	const uint64_t ntasks = (uint64_t)cnt * tasks_per_prime;
	const uint64_t bspan = T.b_max;
	for (uint64_t task = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; task < ntasks;
	     task += (uint64_t)gridDim.x * blockDim.x)
	{
		const uint32_t ip = (uint32_t)(task >> (lt - lc));
		const uint64_t t0 = (task & (tasks_per_prime - 1)) << lc;
		const uint64_t p = pr[ip].p;
		const PosGen gv = gen[ip];
		const uint64_t c = gv.c;
		if (c == 0) continue;
		const Mp m = mp_make(p);
		const uint64_t c2 = mp_mul(m, c, c), c4 = mp_mul(m, c2, c2), c6 = mp_mul(m, c4, c2);
		uint64_t x = mp_toint(m, mp_mul(m, mp_pow(m, c6, t0), c));   // c^(6 t0 + 1), plain
		const bool small_p = p <= bspan;
		// for p > b_max a root r strikes at most r itself, when b_min <= r <= b_max,
		// and its negative p - r, when p - b_max <= r <= p - b_min: one unsigned
		// range test each
		const uint64_t span = T.b_max - T.b_min, neg_lo = p - T.b_max;
		for (uint64_t t = 0; t < (1ull << lc); ++t)
		{
			const uint64_t y = shoup64(x, gv.c4, gv.c4q, p);   // c^(6t+5)
			if (small_p)
			{
				strike_root(T, sb, x, p);
				strike_root(T, sb, p - x, p);
				strike_root(T, sb, y, p);
				strike_root(T, sb, p - y, p);
			}
			else
			{
				if (x - T.b_min <= span) strike_root(T, sb, x, p);
				if (x - neg_lo <= span) strike_root(T, sb, p - x, p);
				if (y - T.b_min <= span) strike_root(T, sb, y, p);
				if (y - neg_lo <= span) strike_root(T, sb, p - y, p);
			}
			x = shoup64(y, gv.c2, gv.c2q, p);                  // c^(6t+7)
		}
	}
	if (sb) flush_smem_bits(T, sb);
}

// ---------------------------------------------------------------------------
// "-" form
// ---------------------------------------------------------------------------

// k in [k0, k0+nk), p = 10k - 1 and 10k + 1, filters of ctsieve.cpp:741-755.
// M = Mp32 when every candidate of the launch is below 2^32.
template <class M>
__global__ void __launch_bounds__(CAND_THREADS) neg_candidates(uint64_t k0, uint64_t nk, uint64_t *out,
                                                               uint32_t *count, unsigned long long *p_last,
                                                               uint32_t cap)
{
	__shared__ uint64_t q1[CAND_THREADS], q2[CAND_THREADS];
	__shared__ uint32_t n1, n2;
	const uint64_t total = 2 * nk;
	for (uint64_t base = blockIdx.x * (uint64_t)CAND_THREADS; base < total; base += (uint64_t)gridDim.x * CAND_THREADS)
	{
		if (threadIdx.x == 0) { n1 = 0; n2 = 0; }
		__syncthreads();
		const uint64_t i = base + threadIdx.x;
		if (i < total)
		{
			const uint64_t k = k0 + (i >> 1);
			const uint64_t p = 10 * k + 2 * (i & 1) - 1;
			bool ok = !((p % 3 == 0) || (p % 7 == 0));
			if (ok && p > 31 && ((p % 11 == 0) || (p % 13 == 0) || (p % 17 == 0) || (p % 19 == 0) || (p % 23 == 0) ||
			                     (p % 29 == 0) || (p % 31 == 0)))
				ok = false;
			if (ok) q1[atomicAdd(&n1, 1u)] = p;
		}
		__syncthreads();
		for (uint32_t j = threadIdx.x; j < n1; j += CAND_THREADS)
		{
			const uint64_t p = q1[j];
			if (!euler2(mp_make_t<M>(p)) || p == 1093ull * 1093 || p == 3511ull * 3511) continue;
			atomicMax(p_last, (unsigned long long)p);
			q2[atomicAdd(&n2, 1u)] = p;
		}
		__syncthreads();
		for (uint32_t j = threadIdx.x; j < n2; j += CAND_THREADS)
		{
			const uint64_t p = q2[j];
			if (!is_prime(mp_make_t<M>(p))) continue;
			const uint32_t idx = atomicAdd(count, 1u);
			if (idx < cap) out[idx] = p;
		}
		__syncthreads();
	}
}

// All roots of b^(2^N) = a (Montgomery form), N = n - 1, struck directly.
template <class M>
__device__ void neg_sqrtn_strike(const M &m, uint64_t a, int N, const StrikeTarget &T, uint32_t *sb,
                                 uint32_t *status)
{
	const uint64_t p = m.p;
	int e = 1;
	for (uint64_t q = (p - 1) >> 1; !(q & 1); q >>= 1) ++e;    // e = v2(p-1)
	if (e > N) e = N;
	if (e > 1 && mp_pow(m, a, (p - 1) >> e) != m.one) return; // not a 2^e-th power
	// one root: repeated square roots while the 2-part allows, then the odd part
	uint64_t r = a, q = (p - 1) >> 1, mm = 1;
	for (int i = 1; i <= N; ++i)
	{
		if (!(q & 1))
		{
			r = mp_sqrt(m, r);
			q >>= 1;
			if (r == 0) break;
		}
		else
		{
			if (mm & 1) mm += q;
			mm >>= 1;
		}
	}
	if (mm > 1) r = mp_pow(m, r, mm);
	if (r == 0) { atomicOr(status, 2u); return; }
	// primitive 2^e-th root of unity from a quadratic non-residue (-1 for e = 1)
	uint64_t u = p - m.one;
	if (e > 1)
	{
		uint32_t d = 2;
		while (jacobi(d, p) != -1 && d < 1000000u) ++d;
		u = mp_pow(m, mp_small(m, d), (p - 1) >> e);
	}
	const uint64_t bspan = T.b_max;
	const bool small_p = p <= bspan;
	for (uint64_t i = 0; i < (1ull << e); i += 2)
	{
		const uint64_t bi = mp_toint(m, r);
		const uint64_t two[2] = { bi, p - bi };
#pragma unroll
		for (int j = 0; j < 2; ++j)
			if (small_p || (two[j] >= T.b_min && two[j] <= T.b_max)) strike_root(T, sb, two[j], p);
		r = mp_mul(m, r, u);
	}
}

// M = Mp32 when every prime of the launch is below 2^32.
template <class M>
__global__ void neg_roots(int n, const uint64_t *primes, const uint32_t *count, uint32_t cap, StrikeTarget T,
                          uint32_t *status)
{
	extern __shared__ uint32_t sbits[];
	uint32_t *sb = T.smem_words > 0 ? sbits : nullptr;
	if (sb)
	{
		for (int w = threadIdx.x; w < T.smem_words; w += blockDim.x) sbits[w] = 0;
		__syncthreads();
	}
	const uint32_t cnt = min(*count, cap);
	if (*count > cap && blockIdx.x == 0 && threadIdx.x == 0) atomicOr(status, 8u);
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x)
	{
		const uint64_t p = primes[i];
		const M m = mp_make_t<M>(p);
		const uint64_t five = mp_small(m, 5);
		const uint64_t s5 = mp_sqrt(m, five);
		if (s5 == 0) { atomicOr(status, 4u); continue; }
		const uint64_t r = mp_half(m, mp_sub(m, m.one, s5));          // (1 - sqrt5)/2
		const uint64_t r2 = mp_sub(m, m.one, r);                       // (1 + sqrt5)/2
		if ((p & 3) == 3)
		{
			const uint64_t rs = (jacobi(mp_toint(m, r), p) != 1) ? r2 : r;
			neg_sqrtn_strike(m, rs, n - 1, T, sb, status);
		}
		else if (jacobi(mp_toint(m, r), p) == 1)
		{
			neg_sqrtn_strike(m, r, n - 1, T, sb, status);
			neg_sqrtn_strike(m, r2, n - 1, T, sb, status);
		}
	}
	if (sb) flush_smem_bits(T, sb);
}

// ---------------------------------------------------------------------------
// Host driver
// ---------------------------------------------------------------------------
constexpr uint64_t K_BLOCK = 1ull << 22;             // candidates k per round
constexpr uint32_t PRIME_CAP = 1u << 22;
constexpr int SMEM_BITMAP_MAX_WORDS = 48 * 1024;     // 192 KB shared bitmap segment

struct SieveDev {
	uint32_t *bits = nullptr;
	void *primes = nullptr;
	PosGen *gen = nullptr;
	uint32_t *count = nullptr;
	unsigned long long *p_last = nullptr;
	uint32_t *status = nullptr;
	~SieveDev()
	{
		cudaFree(bits); cudaFree(primes); cudaFree(gen); cudaFree(count); cudaFree(p_last); cudaFree(status);
	}
};

long long g_sieve_launches = 0;

}  // namespace

extern "C" int ctw_sieve_run(int n, uint64_t b_min, uint64_t b_max, uint64_t p_min, uint64_t p_max, int mode,
                             uint32_t *struck_words, uint64_t *p_last)
{
	if (n < 8 || n > 24) return fail(CTW_E_ARG, "n = %d outside [8, 24]", n);
	if (mode != 1 && mode != -1) return fail(CTW_E_ARG, "mode must be +1 or -1");
	if (b_min < 2 || b_max < b_min) return fail(CTW_E_ARG, "b range must satisfy 2 <= b_min <= b_max");
	if (!struck_words || !p_last) return fail(CTW_E_ARG, "null output");
	if (p_max >= (1ull << 62)) return fail(CTW_E_ARG, "p_max must be below 2^62");
	if (ctw_device_count() == 0) return fail(CTW_E_CUDA, "no CUDA device");
	const uint64_t size = b_max - b_min + 1;
	if (size > (1ull << 36)) return fail(CTW_E_ARG, "b range too large");
	const uint64_t words = (size + 31) / 32;

	// k range exactly as the reference (ctsieve.cpp:682-684, 733-735)
	uint64_t k_min, k_max;
	if (mode > 0)
	{
		k_min = (p_min >> n) / 3;
		k_max = (p_max >> n) / 3;
		while (3 * (k_max << n) + 1 < p_max) ++k_max;
	}
	else
	{
		k_min = p_min / 10;
		k_max = p_max / 10;
		while (10 * k_max + 1 < p_max) ++k_max;
	}
	if (k_min < 1) k_min = 1;

	SieveDev d;
	SV_CUDA(cudaMalloc(&d.bits, words * 4));
	SV_CUDA(cudaMemcpy(d.bits, struck_words, words * 4, cudaMemcpyHostToDevice));
	SV_CUDA(cudaMalloc(&d.primes, (size_t)PRIME_CAP * 16));
	SV_CUDA(cudaMalloc(&d.gen, (size_t)PRIME_CAP * sizeof(PosGen)));
	SV_CUDA(cudaMalloc(&d.count, 4));
	SV_CUDA(cudaMalloc(&d.p_last, 8));
	SV_CUDA(cudaMalloc(&d.status, 4));
	const unsigned long long pl0 = *p_last;
	SV_CUDA(cudaMemcpy(d.p_last, &pl0, 8, cudaMemcpyHostToDevice));
	SV_CUDA(cudaMemset(d.status, 0, 4));

	int sms = 0;
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
	const bool use_smem = words <= (uint64_t)SMEM_BITMAP_MAX_WORDS;
	StrikeTarget T{ d.bits, b_min, b_max, use_smem ? (int)words : 0, nullptr, nullptr, 0, nullptr };
	const size_t smem = use_smem ? words * 4 : 0;
	if (use_smem)
	{
		SV_CUDA(cudaFuncSetAttribute(pos_roots, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
		SV_CUDA(cudaFuncSetAttribute(neg_roots<Mp>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
		SV_CUDA(cudaFuncSetAttribute(neg_roots<Mp32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	}
	// With a shared bitmap, one CTA per SM amortises its clear and flush.
	const int roots_grid = use_smem ? sms : sms * 8;
	const int lchunk = 6;

	for (uint64_t k0 = k_min; k0 <= k_max; k0 += K_BLOCK)
	{
		const uint64_t nk = std::min<uint64_t>(K_BLOCK, k_max - k0 + 1);
		SV_CUDA(cudaMemset(d.count, 0, 4));
		if (mode > 0)
		{
			pos_candidates<<<sms * 8, CAND_THREADS>>>(n, k0, nk, (PosPrime *)d.primes, d.count, d.p_last, PRIME_CAP);
			pos_generators<<<sms * 4, 128>>>(n, (PosPrime *)d.primes, d.count, PRIME_CAP, d.gen, d.status);
			pos_roots<<<roots_grid, 256, smem>>>(n, lchunk, (PosPrime *)d.primes, d.count, PRIME_CAP, d.gen, T);
			g_sieve_launches += 3;
		}
		else
		{
			if (10 * (k0 + nk) + 1 < (1ull << 32))   // 32-bit arithmetic for the whole block
				neg_candidates<Mp32><<<sms * 8, CAND_THREADS>>>(k0, nk, (uint64_t *)d.primes, d.count, d.p_last, PRIME_CAP);
			else
				neg_candidates<Mp><<<sms * 8, CAND_THREADS>>>(k0, nk, (uint64_t *)d.primes, d.count, d.p_last, PRIME_CAP);
			if (10 * (k0 + nk) + 1 < (1ull << 32))   // every prime of the block fits 32-bit arithmetic
				neg_roots<Mp32><<<roots_grid, 128, smem>>>(n, (uint64_t *)d.primes, d.count, PRIME_CAP, T, d.status);
			else
				neg_roots<Mp><<<roots_grid, 128, smem>>>(n, (uint64_t *)d.primes, d.count, PRIME_CAP, T, d.status);
			g_sieve_launches += 2;
		}
		SV_CUDA(cudaGetLastError());
	}
	SV_CUDA(cudaDeviceSynchronize());
	uint32_t st = 0;
	SV_CUDA(cudaMemcpy(&st, d.status, 4, cudaMemcpyDeviceToHost));
	if (st) return fail(CTW_E_COMPUTE, "sieve root computation failed for a prime (status 0x%x)", st);
	SV_CUDA(cudaMemcpy(struck_words, d.bits, words * 4, cudaMemcpyDeviceToHost));
	unsigned long long pl = 0;
	SV_CUDA(cudaMemcpy(&pl, d.p_last, 8, cudaMemcpyDeviceToHost));
	*p_last = pl;
	return CTW_OK;
}

extern "C" int ctw_sieve_factors(int n, uint64_t k_begin, uint64_t k_end, int mode, uint64_t b_max,
                                 uint64_t *pairs, uint64_t cap, uint64_t *count)
{
	if (n < 8 || n > 24) return fail(CTW_E_ARG, "n = %d outside [8, 24]", n);
	if (mode != 1 && mode != -1) return fail(CTW_E_ARG, "mode must be +1 or -1");
	if (!count || (!pairs && cap > 0) || k_end < k_begin || k_begin < 1) return fail(CTW_E_ARG, "bad arguments");
	if (b_max < 2) return fail(CTW_E_ARG, "b_max must be >= 2");
	const uint64_t pk = (mode > 0) ? 3 * (k_end << n) + 1 : 10 * k_end + 1;
	if (pk >= (1ull << 62) || (mode > 0 && (k_end >> (62 - n)) != 0)) return fail(CTW_E_ARG, "p must stay below 2^62");
	if (ctw_device_count() == 0) return fail(CTW_E_CUDA, "no CUDA device");
	*count = 0;
	constexpr uint32_t PAIR_CAP = 1u << 24;              // the reference's factor buffer
	SieveDev d;
	unsigned long long *dpairs = nullptr;
	SV_CUDA(cudaMalloc(&d.primes, (size_t)PRIME_CAP * 16));
	SV_CUDA(cudaMalloc(&d.gen, (size_t)PRIME_CAP * sizeof(PosGen)));
	SV_CUDA(cudaMalloc(&d.count, 8));
	SV_CUDA(cudaMalloc(&d.p_last, 8));
	SV_CUDA(cudaMalloc(&d.status, 4));
	SV_CUDA(cudaMalloc(&dpairs, (size_t)PAIR_CAP * 16));
	struct PairsFree { unsigned long long *p; ~PairsFree() { cudaFree(p); } } pf{ dpairs };
	SV_CUDA(cudaMemset(d.p_last, 0, 8));
	SV_CUDA(cudaMemset(d.status, 0, 4));
	uint32_t *pair_count = d.count + 1;
	StrikeTarget T{ nullptr, 2, b_max, 0, dpairs, pair_count, PAIR_CAP, d.status };
	int sms = 0;
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
	std::vector<unsigned long long> host;
	for (uint64_t k0 = k_begin; k0 < k_end; k0 += K_BLOCK)
	{
		const uint64_t nk = std::min<uint64_t>(K_BLOCK, k_end - k0);
		SV_CUDA(cudaMemset(d.count, 0, 8));
		if (mode > 0)
		{
			pos_candidates<<<sms * 8, CAND_THREADS>>>(n, k0, nk, (PosPrime *)d.primes, d.count, d.p_last, PRIME_CAP);
			pos_generators<<<sms * 4, 128>>>(n, (PosPrime *)d.primes, d.count, PRIME_CAP, d.gen, d.status);
			pos_roots<<<sms * 8, 256, 0>>>(n, 6, (PosPrime *)d.primes, d.count, PRIME_CAP, d.gen, T);
			g_sieve_launches += 3;
		}
		else
		{
			if (10 * (k0 + nk) + 1 < (1ull << 32))   // 32-bit arithmetic for the whole block
				neg_candidates<Mp32><<<sms * 8, CAND_THREADS>>>(k0, nk, (uint64_t *)d.primes, d.count, d.p_last, PRIME_CAP);
			else
				neg_candidates<Mp><<<sms * 8, CAND_THREADS>>>(k0, nk, (uint64_t *)d.primes, d.count, d.p_last, PRIME_CAP);
			if (10 * (k0 + nk) + 1 < (1ull << 32))
				neg_roots<Mp32><<<sms * 8, 128, 0>>>(n, (uint64_t *)d.primes, d.count, PRIME_CAP, T, d.status);
			else
				neg_roots<Mp><<<sms * 8, 128, 0>>>(n, (uint64_t *)d.primes, d.count, PRIME_CAP, T, d.status);
			g_sieve_launches += 2;
		}
		SV_CUDA(cudaGetLastError());
		uint32_t np = 0, st = 0;
		SV_CUDA(cudaMemcpy(&np, pair_count, 4, cudaMemcpyDeviceToHost));
		SV_CUDA(cudaMemcpy(&st, d.status, 4, cudaMemcpyDeviceToHost));
		if (st & 16) return fail(CTW_E_NOMEM, "more than %u factors in one block of 2^22 k", PAIR_CAP);
		if (st) return fail(CTW_E_COMPUTE, "sieve root computation failed for a prime (status 0x%x)", st);
		const size_t old = host.size();
		host.resize(old + 2 * (size_t)np);
		if (np) SV_CUDA(cudaMemcpy(host.data() + old, dpairs, (size_t)np * 16, cudaMemcpyDeviceToHost));
	}
	// deterministic order: by p, then b (the reference's order is that of its atomics)
	const size_t m = host.size() / 2;
	std::vector<size_t> ord(m);
	for (size_t i = 0; i < m; ++i) ord[i] = i;
	std::sort(ord.begin(), ord.end(), [&](size_t a, size_t b) {
		return host[2 * a] != host[2 * b] ? host[2 * a] < host[2 * b] : host[2 * a + 1] < host[2 * b + 1];
	});
	*count = m;
	if (m > cap) return fail(CTW_E_NOMEM, "%zu factors, room for %llu", m, (unsigned long long)cap);
	for (size_t i = 0; i < m; ++i)
	{
		pairs[2 * i] = host[2 * ord[i]];
		pairs[2 * i + 1] = host[2 * ord[i] + 1];
	}
	return CTW_OK;
}

extern "C" long long ctw_sieve_launches(void) { return g_sieve_launches; }

// Roofline probe of the sieve: independent chains of 64-bit Montgomery
// products (mp_mul, the sieve's inner operation) over all SMs.
__global__ void mulmod64_probe_kernel(uint64_t *out, int iters)
{
	Mp m;
	m.p = 0xFFFFFFFFFFC00001ull - 2 * (uint64_t)blockIdx.x;   // odd moduli near 2^64
	uint64_t q = m.p;                                          // p^-1 mod 2^64 (Newton)
	for (int k = 0; k < 6; ++k) q *= 2 - m.p * q;
	m.q = q;
	m.one = 0;
	uint64_t v[4];
#pragma unroll
	for (int j = 0; j < 4; ++j) v[j] = (threadIdx.x * 0x9E3779B97F4A7C15ull + j) % m.p;
	for (int i = 0; i < iters; ++i)
	{
#pragma unroll
		for (int j = 0; j < 4; ++j) v[j] = mp_mul(m, v[j], v[j]);
	}
	uint64_t x = v[0] ^ v[1] ^ v[2] ^ v[3];
	if (x == 0x123456789ull) out[0] = x;
}

extern "C" double ctw_mulmod64_peak(void)
{
	int dev = 0, sms = 0;
	if (cudaGetDevice(&dev) != cudaSuccess) return 0.0;
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	uint64_t *out = nullptr;
	if (cudaMalloc(&out, 64) != cudaSuccess) return 0.0;
	const int grid = sms * 8, block = 256, iters = 4096;
	cudaEvent_t e0, e1;
	cudaEventCreate(&e0);
	cudaEventCreate(&e1);
	mulmod64_probe_kernel<<<grid, block>>>(out, 64);
	float best = 1e30f;
	for (int rep = 0; rep < 3; ++rep)
	{
		cudaEventRecord(e0);
		mulmod64_probe_kernel<<<grid, block>>>(out, iters);
		cudaEventRecord(e1);
		cudaEventSynchronize(e1);
		float ms = 0;
		cudaEventElapsedTime(&ms, e0, e1);
		if (ms < best) best = ms;
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	cudaFree(out);
	return double(grid) * block * 4 * iters / (best * 1e-3);
}

// sv_<n>_<bmin>_<bmax>.dat and cand_<n>_<bmin>_<bmax>.txt in the reference's
// format (sieve/CPU/ctsieve.cpp:591-626): u64 p_min_pos, u64 p_min_neg,
// u64 count, u32 index[count], u32 crc32 (Rosetta CRC-32, ~crc ^ 0xa23777ac);
// the candidate file lists the survivors in increasing order, one per line.
namespace {
uint32_t crc32_update(uint32_t crc32, const void *buf, size_t len)
{
	static uint32_t table[256];
	static bool have = false;
	if (!have)
	{
		for (uint32_t i = 0; i < 256; ++i)
		{
			uint32_t rem = i;
			for (int j = 0; j < 8; ++j) rem = (rem & 1) ? (rem >> 1) ^ 0xedb88320u : rem >> 1;
			table[i] = rem;
		}
		have = true;
	}
	const uint8_t *p = (const uint8_t *)buf;
	uint32_t crc = ~crc32;
	for (size_t i = 0; i < len; ++i) crc = (crc >> 8) ^ table[(crc & 0xff) ^ p[i]];
	return ~crc;
}
}  // namespace

extern "C" int ctw_sieve_write_files(int n, uint64_t b_min, uint64_t b_max, const uint32_t *struck_words,
                                     uint64_t p_min_pos, uint64_t p_min_neg, const char *dir)
{
	if (!struck_words || b_max < b_min) return fail(CTW_E_ARG, "bad arguments");
	const uint64_t size = b_max - b_min + 1;
	std::vector<uint32_t> idx;
	for (uint64_t i = 0; i < size; ++i)
		if (!((struck_words[i >> 5] >> (i & 31)) & 1)) idx.push_back((uint32_t)i);
	const uint64_t cnt = idx.size();
	uint32_t crc = 0;
	crc = crc32_update(crc, &p_min_pos, 8);
	crc = crc32_update(crc, &p_min_neg, 8);
	crc = crc32_update(crc, &cnt, 8);
	crc = crc32_update(crc, idx.data(), idx.size() * 4);
	crc = ~crc ^ 0xa23777acu;
	const std::string base = std::string(dir ? dir : ".") + "/";
	const std::string tag = "_" + std::to_string(n) + "_" + std::to_string(b_min) + "_" + std::to_string(b_max);
	FILE *f = fopen((base + "sv" + tag + ".dat").c_str(), "wb");
	if (!f) return fail(CTW_E_ARG, "cannot write sv file");
	fwrite(&p_min_pos, 8, 1, f);
	fwrite(&p_min_neg, 8, 1, f);
	fwrite(&cnt, 8, 1, f);
	if (cnt) fwrite(idx.data(), 4, idx.size(), f);
	fwrite(&crc, 4, 1, f);
	fclose(f);
	f = fopen((base + "cand" + tag + ".txt").c_str(), "w");
	if (!f) return fail(CTW_E_ARG, "cannot write cand file");
	for (uint32_t i : idx) fprintf(f, "%llu\n", (unsigned long long)(b_min + i));
	fclose(f);
	return CTW_OK;
}
