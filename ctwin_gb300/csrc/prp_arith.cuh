// Modular and wide-integer arithmetic shared by the PRP kernels (device) and the
// host-side table generation (host).  Three NTT primes q = c*3*2^20 + 1 < 2^30,
// so residues and sums of two residues fit 31 bits and the unsigned-min trick
// reduces a sum with one subtraction.
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define CTW_HD __host__ __device__ __forceinline__
#else
#define CTW_HD inline
#endif

namespace ctw {

constexpr int NPRIME = 3;
// q0 = 335*3*2^20+1, q1 = 322*3*2^20+1, q2 = 310*3*2^20+1 (all prime, 3*2^20 | q-1).
constexpr uint32_t Q0 = 1053818881u, Q1 = 1012924417u, Q2 = 975175681u;
constexpr uint32_t QGEN0 = 7u, QGEN1 = 5u, QGEN2 = 17u;   // primitive roots

CTW_HD uint32_t umin32(uint32_t a, uint32_t b) { return a < b ? a : b; }
CTW_HD uint32_t mulhi32(uint32_t a, uint32_t b)
{
#if defined(__CUDA_ARCH__)
	return __umulhi(a, b);
#else
	return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

// a + b mod q, a, b in [0, q)
CTW_HD uint32_t addq(uint32_t a, uint32_t b, uint32_t q) { const uint32_t r = a + b; return umin32(r, r - q); }
// a - b mod q, a, b in [0, q)
CTW_HD uint32_t subq(uint32_t a, uint32_t b, uint32_t q) { const uint32_t r = a - b + q; return umin32(r, r - q); }

// Montgomery product a*b/2^32 mod q for any a < 2^32 and b < q (qi = q^-1 mod 2^32).
// (P. L. Montgomery, Modular multiplication without trial division, 1985.)
CTW_HD uint32_t mmulq(uint32_t a, uint32_t b, uint32_t q, uint32_t qi)
{
	const uint64_t p = (uint64_t)a * b;            // one wide product for lo and hi
	const uint32_t lo = (uint32_t)p, hi = (uint32_t)(p >> 32);
	const uint32_t mq = mulhi32(lo * qi, q);
	const uint32_t r = hi - mq + q;
	return umin32(r, r - q);
}

// Residue of a signed 32-bit digit modulo q (q in (2^29, 2^30)).
CTW_HD uint32_t modq_i32(int32_t d, uint32_t q)
{
	uint32_t u = (d < 0) ? (uint32_t)d + 4u * q : (uint32_t)d;   // [0, 4q), mod 2^32 arithmetic
	u = umin32(u, u - 2 * q);
	return umin32(u, u - q);
}

}  // namespace ctw
