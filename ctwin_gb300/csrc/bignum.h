// Minimal unsigned multiprecision integers for the PRP exponent
// E = b^D - b^{D/2} (cyclo/src/cyclo.h:254-272 builds it with GMP) and the
// Gerbicz-Li block sums (cyclo/src/cyclo.h:315-337).  Little-endian 32-bit
// limbs, Karatsuba above a schoolbook threshold.
#pragma once
#include <algorithm>
#include <cstdint>
#include <vector>

namespace ctw {

using Big = std::vector<uint32_t>;

inline void big_trim(Big &a) { while (!a.empty() && a.back() == 0) a.pop_back(); }

inline Big big_from_u64(uint64_t v)
{
	Big r;
	while (v) { r.push_back((uint32_t)v); v >>= 32; }
	return r;
}

inline Big big_add(const Big &a, const Big &b)
{
	const Big &x = a.size() >= b.size() ? a : b, &y = a.size() >= b.size() ? b : a;
	Big r(x.size() + 1, 0);
	uint64_t c = 0;
	for (size_t i = 0; i < x.size(); ++i)
	{
		const uint64_t s = (uint64_t)x[i] + (i < y.size() ? y[i] : 0) + c;
		r[i] = (uint32_t)s;
		c = s >> 32;
	}
	r[x.size()] = (uint32_t)c;
	big_trim(r);
	return r;
}

// a -= b, requires a >= b
inline void big_sub_inplace(Big &a, const Big &b)
{
	int64_t borrow = 0;
	for (size_t i = 0; i < a.size(); ++i)
	{
		int64_t s = (int64_t)a[i] - (i < b.size() ? (int64_t)b[i] : 0) - borrow;
		borrow = s < 0;
		if (s < 0) s += ((int64_t)1 << 32);
		a[i] = (uint32_t)s;
	}
	big_trim(a);
}

// r[shift..] += v
inline void big_add_shifted(Big &r, const Big &v, size_t shift)
{
	if (r.size() < v.size() + shift + 1) r.resize(v.size() + shift + 1, 0);
	uint64_t c = 0;
	size_t i = 0;
	for (; i < v.size(); ++i)
	{
		const uint64_t s = (uint64_t)r[i + shift] + v[i] + c;
		r[i + shift] = (uint32_t)s;
		c = s >> 32;
	}
	for (size_t k = i + shift; c && k < r.size(); ++k)
	{
		const uint64_t s = (uint64_t)r[k] + c;
		r[k] = (uint32_t)s;
		c = s >> 32;
	}
	if (c) r.push_back((uint32_t)c);
}

inline Big big_mul_school(const Big &a, const Big &b)
{
	if (a.empty() || b.empty()) return Big();
	Big r(a.size() + b.size(), 0);
	for (size_t i = 0; i < a.size(); ++i)
	{
		uint64_t c = 0;
		const uint64_t ai = a[i];
		for (size_t j = 0; j < b.size(); ++j)
		{
			const uint64_t t = ai * b[j] + r[i + j] + c;
			r[i + j] = (uint32_t)t;
			c = t >> 32;
		}
		r[i + b.size()] = (uint32_t)c;
	}
	big_trim(r);
	return r;
}

inline Big big_mul(const Big &a, const Big &b)
{
	constexpr size_t K = 40;
	if (a.size() < K || b.size() < K) return big_mul_school(a, b);
	const size_t m = std::max(a.size(), b.size()) / 2;
	auto lo = [m](const Big &x) { Big r(x.begin(), x.begin() + std::min(m, x.size())); big_trim(r); return r; };
	auto hi = [m](const Big &x) { return x.size() > m ? Big(x.begin() + m, x.end()) : Big(); };
	const Big a0 = lo(a), a1 = hi(a), b0 = lo(b), b1 = hi(b);
	const Big z0 = big_mul(a0, b0), z2 = big_mul(a1, b1);
	Big z1 = big_mul(big_add(a0, a1), big_add(b0, b1));
	big_sub_inplace(z1, z0);
	big_sub_inplace(z1, z2);
	Big r = z0;
	big_add_shifted(r, z1, m);
	big_add_shifted(r, z2, 2 * m);
	big_trim(r);
	return r;
}

inline size_t big_bitlen(const Big &a)
{
	if (a.empty()) return 0;
	return 32 * (a.size() - 1) + (32 - __builtin_clz(a.back()));
}

inline int big_bit(const Big &a, long long i)
{
	if (i < 0 || (size_t)(i >> 5) >= a.size()) return 0;
	return (a[(size_t)(i >> 5)] >> (i & 31)) & 1;
}

// b^(2^k)
inline Big big_pow2k(uint32_t b, int k)
{
	Big r = big_from_u64(b);
	for (int i = 0; i < k; ++i) r = big_mul(r, r);
	return r;
}

// E = b^D - b^{D/2}, D = 2^ln
inline Big prp_exponent(uint32_t b, int ln)
{
	Big h = big_pow2k(b, ln - 1);
	Big e = big_mul(h, h);
	big_sub_inplace(e, h);
	return e;
}

// Sum of the B-bit blocks of e (Gerbicz-Li residue exponent).
inline Big big_block_sum(const Big &e, int B)
{
	Big res;
	const size_t nb = big_bitlen(e);
	for (size_t pos = 0; pos < nb; pos += (size_t)B)
	{
		Big blk((size_t)(B + 31) / 32 + 1, 0);
		for (int k = 0; k < B; ++k)
			if (big_bit(e, (long long)(pos + k))) blk[(size_t)k >> 5] |= 1u << (k & 31);
		big_trim(blk);
		res = big_add(res, blk);
	}
	return res;
}

}  // namespace ctw
