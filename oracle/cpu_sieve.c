/*
 * ORACLE — test infrastructure only.  CPU restatement of the reference CPU sieve
 * (sieve/CPU/ctsieve.cpp).  Only tests/, the smoke check of __graft_entry__ and
 * the cpu_baseline / reference legs of bench.py may load this file's library.
 *
 *   jacobi                     sieve/CPU/ctsieve.cpp:24-64
 *   Mod (slow modular ops)     :66-170
 *   MpArith (64-bit Montgomery, Tonelli-Shanks sqrt, sqrtn, prp)   :172-382
 *   check_root                 :653-676
 *   check_pos  (p = 3k2^n+1)   :678-726
 *   check_neg  (p = 10k+-1)    :728-787
 *   "ini" p limits and order   :790-811
 *
 * The bitmap holds one byte per b in [b_min, b_max]; 1 = struck.
 * orc_sieve_pos/neg with nthreads > 1 split the k range into contiguous slices,
 * each thread striking a private bitmap that is OR-ed at the end.  For every
 * prime p the reference strikes exactly the b with p | Phi(b), and a composite
 * p that passes its Fermat filter strikes only b already struck by a smaller
 * prime factor, so the union equals the sequential result.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

typedef unsigned __int128 u128;

static int jacobi(uint64_t m, uint64_t n)
{
	int k = 1;
	while (m != 0)
	{
		int odd = 0;
		while (m % 2 == 0) { m /= 2; odd = !odd; }
		if (odd && (n % 8 != 1) && (n % 8 != 7)) k = -k;
		if (m == 1) return k;
		if ((m % 4 == 3) && (n % 4 == 3)) k = -k;
		const uint64_t t = n; n = m; m = t;
		m %= n;
	}
	return 0;
}

/* ---- Mod: plain modular arithmetic ---- */
static uint64_t md_mul(uint64_t a, uint64_t b, uint64_t n) { return (uint64_t)(((u128)a * b) % n); }
static uint64_t md_sub(uint64_t a, uint64_t b, uint64_t n) { const uint64_t c = (a < b) ? n : 0; return a - b + c; }
static int ilog2_64(uint64_t x) { return 63 - __builtin_clzll(x); }
static uint64_t md_pow(uint64_t a, uint64_t e, uint64_t n)
{
	uint64_t r = a;
	for (int b = ilog2_64(e) - 1; b >= 0; --b)
	{
		r = md_mul(r, r, n);
		if (e & ((uint64_t)1 << b)) r = md_mul(r, a, n);
	}
	return r;
}
static int md_spsp(uint64_t n, uint64_t p)
{
	uint64_t r = n - 1; int k = 0;
	for (; r % 2 == 0; r /= 2) ++k;
	uint64_t x = md_pow(p, r, n);
	if (x == 1) return 1;
	for (; k > 0; --k) { if (x == n - 1) return 1; x = md_mul(x, x, n); }
	return 0;
}
/* Deterministic for n < 2^64 (bases 2..37). */
static int md_isprime(uint64_t n)
{
	static const uint64_t bases[12] = { 2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37 };
	static const uint64_t lim[12] = { 2047ull, 1373653ull, 25326001ull, 3215031751ull, 2152302898747ull,
		3474749660383ull, 341550071728321ull, 0, 3825123056546413051ull, 0, 0, 0 };
	if (n < 2) return 0;
	if (n % 2 == 0) return n == 2;
	if (n < 9) return 1;
	for (int i = 0; i < 12; ++i)
	{
		if (!md_spsp(n, bases[i])) return 0;
		if (lim[i] && n < lim[i]) return 1;
	}
	return 1;
}

/* ---- MpArith: 64-bit Montgomery ---- */
typedef struct { uint64_t p, q, one, r2; } mpa;
static uint64_t mul_hi64(uint64_t a, uint64_t b) { return (uint64_t)(((u128)a * b) >> 64); }
static uint64_t mp_redc(const mpa *m, u128 t)
{
	const uint64_t mp = mul_hi64((uint64_t)t * m->q, m->p), t_hi = (uint64_t)(t >> 64), r = t_hi - mp;
	return (t_hi < mp) ? r + m->p : r;
}
static uint64_t mp_mul(const mpa *m, uint64_t a, uint64_t b) { return mp_redc(m, (u128)a * b); }
static uint64_t mp_add(const mpa *m, uint64_t a, uint64_t b) { const uint64_t c = (a >= m->p - b) ? m->p : 0; return a + b - c; }
static uint64_t mp_sub(const mpa *m, uint64_t a, uint64_t b) { const uint64_t c = (a < b) ? m->p : 0; return a - b + c; }
static uint64_t mp_half(const mpa *m, uint64_t a) { return (a % 2 == 0) ? a / 2 : a / 2 + m->p / 2 + 1; }
static uint64_t mp_redc_short(const mpa *m, uint64_t t) { const uint64_t mp = mul_hi64(t * m->q, m->p); return (mp != 0) ? m->p - mp : 0; }
static uint64_t mp_toint(const mpa *m, uint64_t r) { return mp_redc_short(m, r); }
static uint64_t mp_pow(const mpa *m, uint64_t a, uint64_t e)
{
	uint64_t r = a;
	for (int b = ilog2_64(e) - 1; b >= 0; --b)
	{
		r = mp_mul(m, r, r);
		if (e & ((uint64_t)1 << b)) r = mp_mul(m, r, a);
	}
	return r;
}
static void mp_init(mpa *m, uint64_t p)
{
	uint64_t inv = 1, prev = 0;
	while (inv != prev) { prev = inv; inv *= 2 - p * inv; }
	m->p = p; m->q = inv; m->one = (0 - p) % p;
	uint64_t t = mp_add(m, m->one, m->one); t = mp_add(m, t, t);
	t = mp_add(m, t, t); t = mp_add(m, t, t);
	for (int i = 0; i < 4; ++i) t = mp_mul(m, t, t);
	m->r2 = t;
}
static uint64_t mp_tomp(const mpa *m, uint64_t n) { return mp_mul(m, n, m->r2); }

/* 2^((p-1)/2) == +-1 (ctsieve.cpp:368-381) */
static int mp_prp(const mpa *m)
{
	const uint64_t e = (m->p - 1) / 2;
	int b = ilog2_64(e) - 1;
	uint64_t r = mp_add(m, m->one, m->one); r = mp_add(m, r, r);
	if (e & ((uint64_t)1 << b)) r = mp_add(m, r, r);
	for (--b; b >= 0; --b)
	{
		r = mp_mul(m, r, r);
		if (e & ((uint64_t)1 << b)) r = mp_add(m, r, r);
	}
	return (r == m->one) || (r == m->p - m->one);
}

/* sqrt: 3 mod 4, 5 mod 8, else Tonelli-Shanks; 0 if none (ctsieve.cpp:258-300). */
static uint64_t mp_sqrt(const mpa *m, uint64_t a)
{
	const uint64_t p = m->p;
	if ((a == 0) || (a == m->one)) return a;
	if (p % 4 == 3) return mp_pow(m, a, (p + 1) / 4);
	if (p % 8 == 5)
	{
		const uint64_t b = mp_add(m, a, a);
		const uint64_t v = mp_pow(m, b, (p - 5) / 8);
		const uint64_t i = mp_mul(m, b, mp_mul(m, v, v));
		return mp_mul(m, mp_mul(m, a, v), mp_sub(m, i, m->one));
	}
	uint64_t q = p - 1; unsigned int e = 0; while (q % 2 == 0) { q /= 2; ++e; }
	uint64_t z = 3; while (jacobi(z, p) != -1) ++z;
	z = mp_pow(m, mp_tomp(m, z), q);
	uint64_t y = z;
	unsigned int r = e;
	uint64_t x = mp_pow(m, a, (q - 1) / 2);
	uint64_t b = mp_mul(m, a, mp_mul(m, x, x));
	x = mp_mul(m, a, x);
	for (size_t j = 0; j < 64; ++j)
	{
		if (b == m->one) return x;
		unsigned int mm = 1;
		uint64_t t = b; while (mm < r) { t = mp_mul(m, t, t); if (t == m->one) break; ++mm; }
		if (mm == r) break;
		t = y; for (size_t i = 0; i < r - 1 - mm; ++i) t = mp_mul(m, t, t);
		y = mp_mul(m, t, t);
		r = mm;
		x = mp_mul(m, x, t);
		b = mp_mul(m, b, y);
	}
	return 0;
}

/* Returns 1 and sets *s, 0 if no root, -1 on a calculation error for a prime. */
static int mp_sqrt_checked(const mpa *m, uint64_t a, uint64_t *s)
{
	*s = mp_sqrt(m, a);
	if (mp_mul(m, *s, *s) != a)
	{
		*s = 0;
		return md_isprime(m->p) ? -1 : 0;
	}
	return 1;
}

/* All n-th-power-of-2 roots of a (ctsieve.cpp:314-360); returns count, -1 on error. */
static int mp_sqrtn(const mpa *m, uint64_t a, int n, uint64_t *L, int cap)
{
	const uint64_t p = m->p;
	int e = 1; for (uint64_t q = (p - 1) / 2; q % 2 == 0; q /= 2) e++;
	if (e > n) e = n;
	if ((e > 1) && mp_pow(m, a, (p - 1) >> e) != m->one) return 0;
	uint64_t r = a, q = (p - 1) / 2, mm = 1;
	for (int i = 1; i <= n; ++i)
	{
		if (q % 2 == 0)
		{
			uint64_t s;
			if (mp_sqrt_checked(m, r, &s) < 0) return -1;
			r = s;
			q /= 2;
			if (r == 0) break;
		}
		else
		{
			if (mm % 2 != 0) mm += q;
			mm /= 2;
		}
	}
	if (mm > 1) r = mp_pow(m, r, mm);
	if (r == 0) return md_isprime(p) ? -1 : 0;
	uint64_t u = 2;
	while (1)
	{
		if (jacobi(u, p) == -1) break;
		++u; if ((u == 4) || (u == 9)) ++u;
	}
	u = mp_pow(m, mp_tomp(m, u), (p - 1) >> e);
	const int s = 1 << e;
	int cnt = 0;
	for (int i = 0; i < s; i += 2)
	{
		const uint64_t b = mp_toint(m, r);
		if (cnt + 2 > cap) return -1;
		L[cnt++] = b; L[cnt++] = p - b;
		r = mp_mul(m, r, u);
	}
	return cnt;
}

typedef struct {
	int n;
	uint64_t b_min, b_max;
	uint8_t *bits;     /* size b_max - b_min + 1 */
	int error;         /* 1 = a verification failed for a prime */
	uint64_t err_p, err_b;
} sieve_ctx;

/* 1 ok, 0 = abort this p (composite), -1 = error */
static int check_root(sieve_ctx *c, uint64_t b, uint64_t p, int is_pos)
{
	const uint64_t res = is_pos ? (p - 1) : 1;
	for (uint64_t s = b; s <= c->b_max; s += p)
	{
		if (s >= c->b_min && !c->bits[s - c->b_min])
		{
			const uint64_t x = md_pow(s, (uint64_t)1 << (c->n - 1), p), r = md_sub(md_mul(x, x, p), x, p);
			if (r == res) c->bits[s - c->b_min] = 1;
			else if (md_isprime(p)) { c->error = 1; c->err_p = p; c->err_b = s; return -1; }
			else return 0;
		}
		if (s > UINT64_MAX - p) break;
	}
	return 1;
}

static uint64_t pos_k_max(int n, uint64_t p_max)
{
	uint64_t k_max = (p_max >> n) / 3;
	if (p_max != UINT64_MAX) while (3 * (k_max << n) + 1 < p_max) ++k_max;
	return k_max;
}

/* check_pos over k in [k_lo, k_hi]; returns the last p that passed the filter, or 0 */
static uint64_t check_pos_range(sieve_ctx *c, uint64_t k_lo, uint64_t k_hi)
{
	const int n = c->n;
	uint64_t last = 0;
	for (uint64_t k = k_lo; k <= k_hi; ++k)
	{
		const uint64_t p = 3 * (k << n) + 1;
		if ((p % 5 == 0) || (p % 7 == 0) || (p % 11 == 0) || (p % 13 == 0) || (p % 17 == 0)
		 || (p % 19 == 0) || (p % 23 == 0) || (p % 29 == 0) || (p % 31 == 0)) continue;
		mpa mp; mp_init(&mp, p);
		if (!mp_prp(&mp)) continue;
		uint64_t a = 5, ma = mp_add(&mp, mp_add(&mp, mp_add(&mp, mp.one, mp.one), mp_add(&mp, mp.one, mp.one)), mp.one);
		int found = 1;
		while (1)
		{
			if ((jacobi(a, p) == -1) && (mp_pow(&mp, ma, k << (n - 1)) != p - mp.one)) break;
			++a; ma = mp_add(&mp, ma, mp.one);
			if (a % 3 == 0) { ++a; ma = mp_add(&mp, ma, mp.one); }
			if (a > (1u << 20)) { found = 0; break; }   /* composite p only */
		}
		if (found)
		{
			const uint64_t cc = mp_pow(&mp, ma, k), b2 = mp_mul(&mp, cc, cc), b4 = mp_mul(&mp, b2, b2);
			uint64_t b = mp_toint(&mp, cc);
			for (uint64_t i = 1; i < ((uint64_t)3 << (n - 1)); i += 6)
			{
				int r;
				if ((r = check_root(c, b, p, 1)) <= 0) { if (r < 0) return last; break; }
				if ((r = check_root(c, p - b, p, 1)) <= 0) { if (r < 0) return last; break; }
				b = mp_mul(&mp, b, b4);
				if ((r = check_root(c, b, p, 1)) <= 0) { if (r < 0) return last; break; }
				if ((r = check_root(c, p - b, p, 1)) <= 0) { if (r < 0) return last; break; }
				b = mp_mul(&mp, b, b2);
			}
		}
		last = p;
	}
	return last;
}

static uint64_t neg_k_max(uint64_t p_max)
{
	uint64_t k_max = p_max / 10;
	if (p_max != UINT64_MAX) while (10 * k_max + 1 < p_max) ++k_max;
	return k_max;
}

static uint64_t check_neg_range(sieve_ctx *c, uint64_t k_lo, uint64_t k_hi)
{
	const int n = c->n;
	uint64_t last = 0;
	uint64_t *L = NULL, *L1 = NULL, *L2 = NULL;
	const int cap = 2 << (n > 1 ? n - 1 : 1);
	L = (uint64_t *)malloc(sizeof(uint64_t) * 2 * cap);
	L1 = (uint64_t *)malloc(sizeof(uint64_t) * cap);
	L2 = (uint64_t *)malloc(sizeof(uint64_t) * cap);
	for (uint64_t k = k_lo; k <= k_hi; ++k)
	{
		for (uint64_t i = 0; i <= 1; ++i)
		{
			const uint64_t p = 10 * k + 2 * i - 1;
			if ((p % 3 == 0) || (p % 7 == 0)) continue;
			if (p > 31)
			{
				if ((p % 11 == 0) || (p % 13 == 0) || (p % 17 == 0) || (p % 19 == 0)
				 || (p % 23 == 0) || (p % 29 == 0) || (p % 31 == 0)) continue;
			}
			mpa mp; mp_init(&mp, p);
			if (!(mp_prp(&mp) && (p != 1093ull * 1093) && (p != 3511ull * 3511))) continue;
			int cnt = 0;
			uint64_t s5;
			const int sr = mp_sqrt_checked(&mp, mp_tomp(&mp, 5), &s5);
			if (sr < 0) { c->error = 1; c->err_p = p; goto done; }
			if (sr > 0 && s5 != 0)
			{
				const uint64_t r = mp_half(&mp, mp_sub(&mp, mp.one, s5));
				if (p % 4 == 3)
				{
					const uint64_t rs = (jacobi(mp_toint(&mp, r), p) != 1) ? mp_sub(&mp, mp.one, r) : r;
					cnt = mp_sqrtn(&mp, rs, n - 1, L, 2 * cap);
				}
				else if (jacobi(mp_toint(&mp, r), p) == 1)
				{
					const int c1 = mp_sqrtn(&mp, r, n - 1, L1, cap);
					const int c2 = mp_sqrtn(&mp, mp_sub(&mp, mp.one, r), n - 1, L2, cap);
					if (c1 < 0 || c2 < 0) cnt = -1;
					else { memcpy(L, L1, sizeof(uint64_t) * c1); memcpy(L + c1, L2, sizeof(uint64_t) * c2); cnt = c1 + c2; }
				}
				if (cnt < 0) { c->error = 1; c->err_p = p; goto done; }
			}
			for (int j = 0; j < cnt; ++j)
			{
				const int r = check_root(c, L[j], p, 0);
				if (r < 0) goto done;
				if (r == 0) break;
			}
			last = p;
		}
	}
done:
	free(L); free(L1); free(L2);
	return last;
}

typedef struct {
	sieve_ctx c;
	uint64_t k_lo, k_hi, last;
	int pos;
} worker;

static void *run_worker(void *arg)
{
	worker *w = (worker *)arg;
	w->last = w->pos ? check_pos_range(&w->c, w->k_lo, w->k_hi) : check_neg_range(&w->c, w->k_lo, w->k_hi);
	return NULL;
}

/* mode +1: check_pos from p_min to p_max; -1: check_neg.  bits: caller's bitmap
   (1 = struck), updated in place.  *p_last <- last p processed (unchanged if none).
   Returns 0, or -1 on a calculation error (err_pb[0..1] = p, b). */
int orc_sieve(int n, uint64_t b_min, uint64_t b_max, uint64_t p_min, uint64_t p_max, int mode,
              uint8_t *bits, int nthreads, uint64_t *p_last, uint64_t *err_pb)
{
	uint64_t k_min, k_max;
	if (mode > 0) { k_min = (p_min >> n) / 3; k_max = pos_k_max(n, p_max); }
	else { k_min = p_min / 10; k_max = neg_k_max(p_max); }
	if (k_min < 1) k_min = 1;   /* k = 0 gives p = 1 or p = -1 */
	if (nthreads < 1) nthreads = 1;
	const uint64_t size = b_max - b_min + 1;
	const uint64_t nk = (k_max >= k_min) ? k_max - k_min + 1 : 0;
	if ((uint64_t)nthreads > nk) nthreads = nk ? (int)nk : 1;
	worker *ws = (worker *)calloc((size_t)nthreads, sizeof(worker));
	pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
	for (int t = 0; t < nthreads; ++t)
	{
		worker *w = &ws[t];
		w->c.n = n; w->c.b_min = b_min; w->c.b_max = b_max;
		w->c.bits = (nthreads == 1) ? bits : (uint8_t *)calloc(size, 1);
		if (nthreads > 1) memcpy(w->c.bits, bits, size);
		w->k_lo = k_min + nk * (uint64_t)t / (uint64_t)nthreads;
		w->k_hi = k_min + nk * (uint64_t)(t + 1) / (uint64_t)nthreads - 1;
		w->pos = (mode > 0);
		if (nk == 0) { w->k_lo = 1; w->k_hi = 0; }
	}
	if (nthreads == 1) run_worker(&ws[0]);
	else
	{
		for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, run_worker, &ws[t]);
		for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
	}
	int rc = 0;
	for (int t = 0; t < nthreads; ++t)
	{
		worker *w = &ws[t];
		if (nthreads > 1)
		{
			for (uint64_t i = 0; i < size; ++i) bits[i] |= w->c.bits[i];
			free(w->c.bits);
		}
		if (w->last > *p_last) *p_last = w->last;
		if (w->c.error && rc == 0) { rc = -1; if (err_pb) { err_pb[0] = w->c.err_p; err_pb[1] = w->c.err_b; } }
	}
	free(ws); free(th);
	return rc;
}

/* Rosetta-code CRC-32 as used by the sv_*.dat trailer (ctsieve.cpp:497-533). */
uint32_t orc_crc32(uint32_t crc32, const uint8_t *buf, size_t len)
{
	static uint32_t table[256];
	static int have = 0;
	if (!have)
	{
		for (uint32_t i = 0; i < 256; ++i)
		{
			uint32_t rem = i;
			for (int j = 0; j < 8; ++j) rem = (rem & 1) ? (rem >> 1) ^ 0xedb88320u : rem >> 1;
			table[i] = rem;
		}
		have = 1;
	}
	uint32_t crc = ~crc32;
	for (size_t i = 0; i < len; ++i) crc = (crc >> 8) ^ table[(crc & 0xff) ^ buf[i]];
	return ~crc;
}
