/*
 * ORACLE — test infrastructure only.  CPU restatement of the reference's PRP
 * squaring engine for ONE candidate (one "lane").  Only tests/, the smoke check
 * of __graft_entry__ and the cpu_baseline leg of bench.py may load this file's
 * library; the product never does.
 *
 * It follows the reference op for op where the register contents depend on it:
 *   - RNS primes P1, P2, P3 and generators 19, 5, 7      cyclo/src/transform.h:26-30,128-130
 *   - Montgomery multiplication (REDC with q = p^-1)       cyclo/ocl/kernel.cl:104-109
 *   - twiddle exponents 3*bitrev(j,s)+1+floor(2j/s) of a   cyclo/src/transform.h:336-368
 *     primitive 6s-th root, first split by the 6th root    cyclo/algo/algo.cpp:74-141
 *   - Garner CRT to a balanced 96-bit integer              cyclo/ocl/kernel.cl:451-460
 *   - two-step Barrett division by b (h = 1 argument)      cyclo/ocl/kernel.cl:462-510
 *   - normalize1 (chunk carry, dup = x2)                   cyclo/ocl/kernel.cl:1029-1051
 *   - normalize2 (chunk carries, wrap -f -> 0, +f -> D/2)  cyclo/ocl/kernel.cl:1053-1081
 *   - getInt / isPrime / RES64                             cyclo/src/transform.h:501-636
 *   - Gerbicz-Li block structure                           cyclo/src/cyclo.h:252-377
 * The transform itself is the scalar loop structure of cyclo/algo/algo.cpp
 * (forward DIF, pointwise square, inverse) with the kernel's Montgomery
 * arithmetic: the product modulo each prime is unique, so any correct transform
 * yields the kernel's residues exactly.
 *
 * A register is D int32 digits (the value the reference keeps as RNS residues
 * of those digits).  The multiplier `mult` of square_dup is 1 (bit clear),
 * 2 (base-2 bit set, the reference's dup) or 3 (base-3 bit set, an extension).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;
typedef __int128 i128;

#define NPRIME 3
static const uint32_t PR[NPRIME] = { 4293918721u, 4253024257u, 4231004161u };
static const uint32_t GEN[NPRIME] = { 19u, 5u, 7u };

typedef struct { uint32_t p, q, r2; } mform;

static uint32_t redc(const mform *m, uint64_t t)
{
	const uint32_t lo = (uint32_t)t, hi = (uint32_t)(t >> 32);
	const uint32_t mp = (uint32_t)(((uint64_t)(lo * m->q) * m->p) >> 32);
	return (hi < mp) ? hi - mp + m->p : hi - mp;
}
static uint32_t mmul(const mform *m, uint32_t a, uint32_t b) { return redc(m, (uint64_t)a * b); }
static uint32_t addm(uint32_t a, uint32_t b, uint32_t p) { const uint32_t c = (a >= p - b) ? p : 0; return a + b - c; }
static uint32_t subm(uint32_t a, uint32_t b, uint32_t p) { const uint32_t c = (a < b) ? p : 0; return a - b + c; }
static uint32_t mulp(uint32_t a, uint32_t b, uint32_t p) { return (uint32_t)(((uint64_t)a * b) % p); }
static uint32_t powp(uint32_t a, uint64_t e, uint32_t p)
{
	uint32_t r = 1;
	while (e) { if (e & 1) r = mulp(r, a, p); a = mulp(a, a, p); e >>= 1; }
	return r;
}
static uint32_t invp(uint32_t a, uint32_t p) { return powp(a, p - 2, p); }
static uint32_t seti(int64_t i, uint32_t p) { int64_t r = i % (int64_t)p; if (r < 0) r += p; return (uint32_t)r; }
static int32_t geti(uint32_t n, uint32_t p) { return (n > p / 2) ? (int32_t)(n - p) : (int32_t)n; }

static void mform_init(mform *m, uint32_t p)
{
	uint32_t inv = 1, prev = 0;
	while (inv != prev) { prev = inv; inv *= 2 - p * inv; }
	m->p = p; m->q = inv;
	const uint64_t r1 = ((uint64_t)1 << 32) % p;
	m->r2 = (uint32_t)((r1 * r1) % p);
}
static uint32_t to_monty(const mform *m, uint32_t a) { return mmul(m, a, m->r2); }

static size_t bitrev(size_t i, size_t n)
{
	size_t r = 0;
	for (size_t k = n, j = i; k > 1; k /= 2, j /= 2) r = (2 * r) | (j % 2);
	return r;
}

typedef struct {
	int ln;
	size_t n;
	mform mf[NPRIME];
	uint32_t *w[NPRIME];    /* Montgomery form of the forward root w[s+j]  */
	uint32_t *wi[NPRIME];   /* Montgomery form of its inverse            */
	uint32_t w1m[NPRIME];   /* Montgomery form of the 6th root w[1]       */
	uint32_t scale[NPRIME]; /* Montgomery form of 2^32 * (2/D) / (1-2w1)  */
	uint32_t invp3_p1, invp3_p2, invp2_p1; /* Garner, Montgomery form     */
} orc_prp_tables;

orc_prp_tables *orc_prp_tables_create(int ln)
{
	orc_prp_tables *t = (orc_prp_tables *)calloc(1, sizeof(orc_prp_tables));
	const size_t n = (size_t)1 << ln;
	t->ln = ln; t->n = n;
	for (int k = 0; k < NPRIME; ++k)
	{
		const uint32_t p = PR[k];
		mform_init(&t->mf[k], p);
		t->w[k] = (uint32_t *)malloc(n * sizeof(uint32_t));
		t->wi[k] = (uint32_t *)malloc(n * sizeof(uint32_t));
		t->w[k][0] = t->wi[k][0] = 0;
		for (size_t s = 1; s < n; s *= 2)
		{
			const uint32_t r_s = powp(GEN[k], (p - 1) / (6 * (uint64_t)s), p);
			for (size_t j = 0; j < s; ++j)
			{
				const uint64_t j_s = 3 * bitrev(j, s) + 1 + (2 * j) / s;
				const uint32_t w = powp(r_s, j_s, p);
				t->w[k][s + j] = to_monty(&t->mf[k], w);
				t->wi[k][s + j] = to_monty(&t->mf[k], invp(w, p));
			}
		}
		const uint32_t w1 = powp(GEN[k], (p - 1) / 6, p);
		t->w1m[k] = to_monty(&t->mf[k], w1);
		/* algo.cpp halves at every inverse stage and in the final stage: 1/D
		   overall, times d2_inv = 2/(1-2w1) halved once more ... net factor
		   (2/D)/(1-2w1).  Pointwise squares come out of Montgomery as x^2/2^32,
		   so the factor also carries 2^32. */
		const uint32_t two32 = (uint32_t)(((uint64_t)1 << 32) % p);
		uint32_t c = mulp(2, invp((uint32_t)(n % p), p), p);
		c = mulp(c, invp(subm(1, mulp(2, w1, p), p), p), p);
		c = mulp(c, two32, p);
		t->scale[k] = to_monty(&t->mf[k], c);
	}
	t->invp2_p1 = to_monty(&t->mf[0], invp(PR[1] % PR[0], PR[0]));
	t->invp3_p1 = to_monty(&t->mf[0], invp(PR[2] % PR[0], PR[0]));
	t->invp3_p2 = to_monty(&t->mf[1], invp(PR[2] % PR[1], PR[1]));
	return t;
}

void orc_prp_tables_destroy(orc_prp_tables *t)
{
	if (!t) return;
	for (int k = 0; k < NPRIME; ++k) { free(t->w[k]); free(t->wi[k]); }
	free(t);
}

/* Forward transform of one prime plane (values in [0,p), not Montgomery). */
static void forward(const orc_prp_tables *t, int k, uint32_t *P)
{
	const size_t n = t->n, n_2 = n / 2;
	const mform *m = &t->mf[k];
	const uint32_t p = m->p;
	for (size_t i = 0; i < n_2; ++i)
	{
		const uint32_t u0 = P[i], u1 = P[i + n_2], u1w = mmul(m, u1, t->w1m[k]);
		P[i] = addm(u0, u1w, p);
		P[i + n_2] = addm(u1, subm(u0, u1w, p), p);
	}
	for (size_t s = 2, mm = n_2; mm >= 2; s *= 2, mm /= 2)
	{
		for (size_t j = 0; j < s; ++j)
		{
			const uint32_t w = t->w[k][s + j];
			for (size_t i = 0, m_2 = mm / 2; i < m_2; ++i)
			{
				const size_t kk = j * mm + i;
				const uint32_t u0 = P[kk], u1w = mmul(m, P[kk + m_2], w);
				P[kk] = addm(u0, u1w, p);
				P[kk + m_2] = subm(u0, u1w, p);
			}
		}
	}
}

/* Inverse transform (no halving; the final scale folds 2/D, 1/(1-2w1), 2^32). */
static void inverse(const orc_prp_tables *t, int k, uint32_t *P)
{
	const size_t n = t->n, n_2 = n / 2;
	const mform *m = &t->mf[k];
	const uint32_t p = m->p;
	for (size_t s = n_2, mm = 2; mm <= n_2; s /= 2, mm *= 2)
	{
		for (size_t j = 0; j < s; ++j)
		{
			const uint32_t wi = t->wi[k][s + j];
			for (size_t i = 0, m_2 = mm / 2; i < m_2; ++i)
			{
				const size_t kk = j * mm + i;
				const uint32_t u0 = P[kk], u1 = P[kk + m_2];
				P[kk] = addm(u0, u1, p);
				P[kk + m_2] = mmul(m, subm(u0, u1, p), wi);
			}
		}
	}
	for (size_t i = 0; i < n_2; ++i)
	{
		const uint32_t u0 = P[i], u1 = P[i + n_2];
		const uint32_t v0 = subm(u0, mmul(m, addm(u0, u1, p), t->w1m[k]), p);
		P[i] = mmul(m, v0, t->scale[k]);
		P[i + n_2] = mmul(m, subm(u1, u0, p), t->scale[k]);
	}
}

/* Garner CRT to the balanced representative in (-P1P2P3/2, P1P2P3/2]. */
static i128 garner3(const orc_prp_tables *t, uint32_t r1, uint32_t r2, uint32_t r3)
{
	const uint32_t u13 = mmul(&t->mf[0], subm(r1, r3, PR[0]), t->invp3_p1);
	const uint32_t u23 = mmul(&t->mf[1], subm(r2, r3, PR[1]), t->invp3_p2);
	const uint32_t u123 = mmul(&t->mf[0], subm(u13, u23, PR[0]), t->invp2_p1);
	const u128 p2p3 = (u128)PR[1] * PR[2], P = p2p3 * PR[0];
	const u128 n = p2p3 * u123 + (u128)u23 * PR[2] + r3;
	return (n > P / 2) ? (i128)n - (i128)P : (i128)n;
}

/* Barrett quotient/remainder of a by b with the h = 1 argument of the kernel. */
static uint32_t barrett(uint64_t a, uint32_t b, uint32_t b_inv, int b_s, uint32_t *a_p)
{
	const uint32_t d = (uint32_t)(((uint64_t)(uint32_t)(a >> b_s) * b_inv) >> 32);
	const uint32_t r = (uint32_t)a - d * b;
	const int o = (r >= b);
	*a_p = o ? d + 1 : d;
	return o ? r - b : r;
}

/* Truncated division of f by b in two 29-bit steps; f <- quotient. */
static int32_t reduce(i128 *f, uint32_t b, uint32_t b_inv, int b_s)
{
	const int s = (*f < 0);
	const u128 t = s ? (u128)(-*f) : (u128)*f;
	const uint64_t t_h = (uint64_t)(t >> 29);
	const uint32_t t_l = (uint32_t)t & ((1u << 29) - 1);
	uint32_t d_h, d_l;
	const uint32_t r_h = barrett(t_h, b, b_inv, b_s, &d_h);
	const uint32_t r_l = barrett(((uint64_t)r_h << 29) | t_l, b, b_inv, b_s, &d_l);
	const uint64_t d = ((uint64_t)d_h << 29) | d_l;
	*f = s ? -(i128)d : (i128)d;
	return s ? -(int32_t)r_l : (int32_t)r_l;
}

static void b_params(uint32_t b, uint32_t *b_inv, int *b_s)
{
	const int s = (31 - __builtin_clz(b)) - 1;
	*b_s = s;
	*b_inv = (uint32_t)(((uint64_t)1 << (s + 32)) / b);
}

/* Carry of the Garner integers y[] (x mult) into digits x[], then the chunk
   carries with the wrap rule of x^D = x^{D/2} - 1. */
static void normalize(const orc_prp_tables *t, int32_t *x, const i128 *y, uint32_t b, int mult, int csize)
{
	const size_t n = t->n, nc = n / (size_t)csize;
	uint32_t b_inv; int b_s; b_params(b, &b_inv, &b_s);
	int64_t *f = (int64_t *)malloc(nc * sizeof(int64_t));
	for (size_t j = 0; j < nc; ++j)
	{
		i128 a = 0;
		for (int c = 0; c < csize; ++c)
		{
			const size_t k = j * csize + c;
			a += y[k] * mult;
			x[k] = reduce(&a, b, b_inv, b_s);
		}
		f[j] = (int64_t)a;
	}
	for (size_t id = 0; id < nc; ++id)
	{
		const size_t j = (id + 1) % nc;
		i128 a = f[id];
		if (j == 0) a = -a;
		else if (j == nc / 2) a += f[nc - 1];
		int c;
		int done = 0;
		for (c = 0; c < csize - 1; ++c)
		{
			const size_t k = j * csize + c;
			a += x[k];
			x[k] = reduce(&a, b, b_inv, b_s);
			if (a == 0) { done = 1; break; }
		}
		if (!done) x[j * csize + csize - 1] += (int32_t)(int64_t)a;
	}
	free(f);
}

/* x <- x^2 * mult  (mult in {1,2,3}); x holds D digits. */
void orc_square_dup(const orc_prp_tables *t, int32_t *x, uint32_t b, int mult, int csize)
{
	const size_t n = t->n;
	uint32_t *P[NPRIME];
	i128 *y = (i128 *)malloc(n * sizeof(i128));
	for (int k = 0; k < NPRIME; ++k)
	{
		P[k] = (uint32_t *)malloc(n * sizeof(uint32_t));
		for (size_t i = 0; i < n; ++i) P[k][i] = seti(x[i], PR[k]);
		forward(t, k, P[k]);
		for (size_t i = 0; i < n; ++i) P[k][i] = mmul(&t->mf[k], P[k][i], P[k][i]);
		inverse(t, k, P[k]);
	}
	for (size_t i = 0; i < n; ++i) y[i] = garner3(t, P[0][i], P[1][i], P[2][i]);
	normalize(t, x, y, b, mult, csize);
	for (int k = 0; k < NPRIME; ++k) free(P[k]);
	free(y);
}

/* Exact integer coefficients of x*y mod (X^D - X^{D/2} + 1), no carry:
   out[2i] = low 64 bits, out[2i+1] = high 64 bits (two's complement). */
void orc_poly_mul_coeffs(const orc_prp_tables *t, const int32_t *x, const int32_t *yv, int64_t *out)
{
	const size_t n = t->n;
	uint32_t *P[NPRIME], *Q = (uint32_t *)malloc(n * sizeof(uint32_t));
	for (int k = 0; k < NPRIME; ++k)
	{
		P[k] = (uint32_t *)malloc(n * sizeof(uint32_t));
		for (size_t i = 0; i < n; ++i) { P[k][i] = seti(x[i], PR[k]); Q[i] = seti(yv[i], PR[k]); }
		forward(t, k, P[k]);
		forward(t, k, Q);
		for (size_t i = 0; i < n; ++i) P[k][i] = mmul(&t->mf[k], P[k][i], Q[i]);
		inverse(t, k, P[k]);
	}
	for (size_t i = 0; i < n; ++i)
	{
		const i128 v = garner3(t, P[0][i], P[1][i], P[2][i]);
		out[2 * i] = (int64_t)(uint64_t)(u128)v;
		out[2 * i + 1] = (int64_t)(v >> 64);
	}
	for (int k = 0; k < NPRIME; ++k) free(P[k]);
	free(Q);
}

/* x <- x * y. */
void orc_mul(const orc_prp_tables *t, int32_t *x, const int32_t *yv, uint32_t b, int csize)
{
	const size_t n = t->n;
	uint32_t *P[NPRIME], *Q = (uint32_t *)malloc(n * sizeof(uint32_t));
	i128 *y = (i128 *)malloc(n * sizeof(i128));
	for (int k = 0; k < NPRIME; ++k)
	{
		P[k] = (uint32_t *)malloc(n * sizeof(uint32_t));
		for (size_t i = 0; i < n; ++i) { P[k][i] = seti(x[i], PR[k]); Q[i] = seti(yv[i], PR[k]); }
		forward(t, k, P[k]);
		forward(t, k, Q);
		for (size_t i = 0; i < n; ++i) P[k][i] = mmul(&t->mf[k], P[k][i], Q[i]);
		inverse(t, k, P[k]);
	}
	for (size_t i = 0; i < n; ++i) y[i] = garner3(t, P[0][i], P[1][i], P[2][i]);
	normalize(t, x, y, b, 1, csize);
	for (int k = 0; k < NPRIME; ++k) free(P[k]);
	free(Q); free(y);
}

/* f = f' * b + r with 0 <= r < b (transform.h:488-497). */
static uint32_t reduce_pos(int64_t *f, uint32_t b)
{
	int64_t d = *f / (int64_t)b, r = *f % (int64_t)b;
	if (r < 0) { r += b; --d; }
	*f = d;
	return (uint32_t)r;
}

/* Canonical digits of x mod N = b^D - b^{D/2} + 1, each in [0, b).  Digits are
   read as the reference does, through their balanced residue mod P3. Returns 0,
   or -1 where the reference's "getInt failed" would fire. */
int orc_get_int(size_t n, const int32_t *x_in, uint32_t b, uint32_t *x)
{
	int64_t f = 0;
	for (size_t j = 0; j < n; ++j)
	{
		int64_t e = f + geti(seti(x_in[j], PR[2]), PR[2]);
		x[j] = reduce_pos(&e, b);
		f = e;
	}
	while (f != 0)
	{
		int64_t e = -f;
		for (size_t j = 0; j < n / 2; ++j) { e += (int32_t)x[j]; x[j] = reduce_pos(&e, b); }
		e += f;
		for (size_t j = n / 2; j < n; ++j) { e += (int32_t)x[j]; x[j] = reduce_pos(&e, b); if (e == 0) break; }
		f = e;
	}
	int overflow = 1;
	for (size_t j = n - 1; j >= n / 2; --j) if (x[j] != b - 1) { overflow = 0; break; }
	if (overflow)
	{
		overflow = 0;
		for (size_t j = n / 2 - 1; j > 0; --j) if (x[j] != 0) { overflow = 1; break; }
		if (!overflow) overflow = (x[0] != 0);
	}
	if (overflow)
	{
		int32_t carry = 0;
		for (size_t j = 0; j < n / 2; ++j)
		{
			const int32_t s = (int32_t)x[j] - ((j == 0) ? 1 : 0) + carry;
			if (s < 0) { x[j] = (uint32_t)s + b; carry = -1; } else { x[j] = (uint32_t)s; carry = 0; break; }
		}
		if (carry != 0) return -1;
		for (size_t j = n / 2; j < n; ++j) x[j] = 0;
	}
	return 0;
}

/* PRP iff digits are (1,0,...,0); err iff all zero; RES64 = sum x_j b^j mod 2^64. */
int orc_is_prime(size_t n, const uint32_t *x, uint32_t b, int *prm, uint64_t *res64)
{
	int p = (x[0] == 1), err = (x[0] == 0);
	uint64_t r = x[0], bi = b;
	for (size_t j = 1; j < n; ++j)
	{
		p &= (x[j] == 0); err &= (x[j] == 0);
		r += (uint64_t)x[j] * bi; bi *= b;
	}
	*prm = p; *res64 = r;
	return err;
}

static int tstbit(const uint32_t *e, size_t nw, long i)
{
	if (i < 0 || (size_t)(i >> 5) >= nw) return 0;
	return (e[i >> 5] >> (i & 31)) & 1;
}

static int ilog2_32(uint32_t n) { return 31 - __builtin_clz(n); }

/* One whole Fermat test of b with exponent E (little-endian words, E > 0),
   including the Gerbicz-Li blocks, as cyclo::check does for one lane.
   base is 2 (reference) or 3.  Returns 0 on success, -1 on an internal error
   (the reference's "computation failed"/"getInt failed").  */
int orc_prp_check(int ln, uint32_t b, uint32_t base, const uint32_t *e, size_t nw, int csize,
                  int *is_prp, uint64_t *res64, int *gl_ok, uint32_t *digits_out)
{
	orc_prp_tables *t = orc_prp_tables_create(ln);
	const size_t n = t->n;
	const int mult = (int)base;
	long i0 = (long)nw * 32 - 1;
	while (i0 > 0 && !tstbit(e, nw, i0)) --i0;
	const int L = 2 << (ilog2_32((uint32_t)i0) / 2), B_GL = (int)((i0 - 1) / L) + 1;

	int32_t *r0 = (int32_t *)calloc(n, sizeof(int32_t)), *r1 = (int32_t *)calloc(n, sizeof(int32_t));
	int32_t *r2 = (int32_t *)calloc(n, sizeof(int32_t));
	uint32_t *c0 = (uint32_t *)malloc(n * sizeof(uint32_t)), *c1 = (uint32_t *)malloc(n * sizeof(uint32_t));
	uint32_t *c2 = (uint32_t *)malloc(n * sizeof(uint32_t));
	r0[0] = 1; r1[0] = 1;
	int rc = 0;
	for (long i = i0; i >= 0; --i)
	{
		orc_square_dup(t, r0, b, tstbit(e, nw, i) ? mult : 1, csize);
		if ((i % B_GL == 0) && (i / B_GL != 0))
		{
			memcpy(r2, r0, n * sizeof(int32_t));
			orc_mul(t, r0, r1, b, csize);
			memcpy(r1, r0, n * sizeof(int32_t));
			memcpy(r0, r2, n * sizeof(int32_t));
		}
	}
	if (orc_get_int(n, r0, b, c0)) rc = -1;

	/* d(t+1) = d(t) * result */
	memcpy(r2, r1, n * sizeof(int32_t));
	orc_mul(t, r0, r1, b, csize);
	memcpy(r1, r2, n * sizeof(int32_t));
	memcpy(r2, r0, n * sizeof(int32_t));

	/* res = sum of the B_GL-bit blocks of E */
	const size_t nres = nw + 2;
	uint32_t *res = (uint32_t *)calloc(nres, sizeof(uint32_t));
	for (long pos = 0; pos < (long)nw * 32; pos += B_GL)
	{
		for (int k = 0; k < B_GL; ++k)
		{
			if (!tstbit(e, nw, pos + k)) continue;
			/* res += 2^k */
			size_t w = (size_t)k >> 5;
			uint64_t carry = (uint64_t)1 << (k & 31);
			for (; w < nres && carry; ++w)
			{
				const uint64_t s = (uint64_t)res[w] + carry;
				res[w] = (uint32_t)s;
				carry = s >> 32;
			}
		}
	}
	long j0 = (long)nres * 32 - 1;
	while (j0 > 0 && !tstbit(res, nres, j0)) --j0;

	/* 2^res * d(t)^{2^B} */
	memset(r0, 0, n * sizeof(int32_t)); r0[0] = 1;
	for (long i = j0; i >= B_GL; --i) orc_square_dup(t, r0, b, tstbit(res, nres, i) ? mult : 1, csize);
	orc_mul(t, r0, r1, b, csize);
	for (long i = B_GL - 1; i >= 0; --i) orc_square_dup(t, r0, b, (i <= j0 && tstbit(res, nres, i)) ? mult : 1, csize);

	int prm = 0; uint64_t r64 = 0;
	if (orc_is_prime(n, c0, b, &prm, &r64)) rc = -1;
	if (orc_get_int(n, r0, b, c1)) rc = -1;
	if (orc_get_int(n, r2, b, c2)) rc = -1;
	*gl_ok = (memcmp(c1, c2, n * sizeof(uint32_t)) == 0);
	*is_prp = prm; *res64 = r64;
	if (digits_out) memcpy(digits_out, c0, n * sizeof(uint32_t));

	free(res); free(r0); free(r1); free(r2); free(c0); free(c1); free(c2);
	orc_prp_tables_destroy(t);
	return rc;
}

/* Squarings/s baseline helper: run `count` squarings (mult pattern from e) on x. */
void orc_square_loop(const orc_prp_tables *t, int32_t *x, uint32_t b, int mult, int csize,
                     const uint32_t *e, size_t nw, long i_hi, long count)
{
	for (long i = i_hi; i > i_hi - count; --i)
		orc_square_dup(t, x, b, tstbit(e, nw, i) ? mult : 1, csize);
}
