// Launch interface of the PRP squaring kernels (host <-> device).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "prp_arith.cuh"

namespace ctw {

constexpr int MAX_LG = 4;          // up to 16 CTAs (one thread-block cluster) per candidate
constexpr int MAX_G = 1 << MAX_LG;
constexpr int MAX_INLINE_LANES = 4096;  // lanes whose dup bits fit the launch parameters

enum PrpOp : int { OP_SQUARE = 0, OP_MUL = 1 };

// Per-lane register moves of a pool tick (prp_aux_launch): ops is a bit mask
// executed in bit order, arg the value written by the set operations.
struct PrpLaneAux {
	uint32_t ops;
	uint32_t arg;
};
enum PrpAuxOp : uint32_t {
	AUX_INIT = 1,          // r0 = r1 = arg
	AUX_SAVE_D = 2,        // r3 = r1          d(t)
	AUX_SAVE_X = 4,        // r2 = r0          the result
	AUX_SAVE_D1 = 8,       // r4 = r1          d(t+1)
	AUX_SET_Y = 16,        // r0 = arg         verify accumulator
	AUX_LOAD_D = 32,       // r1 = r3          d(t) as multiply operand
	AUX_TAKE_PRODUCT = 64, // r0 = r1          y <- y * d(t)
	AUX_SAVE_Y = 128,      // r5 = r0          verify result
};

struct PrpKernelArgs {
	const int32_t *reg_in;      // [lanes][D] digits of x
	int32_t *reg_out;           // [lanes][D] digits of the result (may alias reg_in)
	const int32_t *reg_y;       // [lanes][D] digits of y (OP_MUL)
	uint32_t *scratch;          // [lanes][G][3][M] transform of y (OP_MUL)
	const uint32_t *tf;         // [3][G][M] local forward roots (Montgomery form)
	const uint32_t *ti;         // [3][G][M] local inverse roots
	const uint32_t *tfs;        // [G][3][256][2] (w, floor(w 2^32/q)) roots of local levels 0..7 (M = 4096 only)
	const uint32_t *tis;        // the same for the inverse roots
	const uint32_t *lane_b;     // [lanes][4] = b, floor(2^(s+32)/b), s = ilog2(b)-1, 1 if 64-bit carries are exact for b
	const uint32_t *bits;       // [lanes][nwords] exponent bits
	uint32_t *status;           // error flags (0 = ok)
	long long i_hi;             // first (most significant) bit index processed
	int count;                  // squarings in this launch (OP_SQUARE)
	int nwords;
	int lm;                     // log2 of coefficients per CTA
	int csize;                  // carry chunk (8..64), as the reference's CSIZE
	int mult;                   // multiplier applied when a bit is set (2 = base 2, 3 = base 3)
	int op;
	int tw_smem;                // 1: copy the local roots into shared memory
	int swz_b;                  // swizzle selector of the shared planes (prp_swizzle_bit)
	int scols;                  // columns per staging round of the cross-CTA levels
	int narrow;                 // 1: |coefficients| * 3 + carries < 2^62, carry in 64-bit arithmetic
	int minus;                  // 1: arithmetic mod N- = b^Dn - b^{Dn/2} - 1 on the transform of degree 2 Dn
	int nprime;                 // NTT primes: 3, or 2 when every product coefficient fits (prp_two_primes_exact)
	int dense;                  // two-prime cluster launches at two CTAs per SM: 0 when lanes x CTAs fill the SMs, 1 always, -1 never
	uint32_t omega[3];          // 6th root w1 (Montgomery form)
	uint32_t k1[3];             // S / (2 w1 - 1)
	uint32_t sc[3];             // S = 2^32 * 2 / D   (Montgomery form)
	uint32_t ginv[3];           // Garner: q2^-1 mod q1, q2^-1 mod q0, q1^-1 mod q0 (Montgomery forms)
	uint32_t tcf[3][MAX_G];     // cross-CTA forward roots w[1..G-1], plain
	uint32_t tcfq[3][MAX_G];    // their Shoup quotients floor(w 2^32 / q)
	uint32_t tci[3][MAX_G];     // cross-CTA inverse roots, plain
	uint32_t tciq[3][MAX_G];
	int use_dupmask;            // 1: the bit of lane l is bit l of dupmask (count == 1)
	uint64_t dupmask[MAX_INLINE_LANES / 64];
};

enum PrpStatus : uint32_t {
	ST_OK = 0,
	ST_BARRETT_RANGE = 1,       // quotient outside the two-step Barrett range
	ST_DIGIT_RANGE = 2,         // a digit left the int32 range
	ST_GRID_WAIT = 4,           // a grid wait (barrier, carry count, published word) ran out: results void
};

constexpr int GRID_BAR_WORDS = 32 + 128;

// Buffers of the grid kernel (prp_grid.cu): one candidate on G = 2^lg CTAs of a
// cooperative launch, transposes and run-end carries through L2.
struct PrpGridArgs {
	uint32_t *gx;               // [lanes][G][3][M] published column planes } zero at launch (their
	uint32_t *gr;               // [lanes][G][3][M] published row planes    } words carry a parity bit)
	long long *gc;              // [lanes][G][G] run-end carries
	unsigned *bar;              // [lanes][GRID_BAR_WORDS], zero at launch: word 0 the grid barrier
	                            // count, words 32 + g the carry publications of CTA g
	const uint32_t *xr;         // [3][2][128] cross-level roots (Montgomery): forward, inverse
	int test_mute;              // testing only: 1 + a CTA whose first publication of the launch is
	                            // skipped (its readers' waits run out); 0 in every normal launch
};
// Grid splits with a kernel: 2^lg CTAs of 2^lm coefficients for (lg, lm) =
// (5, 12), (6, 12) (D = 2^17, 2^18), (5, 11), (6, 11), (7, 11) (D = 2^16..2^18)
// and (6, 10) (D = 2^16).
bool prp_grid_supported(int lg, int lm);
// Threads of a grid CTA: one per (prime, radix-16 group) for 4096 and 2048
// coefficients, one per (prime, radix-8 group) for 1024 (measured: 2^16 +3 %
// with twice the threads, 2^17 / 2^18 -1..3 %).
__host__ __device__ constexpr int prp_grid_threads(int lm, int np)
{
	return lm == 12 ? np * 256 : (lm == 10 ? np * (1 << lm) / 8 : np * (1 << lm) / 16);
}
size_t prp_grid_smem_bytes(int lg, int lm, int tw_smem, int np);
cudaError_t prp_grid_launch(const PrpKernelArgs &a, const PrpGridArgs &ga, int lg, int lanes, cudaStream_t stream);
// Lanes of degree 2^(lm + lg) one cooperative grid launch can hold on this device.
int prp_grid_max_lanes(int lg, int lm, int np);

size_t prp_smem_bytes(int lm, int lg, int tw_smem, int np = 3);
// Words of the Shoup root tables of one CTA (both directions), 0 unless M = 4096.
inline size_t prp_shoup_words(int lm, int np = 3) { return lm == 12 ? 2 * (size_t)np * 256 * 2 : 0; }
int prp_threads(int lm, int np = 3, int lg = 0);
// Whether a cluster split D = 2^lg CTAs x 2^lm coefficients has a kernel.
bool prp_split_supported(int lm, int lg);
// Whether that split also has a two-prime kernel (one CTA, or 4096 coefficients per CTA).
bool prp_two_prime_split(int lm, int lg);

// Two primes carry the exact product when every coefficient stays inside
// (-q0 q1 / 2, q0 q1 / 2), q0 q1 = 2^59.89.  Digits satisfy |d| <= b (the carry
// leaves |d| < b, plus at most 1 in a chunk's last digit), and a coefficient
// sums at most `terms` products of two digits: 1.5 D for N+ (X^D = X^{D/2} - 1
// folds at most 1.5 D products into one coefficient) and Dn for the exact N-
// product of degree < 2 Dn.  So two primes serve b when 2 terms (b + 1)^2 < q0 q1.
inline bool prp_two_primes_exact(double terms, uint32_t bmax)
{
	const double bb = (double)bmax + 1.0;
	return 2.0 * terms * bb * bb * (1.0 + 1e-12) < (double)Q0 * (double)Q1;
}
cudaError_t prp_launch(const PrpKernelArgs &a, int lg, int lanes, cudaStream_t stream);
// The two-prime branch of prp_launch (prp_kernels_np2.cu).
cudaError_t prp_launch_np2(const PrpKernelArgs &a, int lg, int lanes, cudaStream_t stream);
// SM count of the current device (cached).
int prp_device_sms();
// Register moves of a pool tick (PrpLaneAux) for lanes of degree 2^ln; six
// register planes `reg_stride` words apart.
cudaError_t prp_aux_launch(const PrpLaneAux *aux, int32_t *regs, long long reg_stride, int ln, int lanes,
                           cudaStream_t stream);

// Integer-multiply throughput probe (roofline denominator): returns IMAD/s.
double imad_peak(int device);
double modmul_peak(int device, int kind);

}  // namespace ctw
