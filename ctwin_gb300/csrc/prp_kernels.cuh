// Launch interface of the PRP squaring kernels (host <-> device).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ctw {

constexpr int MAX_LG = 4;          // up to 16 CTAs (one thread-block cluster) per candidate
constexpr int MAX_G = 1 << MAX_LG;
constexpr int MAX_INLINE_LANES = 4096;  // lanes whose dup bits fit the launch parameters

enum PrpOp : int { OP_SQUARE = 0, OP_MUL = 1 };

// Per-lane command of a pool launch (PrpKernelArgs::cmd != null).  Every lane
// of one launch runs the same operation, but from its own registers and, for
// squarings, its own exponent position and count; a lane with count <= 0 is
// idle (all CTAs of its cluster return at once).
struct PrpLaneCmd {
	int32_t count;              // OP_SQUARE: squarings; OP_MUL: > 0 to take part
	int32_t i_hi;               // OP_SQUARE: index of the first bit in this lane's exponent words
	uint8_t r_in, r_y, r_out;   // register indices into regs (reg_stride words apart)
	uint8_t aux;                // prp_aux_launch: bit 0 copy r0 -> r3, bit 1 r0 <- aux_arg, bit 2 r1 <- aux_arg
	uint32_t aux_arg;
};
static_assert(sizeof(PrpLaneCmd) == 16, "PrpLaneCmd is one 16-byte load");

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
	long long i_hi;             // first (most significant) bit index processed; with cmd: squarings of
	                            // the lane's command skipped by earlier launches of the same tick
	int count;                  // squarings in this launch (OP_SQUARE); with cmd: the most per lane
	int nwords;
	int lm;                     // log2 of coefficients per CTA
	int csize;                  // carry chunk (8..64), as the reference's CSIZE
	int mult;                   // multiplier applied when a bit is set (2 = base 2, 3 = base 3)
	int op;
	int tw_smem;                // 1: copy the local roots into shared memory
	int swz_b;                  // swizzle selector of the shared planes (prp_swizzle_bit)
	int scols;                  // columns per staging round of the cross-CTA levels
	int narrow;                 // 1: |coefficients| * 3 + carries < 2^62, carry in 64-bit arithmetic
	uint32_t omega[3];          // 6th root w1 (Montgomery form)
	uint32_t k1[3];             // S / (2 w1 - 1)
	uint32_t sc[3];             // S = 2^32 * 2 / D   (Montgomery form)
	uint32_t ginv[3];           // Garner: q2^-1 mod q1, q2^-1 mod q0, q1^-1 mod q0 (Montgomery forms)
	uint32_t tcf[3][MAX_G];     // cross-CTA forward roots w[1..G-1], plain
	uint32_t tcfq[3][MAX_G];    // their Shoup quotients floor(w 2^32 / q)
	uint32_t tci[3][MAX_G];     // cross-CTA inverse roots, plain
	uint32_t tciq[3][MAX_G];
	const PrpLaneCmd *cmd;      // per-lane commands, or null for a uniform launch
	int32_t *regs;              // register file [r][lanes][D] addressed by cmd
	long long reg_stride;       // words between two registers of regs
	int use_dupmask;            // 1: the bit of lane l is bit l of dupmask (count == 1)
	uint64_t dupmask[MAX_INLINE_LANES / 64];
};

enum PrpStatus : uint32_t {
	ST_OK = 0,
	ST_BARRETT_RANGE = 1,       // quotient outside the two-step Barrett range
	ST_DIGIT_RANGE = 2,         // a digit left the int32 range
};

size_t prp_smem_bytes(int lm, int lg, int tw_smem);
// Words of the Shoup root tables of one CTA (both directions), 0 unless M = 4096.
inline size_t prp_shoup_words(int lm) { return lm == 12 ? 2 * 3 * 256 * 2 : 0; }
int prp_threads(int lm);
// Whether a cluster split D = 2^lg CTAs x 2^lm coefficients has a kernel.
bool prp_split_supported(int lm, int lg);
cudaError_t prp_launch(const PrpKernelArgs &a, int lg, int lanes, cudaStream_t stream);
// Register set-up of a pool tick (PrpLaneCmd::aux) for lanes of degree 2^ln.
cudaError_t prp_aux_launch(const PrpLaneCmd *cmd, int32_t *regs, long long reg_stride, int ln, int lanes,
                           cudaStream_t stream);

// Integer-multiply throughput probe (roofline denominator): returns IMAD/s.
double imad_peak(int device);

}  // namespace ctw
