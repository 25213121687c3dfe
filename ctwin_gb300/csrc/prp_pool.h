// Pool internals shared with the server: slot states, prepared tests and the
// tick program of one slot.
#pragma once
#include <cstdint>

#include "bignum.h"
#include "prp_kernels.cuh"

struct ctw_pool;

namespace ctw {

constexpr int POOL_TMAX = 8;       // ticks per graph launch
constexpr int POOL_SQ_CHUNK = 64;  // squarings per kernel launch within a tick
constexpr int POOL_REGS = 6;       // x/y, d, result, d(t), d(t+1), verify result

enum SlotState : int { SLOT_FREE = 0, SLOT_ACTIVE = 1, SLOT_FINISHED = 2 };

// A test with its exponent E = b^D - b^{D/2} and Gerbicz-Li block sum, ready to admit.
struct PreparedTest {
	uint32_t b = 0;
	int B = 0;
	Big E, res;
};

struct PoolSlot {
	int state = SLOT_FREE;
	int tk = 0;                // next tick of the program
	int nb = 0, kh = 0;        // main blocks, verify ticks above the low block
	long long P = 0;           // E padded to nb * B bits
	uint64_t tag = 0;
	uint32_t b = 0;
	long long squarings = 0;   // squarings and multiplies issued
	long long done_seq = -1;   // graph launch whose completion finishes the test
	PreparedTest t;
};

// One tick of one slot: register moves before the squarings and after the
// multiply, and which B exponent bits the squarings take (source 0: E,
// 1: the block sum; bits [lo, lo + B), most significant first).
struct SlotTick {
	uint32_t before = 0, after = 0;
	int source = 0;
	long long lo = 0;
	bool last = false;
};

double mono_seconds();
int gl_block_for(long long i0);
int default_gl_block(int ln);
size_t pool_slot_bytes(int ln, int B);
// Device bytes of a whole pool (slots, root tables, status), as pool creation allocates them.
size_t pool_bytes_estimate(int ln, int lg, int slots, int B);
// E = b^D - b^{D/2} (N+) or b^D - b^{D/2} - 2 (N-, minus) for D = 2^ln, and its block sum.
void slot_prepare(PreparedTest &t, int ln, int B, bool minus = false);
void slot_start(PoolSlot &s, PreparedTest &&t, uint64_t tag);
SlotTick slot_tick(PoolSlot &s, int B);

int pool_admit_prepared(ctw_pool *p, PreparedTest &&t, uint64_t tag, double t_submit);
int pool_block(const ctw_pool *p);
int pool_degree(const ctw_pool *p);
int pool_free_slots(const ctw_pool *p);
int pool_active(const ctw_pool *p);
int pool_in_flight(const ctw_pool *p);
size_t pool_bytes(const ctw_pool *p);

}  // namespace ctw
