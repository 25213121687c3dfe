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

enum SlotState : int { SLOT_FREE = 0, SLOT_MAIN = 1, SLOT_VERIFY1 = 2, SLOT_VERIFY2 = 3, SLOT_FINISHED = 4 };

struct PoolSlot {
	int state = SLOT_FREE;
	bool fresh = false;        // registers still to be set to 1
	long long pos = 0;         // main phase: index of the next exponent bit
	int j0 = -1;               // top bit of the Gerbicz-Li block sum
	uint64_t tag = 0;
	uint32_t b = 0;
	long long squarings = 0;   // squarings and multiplies issued
	long long done_seq = -1;   // graph launch whose completion finishes the test
};

// A test with its exponent E = b^D - b^{D/2} and block sum, ready to admit.
struct PreparedTest {
	uint32_t b = 0;
	int B = 0;
	Big E, res;
};

double mono_seconds();
int gl_block_for(long long i0);
int default_gl_block(int ln);
size_t pool_slot_bytes(int ln, int B);
// Device bytes of a whole pool (slots, root tables, status), as pool creation allocates them.
size_t pool_bytes_estimate(int ln, int lg, int slots, int B);
void slot_prepare(PreparedTest &t, int ln, int B);
void slot_start(PoolSlot &s, const PreparedTest &t, uint64_t tag);
bool slot_tick(PoolSlot &s, int B, int r0, PrpLaneCmd &aux, PrpLaneCmd &sq, PrpLaneCmd &mul);

int pool_admit_prepared(ctw_pool *p, const PreparedTest &t, uint64_t tag, double t_submit);
int pool_block(const ctw_pool *p);
int pool_degree(const ctw_pool *p);
int pool_free_slots(const ctw_pool *p);
int pool_active(const ctw_pool *p);
int pool_in_flight(const ctw_pool *p);
size_t pool_bytes(const ctw_pool *p);

}  // namespace ctw
