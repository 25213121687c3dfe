/*
 * ctwin_gb300 — GB300 (sm_103a) engine for the two data-parallel hot paths of
 * galloty/ctwin: the cyclotomic PRP squaring engine and the modular-root sieve.
 *
 * C ABI.  Plain pointers and sizes; every function returns 0 on success or a
 * negative CTW_E* code, and never exits or throws (the reference's engine calls
 * exit() on OpenCL errors, cyclo/src/ocl.h:106-113).  ctw_last_error() gives the
 * message of the last failure on the calling thread.  Handles are opaque, owned
 * by the caller, not thread-safe; each PRP handle owns one CUDA stream.
 * All citations are paths inside the reference project.
 */
#ifndef CTWIN_GB300_H
#define CTWIN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CTW_OK 0
#define CTW_E_ARG (-1)        /* invalid argument */
#define CTW_E_CUDA (-2)       /* CUDA runtime error (no device, launch failure, ...) */
#define CTW_E_NOMEM (-3)      /* device or host allocation failed */
#define CTW_E_COMPUTE (-4)    /* arithmetic self-check failed (range, getInt, zero residue) */
#define CTW_E_GERBICZ (-5)    /* Gerbicz-Li check failed */
#define CTW_STOPPED 1         /* a run stopped at a checkpoint on request (not an error) */

const char *ctw_last_error(void);
/* Library version string. */
const char *ctw_version(void);
/* Number of visible CUDA devices (0 when none); never fails. */
int ctw_device_count(void);

/* ------------------------------------------------------------------------ */
/* PRP engine: Fermat test of N = Phi_{3*2^n}(b) = b^D - b^{D/2} + 1, D = 2^n */
/* ------------------------------------------------------------------------ */

typedef struct ctw_prp ctw_prp;

/* Create an engine for degree D = 2^log2_degree (8..18) and `lanes` candidates
 * of that degree (the reference uses 64 lanes, VSIZE).  Registers 0..2 hold
 * one residue per lane each, initialised to 0.
 * Replaces: engine ctor + allocMemory + createKernels (cyclo/src/engine.h:40-65,132)
 *           and transform ctor / initEngine roots (cyclo/src/transform.h:300-433). */
int ctw_prp_create(int log2_degree, int lanes, ctw_prp **out);
/* An engine for the twin partner N- = b^D - b^{D/2} - 1 (D = 2^log2_degree,
 * 8..16), which the sieve's "-" form pairs with N+ (sieve/CPU/ctsieve.cpp:
 * 434-439); the reference has no PRP test for it.  The product of two residues
 * of degree < D is taken exactly on the transform of degree 2D and folded
 * with b^D = b^{D/2} + 1.  Every call of the PRP engine applies:
 * ctw_prp_run tests N- (exponent N- - 1 = b^D - b^{D/2} - 2), get_digits and
 * is_prime give the canonical residue mod N- (D digits per lane), while
 * read_regs / write_regs move the 2D-word registers of the transform. */
int ctw_prp_create_minus(int log2_degree, int lanes, ctw_prp **out);
/* The same with an explicit cluster split: 2^log2_ctas CTAs per candidate
 * (-1: the default split).  Registers and results do not depend on the split;
 * it is an autotuning choice (ctw_prp_autotune).  CTW_E_ARG when the degree
 * has no kernel for that split. */
int ctw_prp_create_split(int log2_degree, int lanes, int log2_ctas, ctw_prp **out);
int ctw_prp_destroy(ctw_prp *h);

/* Carry chunk size, 8/16/32/64 (the reference's CSIZE, autotuned there,
 * cyclo/src/transform.h:383-419).  Register digits depend on it; canonical
 * results do not.  Default 8. */
int ctw_prp_set_csize(ctw_prp *h, int csize);
/* Base of the Fermat test: 2 (the reference) or 3.  Sets the multiplier that
 * square_dup applies for a set bit.  Default 2. */
int ctw_prp_set_base(ctw_prp *h, uint32_t base);

/* b of each lane, 64 <= b < 2^31; count == lanes.
 * Replaces transform::set_b / engine::writeMemory_b (cyclo/src/transform.h:472-486). */
int ctw_prp_set_b(ctw_prp *h, const uint32_t *b, int count);
/* NTT primes: 0 (default) uses two primes whenever every product coefficient
 * of the current b fits in them (2 * terms * (b + 1)^2 < q0 q1 with terms =
 * 1.5 D, or D for N-) and the split has a two-prime kernel (one CTA, or 4096
 * coefficients per CTA); 3 always uses three.  Registers are the same either
 * way: the products are exact integers.  No reference counterpart (the
 * reference always uses three primes, cyclo/src/transform.h:26-28). */
int ctw_prp_set_prime_count(ctw_prp *h, int count);
/* Primes the next launch uses (2 or 3). */
int ctw_prp_prime_count(ctw_prp *h);
/* 1 when a test of degree 2^log2_degree (N- when minus != 0) and this b runs
 * on two primes with the default split; host only, no device needed. */
int ctw_prp_two_primes(int log2_degree, int minus, uint32_t b);

/* Register 0 of every lane <- a.   Replaces engine::set (cyclo/src/engine.h:231-237). */
int ctw_prp_set(ctw_prp *h, uint32_t a);
/* Register dst <- register src.    Replaces engine::copy (cyclo/src/engine.h:240-247). */
int ctw_prp_copy(ctw_prp *h, int dst, int src);
/* reg0 <- reg0^2 * base^{bit(lane)}, bit(lane) = bit (lane % 64) of
 * lane_mask_words[lane / 64].  Asynchronous on the handle's stream.
 * Replaces engine::squareDup(ln, dup) (cyclo/src/engine.h:387-419). */
int ctw_prp_square_dup(ctw_prp *h, const uint64_t *lane_mask_words);
/* reg0 <- reg0 * reg1.   Replaces engine::mul (cyclo/src/engine.h:421-433). */
int ctw_prp_mul(ctw_prp *h);
/* reg_out <- reg_a * reg_b (registers 0..2; reg_out may equal reg_a or reg_b). */
int ctw_prp_mul_regs(ctw_prp *h, int reg_out, int reg_a, int reg_b);
/* reg0 <- reg0^(2^count) * base^(bits of e), processing bit i_hi down to
 * i_hi - count + 1 of each lane's exponent e (little-endian 32-bit words,
 * nwords per lane, lanes * nwords words in total).  One launch, the residue
 * stays in shared memory between squarings. */
int ctw_prp_square_bits(ctw_prp *h, const uint32_t *e_words, int nwords, long long i_hi, int count);
/* Upload the per-lane exponents once (lanes * nwords words) and keep them in
 * device memory; ctw_prp_square_resident then squares over bits i_hi down to
 * i_hi - count + 1 of that resident copy without any host transfer. */
int ctw_prp_load_exponent(ctw_prp *h, const uint32_t *e_words, int nwords);
int ctw_prp_square_resident(ctw_prp *h, long long i_hi, int count);

/* Canonical digits (each in [0, b)) of register reg for every lane: out has
 * lanes * D entries, lane-major.  Blocks until the stream is idle.
 * Replaces transform::getInt (cyclo/src/transform.h:501-597). */
int ctw_prp_get_digits(ctw_prp *h, int reg, uint32_t *out);
/* PRP flag and RES64 (sum x_j b^j mod 2^64) of register reg per lane; returns
 * CTW_E_COMPUTE if a lane's residue is zero.
 * Replaces transform::isPrime (cyclo/src/transform.h:600-636). */
int ctw_prp_is_prime(ctw_prp *h, int reg, uint8_t *is_prp, uint64_t *res64);
/* Raw register digits (signed, as the device keeps them), lanes * D int32 per
 * register, registers first..first+nregs-1.  Context save/restore
 * (cyclo/src/transform.h:445-468 keeps the same digits as RNS residues). */
int ctw_prp_read_regs(ctw_prp *h, int first, int nregs, int32_t *out);
int ctw_prp_write_regs(ctw_prp *h, int first, int nregs, const int32_t *in);

/* Whole Fermat test of `count` (<= lanes) candidates of this degree, including
 * the Gerbicz-Li check, as cyclo::check(b) (cyclo/src/cyclo.h:252-377).
 * Lanes past count repeat the last b (cyclo/src/cyclo.h:233-236).
 * Outputs per candidate: is_prp, res64, gl_ok (1 = Gerbicz-Li passed). */
int ctw_prp_run(ctw_prp *h, const uint32_t *b, int count, uint8_t *is_prp, uint64_t *res64, uint8_t *gl_ok);
/* ctw_prp_run with resume and checkpoints, as cyclo::check(b, ctx, k, ri)
 * (cyclo/src/cyclo.h:252-377).  i_start < 0 starts afresh (registers 0 and 1
 * set to 1); i_start >= 0 resumes before the squaring of bit i_start with
 * registers 0 (x) and 1 (d) as they are (restored with
 * ctw_prp_read_context).  checkpoint(user, i), if not NULL, is called on the
 * host after every Gerbicz-Li multiply, i being the next bit to square and
 * the device idle (the reference saves one squaring earlier; either point
 * resumes correctly); a nonzero return stops the run with CTW_STOPPED and the
 * registers at that point. */
typedef int (*ctw_checkpoint_fn)(void *user, long long i);
int ctw_prp_run_ex(ctw_prp *h, const uint32_t *b, int count, long long i_start, ctw_checkpoint_fn checkpoint,
                   void *user, uint8_t *is_prp, uint64_t *res64, uint8_t *gl_ok);
/* Save registers 0 and 1 with (k, i, elapsed) as the reference's context file
 * (cyclo/src/cyclo.h:146-177, cyclo/src/transform.h:458-468, file.h CRC32):
 * version 1, k, i (int32), elapsed (double), for registers 0..1 the residues of
 * every digit mod the reference's primes 4293918721, 4253024257 (pairs) and
 * 4231004161, indexed (register * D + j) * lanes + lane, then the CRC32
 * trailer; written to path.new, the previous file kept as path.old.  Files are
 * interchangeable with the reference's when lanes = 64. */
int ctw_prp_save_context(ctw_prp *h, const char *path, int k, int i, double elapsed);
/* Read such a file (path, else path.old) into registers 0 and 1: 0 = read,
 * 1 = no file, CTW_E_ARG = invalid (bad size, CRC or residues). */
int ctw_prp_read_context(ctw_prp *h, const char *path, int *k, int *i, double *elapsed);
/* Encode / decode the context bytes of digits [nregs][D][lanes]-ordered as
 * the reference lays them out, without a device (bytes: 20 + 12 * nregs * D *
 * lanes + 4).  decode returns CTW_E_ARG on a bad CRC or inconsistent residues. */
size_t ctw_context_bytes(int log2_degree, int lanes, int nregs);
int ctw_context_encode(int log2_degree, int lanes, int nregs, const int32_t *digits, int k, int i, double elapsed,
                       uint8_t *out);
int ctw_context_decode(int log2_degree, int lanes, int nregs, const uint8_t *in, size_t size, int32_t *digits,
                       int *k, int *i, double *elapsed);
/* The cyclog file loop (cyclo/src/cyclo.h:416-480): b values of `filename`
 * (one per line) in vectors of 64 (the last padded with its last b), the CSIZE
 * of filename.ini (tuned and written when absent), cyclo.ctx in workdir
 * (resumed when present, saved every save_every_s seconds at checkpoints and
 * when stopping), result lines appended to workdir/result_c.txt in the
 * reference's words ("... is a probable prime." / "... is composite. RES64:
 * %016X"), PRP b appended to workdir/prp_<n>.txt.  minus != 0 tests the twin
 * partners N- instead (lines "... - 1 is ...", PRPs to prpm_<n>.txt, context
 * cyclom.ctx).  The run stops (context saved, CTW_STOPPED) when *quit becomes
 * nonzero or after stop_after checkpoints (0 = never).  0 = all done. */
int ctw_cyclo_check_file(int n, const char *filename, const char *workdir, int minus, double save_every_s,
                         volatile int *quit, int stop_after);

/* Block until all work queued on the handle's stream is done. */
int ctw_prp_sync(ctw_prp *h);
/* The handle's cudaStream_t (as void *), for event timing by the caller. */
void *ctw_prp_stream(ctw_prp *h);
/* Launch geometry chosen for this degree: CTAs per lane (cluster size),
 * threads per CTA, dynamic shared memory per CTA in bytes. */
int ctw_prp_geometry(ctw_prp *h, int *ctas_per_lane, int *threads, int *smem_bytes);
/* Kernel launches issued by this handle since creation. */
long long ctw_prp_launches(ctw_prp *h);
/* Degree of the tested numbers (log2), lanes, and 1 for an N- engine. */
int ctw_prp_shape(ctw_prp *h, int *log2_degree, int *lanes, int *minus);
/* Testing only, no counterpart in the reference: in the next launch of a grid
 * handle the grid-barrier counter starts out of reach and CTA 0 skips its first
 * publication of columns, so that the other CTAs' bounded waits (50 ms of
 * %globaltimer each, on the barrier or on the published words) run out.  That
 * launch ends with CTW_E_COMPUTE (status ST_GRID_WAIT, results void) and the
 * handle stays usable; later launches are unaffected.  CTW_E_ARG for a
 * non-grid split. */
int ctw_prp_test_unreachable_barrier(ctw_prp *h);

/* z = x * y for `lanes` candidates of degree D = 2^log2_degree (8..14), with
 * x, y, z caller-owned DEVICE buffers of lanes * D int32 digits (the register
 * format of ctw_prp_read_regs) and b[lanes] on the host; the result is the one
 * ctw_prp_mul_regs gives.  No counterpart in the reference.
 * For callers that must not allocate device memory (a host that reserved the
 * GPU's memory for itself, a pooling allocator that forbids cudaMalloc, a
 * pipeline that cannot take cudaMalloc's device-wide synchronisation): it
 * allocates nothing and uses fixed __device__ arrays the library holds on every
 * GPU until exit (4 MiB scratch, so lanes * 12 * D <= 4 MiB and lanes <= 1024;
 * larger requests fail with CTW_E_ARG).  Calls share those arrays: calls that
 * overlap on the GPU (other streams, other threads) race and must be
 * serialised by the caller.  The first call on each device sets the arrays up
 * (symbol addresses, root tables uploaded on `stream`, which it synchronises)
 * and should come before any stream capture.  The set-up is kept per device
 * ordinal for the device's primary context (the runtime's own); a caller that
 * makes another driver context current on that device is not supported.
 * z may be x or y, or both (x == y squares): each CTA reads the words of x
 * and y that it later writes in z, and reads them before it writes.
 * Runs on `stream` (a cudaStream_t, NULL = default) and returns after it has
 * synchronised the stream; CTW_E_ARG when `stream` is being captured into a
 * graph. */
int ctw_prp_mul_noalloc(int log2_degree, int lanes, const uint32_t *b, const int32_t *x_dev,
                        const int32_t *y_dev, int32_t *z_dev, int csize, void *stream);

/* Pick the cluster split and carry chunk of degree 2^log2_degree for `lanes`
 * resident candidates by timing every supported (split, csize) pair on the
 * device (the reference times its CSIZE candidates the same way,
 * cyclo/src/transform.h:383-419) with b inside the two-prime bound.  Results
 * are cached per (degree, lanes) for the life of the process.  Outputs may be NULL. */
int ctw_prp_autotune(int log2_degree, int lanes, int *log2_ctas, int *csize, double *us_per_squaring);
/* The same for tests on `primes` NTT primes: 2 (b within the two-prime bound,
 * what ctw_prp_autotune tunes for) or 3 (b above it).  Cached per (degree,
 * lanes, primes). */
int ctw_prp_autotune_primes(int log2_degree, int lanes, int primes, int *log2_ctas, int *csize,
                            double *us_per_squaring);

/* ------------------------------------------------------------------------ */
/* Pools: many resident tests of one degree, each at its own bit position.  */
/* No counterpart in the reference, which runs one vector of 64 candidates   */
/* of one degree to completion (cyclo/src/cyclo.h:457-478).                  */
/* ------------------------------------------------------------------------ */

#define CTW_E_FULL (-6)       /* no free slot */

/* One finished test (pool or server).  Times are seconds on the owner's clock
 * (CLOCK_MONOTONIC of the process for pools, the server's clock for servers). */
typedef struct ctw_result {
	uint64_t tag;             /* caller's tag */
	uint64_t res64;           /* RES64 of 2^(N-1) mod N (base 3: 3^(N-1)) */
	uint32_t b;
	int32_t log2_degree;
	uint8_t is_prp;           /* residue == 1 */
	uint8_t gl_ok;            /* Gerbicz-Li check passed */
	int8_t status;            /* 0, or the CTW_E_* code of a failed test */
	uint8_t reserved;
	int32_t slot;             /* pool slot; -1: never admitted; -2: the server's grid lane */
	double t_submit, t_admit, t_done;
	long long squarings;      /* squarings and multiplies run for this test */
} ctw_result;

typedef struct ctw_pool ctw_pool;

/* A pool of `slots` (<= 4096) tests of degree 2^log2_degree kept in HBM
 * (six registers and the multiply's scratch per slot).  Every tick runs, for
 * each active slot, gl_block squarings over its own next exponent bits and
 * its Gerbicz-Li multiply, so tests admitted at different times share each
 * launch (continuous batching).  Ticks are queued as CUDA graphs on the pool's
 * stream.  log2_ctas -1 and csize 0 take the default split and CSIZE 8;
 * gl_block 0 takes the reference's rule (cyclo/src/cyclo.h:272) for a 20-bit
 * b.  Results are bit-identical to ctw_prp_run's. */
int ctw_pool_create(int log2_degree, int slots, int log2_ctas, int csize, uint32_t base, int gl_block,
                    ctw_pool **out);
/* A pool of twin partners N- = b^D - b^{D/2} - 1 (D = 2^log2_degree, 8..16;
 * see ctw_prp_create_minus); every pool call applies unchanged. */
int ctw_pool_create_minus(int log2_degree, int slots, int csize, uint32_t base, int gl_block, ctw_pool **out);
int ctw_pool_destroy(ctw_pool *p);
/* Device bytes a pool holds per slot at this degree (admission by footprint). */
size_t ctw_pool_slot_bytes(int log2_degree);
/* Admit a test of b (64 <= b < 2^31) into the lowest free slot; returns the
 * slot (>= 0) or CTW_E_FULL.  The test starts with the next queued tick. */
int ctw_pool_admit(ctw_pool *p, uint32_t b, uint64_t tag);
/* Admit up to `count` tests at once (as many as there are free slots),
 * preparing their exponents on `threads` host threads (0: all cores); tags
 * may be NULL (tag = index).  Returns the number admitted. */
int ctw_pool_admit_many(ctw_pool *p, const uint32_t *b, const uint64_t *tags, int count, int threads);
/* Queue `ticks` ticks (asynchronous; blocks only while two graph launches of
 * this pool are already in flight). */
int ctw_pool_run(ctw_pool *p, int ticks);
/* Retire the tests whose last tick has completed (wait != 0: wait for every
 * queued tick first); returns the number of results waiting to be taken. */
int ctw_pool_collect(ctw_pool *p, int wait);
/* Take up to max results; returns the count. */
int ctw_pool_results(ctw_pool *p, ctw_result *out, int max);
/* Slots, active tests, queued-but-unfinished graph launches, the Gerbicz-Li
 * block, split and csize in use, and squarings issued so far (any may be NULL). */
int ctw_pool_info(ctw_pool *p, int *slots, int *active, int *in_flight, int *gl_block, int *log2_ctas, int *csize,
                  long long *squarings);
/* Copy register reg (0..5) of one slot to the host (after ctw_pool_collect
 * with wait); for tests. */
int ctw_pool_read_slot(ctw_pool *p, int slot, int reg, int32_t *out);
/* NTT primes of the pool's launches: 0 (default) picks two for a launch whose
 * lanes all allow it (as ctw_prp_set_prime_count), 3 always three. */
int ctw_pool_set_prime_count(ctw_pool *p, int count);
/* Primes the next launch over the current slots would use (2 or 3). */
int ctw_pool_prime_count(ctw_pool *p);
void *ctw_pool_stream(ctw_pool *p);
/* The tick program of one test, without a device: per tick 4 int32 words
 * {register moves before the squarings, moves after the multiply (PrpAuxOp
 * bits), exponent source (0 = E, 1 = Gerbicz-Li block sum), lowest bit of the
 * tick's *block bits}.  Returns the tick count (or the count needed when
 * max_ticks is too small). */
int ctw_pool_schedule(int log2_degree, uint32_t b, int gl_block, int32_t *ticks_out, int max_ticks, int *block);

/* Batches of pools of uneven degrees, no counterpart in the reference (its
 * batching is 64 lanes of one degree per vector, cyclo/src/engine.h:19,
 * cyclo/src/cyclo.h:216-241).  A batch drives pools of degrees 2^12..2^15
 * whose split has 4096 coefficients per CTA (log2_ctas = log2_degree - 12;
 * N+ only; slots a multiple of 2^(15 - log2_degree)) tick by tick: per tick
 * every pool's register moves, then ONE persistent launch (per NTT prime
 * count) in which clusters of 8 CTAs take work items from per-degree queues,
 * largest degree first - an item is 2^(15 - k) lanes of a degree-2^k pool,
 * each on 2^(k - 12) CTAs, for the pool's B squarings - then one such launch
 * for every pool's Gerbicz-Li multiply, then the moves after; ticks are
 * replayed from CUDA graphs.  Registers, results and their collection are the
 * pools' own (ctw_pool_collect / ctw_pool_results); a pool in a batch is run
 * only through it.  The caller keeps ownership of the pools. */
typedef struct ctw_batch ctw_batch;
int ctw_batch_create(ctw_pool *const *pools, int count, ctw_batch **out);
int ctw_batch_run(ctw_batch *b, int ticks);
int ctw_batch_destroy(ctw_batch *b);
void *ctw_batch_stream(ctw_batch *b);
/* Persistent launches issued by the batch since creation. */
long long ctw_batch_launches(ctw_batch *b);
/* CTAs per SM of the batch kernel build (1: up to 128 registers a thread;
 * 2, the default: 64 / 80 registers), an autotuning choice. */
int ctw_batch_set_ctas_per_sm(ctw_batch *b, int ctas);

/* ------------------------------------------------------------------------ */
/* Server: a request loop over pools of every degree.  No counterpart in the */
/* reference.                                                                */
/* ------------------------------------------------------------------------ */

typedef struct ctw_server ctw_server;

/* Start a server thread.  hbm_budget_bytes bounds the pools' device memory
 * (0: 80 % of the free memory); a request waits until its class has a free
 * slot, and a new pool is allocated only while the budget allows.  A class is
 * a degree and whether b is within the degree's two-prime bound
 * (ctw_prp_two_primes), so tests above the bound have pools of their own.
 * max_slots caps one pool; ticks_per_launch sets the graph length (1..8);
 * autotune != 0 picks split and csize per class on first use. */
int ctw_server_create(size_t hbm_budget_bytes, int max_slots, uint32_t base, int ticks_per_launch, int autotune,
                      ctw_server **out);
/* Queue a test (thread-safe).  8 <= log2_degree <= 18. */
int ctw_server_submit(ctw_server *s, int log2_degree, uint32_t b, uint64_t tag);
/* Grid lanes: tests of degree >= 2^min_log2_degree (8..18; 0 turns the lanes
 * off) run on one-lane engines instead of in pools, one test per lane at a
 * time; at 2^16..2^18 the engine's default split is the cooperative grid
 * kernel (one test over 64-128 SMs).  The lanes whose CTAs fit on the SMs
 * together hold the device at once (two tests of 64 CTAs, one of 128); lanes
 * and pools take turns at every Gerbicz-Li checkpoint.  Lane results carry
 * slot -2.  Default 16.  Applies to requests submitted afterwards. */
int ctw_server_set_grid_lane(ctw_server *s, int min_log2_degree);
/* Grid lanes that take requests: 1 (the default: large tests first come, first
 * served) or 2 (two tests in flight; they hold the device together when their
 * CTAs fit on the SMs, else in turns). */
int ctw_server_set_grid_lanes(ctw_server *s, int lanes);
/* Create (and tune) the pools of a degree (one per prime class where the degree
 * has a two-prime kernel) ahead of its first request. */
int ctw_server_prepare(ctw_server *s, int log2_degree, int slots);
/* Take up to max finished tests, waiting up to timeout_ms for the first. */
int ctw_server_poll(ctw_server *s, ctw_result *out, int max, int timeout_ms);
/* Submitted, pending (not admitted), active, finished counts; pool bytes allocated. */
int ctw_server_stats(ctw_server *s, long long *submitted, long long *pending, long long *active, long long *finished,
                     size_t *pool_bytes);
/* Seconds since the server started (the clock of ctw_result times). */
double ctw_server_clock(ctw_server *s);
/* Stop the thread and free the pools. */
int ctw_server_destroy(ctw_server *s);

/* Measured 32-bit integer multiply-add throughput of the device (IMAD/s),
 * from an in-library probe kernel; the roofline denominator. */
double ctw_imad_peak(void);
/* Measured throughput of 32-bit modular products (products/s) from probe
 * kernels of independent chains: kind 0 Montgomery (the product the
 * algorithmic count charges 4 IMAD), kind 1 Shoup with a precomputed quotient.
 * 0.0 for another kind or without a device.  No counterpart in the reference. */
double ctw_modmul_peak(int kind);

/* ------------------------------------------------------------------------ */
/* Sieve: strike b in [b_min, b_max] with p | b^(2^n) - b^(2^(n-1)) +- 1      */
/* ------------------------------------------------------------------------ */

/* One sieve pass over the primes of one form:
 *   mode +1: p = 3k*2^n + 1 (Sieve::check_pos, sieve/CPU/ctsieve.cpp:678-726;
 *            GPU kernels sieve/GPU/ocl/kernel.cl:243-320),
 *   mode -1: p = 10k +- 1   (Sieve::check_neg, sieve/CPU/ctsieve.cpp:728-787;
 *            GPU kernels sieve/GPU/ocl/kernel.cl:328-479).
 * The k range is the reference's: k from p_min/(3*2^n) (resp. p_min/10) up to
 * the first k whose p reaches p_max (ctsieve.cpp:682-684, 733-735).
 * struck_words: in/out bitmap, bit i (word i/32, bit i%32) set when b_min + i
 * is struck; existing bits are kept (two calls, + then -, give the reference's
 * "ini" list).  *p_last: in/out, raised to the last p the reference would have
 * processed (its _p_min_pos / _p_min_neg, written to sv_*.dat).
 * 8 <= n <= 24, 2 <= b_min <= b_max, p_max < 2^62. */
int ctw_sieve_run(int n, uint64_t b_min, uint64_t b_max, uint64_t p_min, uint64_t p_max, int mode,
                  uint32_t *struck_words, uint64_t *p_last);
/* Write sv_<n>_<b_min>_<b_max>.dat and cand_<n>_<b_min>_<b_max>.txt into dir,
 * byte-identical to Sieve::write(true) (sieve/CPU/ctsieve.cpp:591-626). */
int ctw_sieve_write_files(int n, uint64_t b_min, uint64_t b_max, const uint32_t *struck_words,
                          uint64_t p_min_pos, uint64_t p_min_neg, const char *dir);
/* Factor pairs of the reference's GPU sieve (sieve/GPU/ocl/kernel.cl:233-479):
 * for every prime p = 3k*2^n + 1 (mode +1) or 10k +- 1 (mode -1) with k in
 * [k_begin, k_end), every root b of b^(2^n) - b^(2^(n-1)) +- 1 mod p with
 * 2 <= b <= b_max, as (p, b) in pairs[2i], pairs[2i+1], sorted by p then b.
 * *count = the number found; CTW_E_NOMEM when it exceeds cap. */
int ctw_sieve_factors(int n, uint64_t k_begin, uint64_t k_end, int mode, uint64_t b_max, uint64_t *pairs,
                      uint64_t cap, uint64_t *count);
/* The ctsieveg run (sieve/GPU/src/ctsieve.h:326-421, main.cpp): blocks of
 * 2^21 k from floor(p_min f) to ceil(p_max f), factors with p in [p_min,
 * p_max] and b <= bMax (5e9, or 1e10 for p >= 1e16 (+) / 1e13 (-)) checked on
 * the host and appended as "p b" lines to workdir/fp<n>_<p_min/1e12>_<p_max/1e12>.txt
 * (fn... for mode -1, lines of one block sorted); after each block
 * workdir/ctx<...> (ctx_n<...>) holds the blocks done and the elapsed time,
 * and a new run resumes from it.  Stops with CTW_STOPPED when *quit becomes
 * nonzero or after stop_after_blocks blocks (0 = never). */
int ctw_gfsieve_check(int n, uint64_t p_min, uint64_t p_max, int mode, const char *workdir, volatile int *quit,
                      int stop_after_blocks, uint64_t *factors_written);
/* Sieve kernel launches issued by this process. */
long long ctw_sieve_launches(void);
/* Measured 64-bit Montgomery multiply throughput of the device (mulmods/s),
 * from an in-library probe kernel; the sieve's roofline denominator. */
double ctw_mulmod64_peak(void);

#ifdef __cplusplus
}
#endif

#endif /* CTWIN_GB300_H */
