// Host stand-ins for the CUDA built-ins the PRP kernels use, so that their
// source compiles with g++ and runs with one host thread per GPU thread (test
// infrastructure: tests/test_kernels_emu_cpu.py).  Shared memory, __syncthreads
// and the clock come from the emulation programs (grid_emu.cpp,
// cluster_emu.cpp); global atomics and fences map to the host's sequentially
// consistent atomics.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <sched.h>
struct dim3 {
	unsigned x, y, z;
	dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
extern thread_local dim3 threadIdx, blockIdx;
extern dim3 blockDim, gridDim;
#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __noinline__
#define __launch_bounds__(...)
#define __align__(n) __attribute__((aligned(n)))
#define __shared__
#define CTW_EMU 1
using std::max;
using std::min;
struct alignas(8) uint2 { uint32_t x, y; };
struct alignas(16) uint4 { uint32_t x, y, z, w; };
struct alignas(16) int4 { int32_t x, y, z, w; };
inline long long __double2ll_rd(double x) { return (long long)std::floor(x); }
inline double __ll2double_rn(long long x) { return (double)x; }
inline uint32_t __umulhi(uint32_t a, uint32_t b) { return (uint32_t)(((uint64_t)a * b) >> 32); }
inline uint64_t __umul64hi(uint64_t a, uint64_t b) { return (uint64_t)(((unsigned __int128)a * b) >> 64); }
inline unsigned atomicOr(unsigned *p, unsigned v) { return __atomic_fetch_or(p, v, __ATOMIC_SEQ_CST); }
inline unsigned atomicAdd(unsigned *p, unsigned v) { return __atomic_fetch_add(p, v, __ATOMIC_SEQ_CST); }
inline void __threadfence() { __atomic_thread_fence(__ATOMIC_SEQ_CST); }
void __syncthreads();
void emu_syncwarp();
inline uint2 make_uint2(uint32_t x, uint32_t y) { return uint2{ x, y }; }
inline uint4 make_uint4(uint32_t x, uint32_t y, uint32_t z, uint32_t w) { return uint4{ x, y, z, w }; }
inline int4 make_int4(int32_t x, int32_t y, int32_t z, int32_t w) { return int4{ x, y, z, w }; }
uint32_t *emu_smem();
unsigned long long emu_timer_ns();
// a thread that polls another CTA's words lets the host threads of that CTA run
inline void emu_yield() { sched_yield(); }
