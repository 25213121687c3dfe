// Host stand-ins for the CUDA built-ins and the runtime calls of the sieve
// (ctwin_gb300/csrc/sieve.cu), so that the whole sieve path - host driver and
// kernels - compiles with g++ and runs on the CPU (test infrastructure:
// tests/test_kernels_emu_cpu.py).  Kernel launches become emu_launch calls
// (the test rewrites the launch syntax); the CTAs of a launch run one after
// another, the threads of a CTA at once, so a kernel's static shared
// variables can be plain statics.  Device memory is host memory.
#pragma once
#include <algorithm>
#include <barrier>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

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
#define __launch_bounds__(...)
#define __align__(n) alignas(n)
#define __shared__ static
using std::max;
using std::min;

inline uint64_t __umul64hi(uint64_t a, uint64_t b) { return (uint64_t)(((unsigned __int128)a * b) >> 64); }
inline uint32_t __umulhi(uint32_t a, uint32_t b) { return (uint32_t)(((uint64_t)a * b) >> 32); }
inline int __clzll(long long x) { return x ? __builtin_clzll((unsigned long long)x) : 64; }
inline int __clz(int x) { return x ? __builtin_clz((unsigned)x) : 32; }
inline int __ffs(int x) { return __builtin_ffs(x); }
inline int __ffsll(long long x) { return __builtin_ffsll(x); }
inline int __popc(unsigned x) { return __builtin_popcount(x); }
inline unsigned atomicAdd(unsigned *p, unsigned v) { return __atomic_fetch_add(p, v, __ATOMIC_SEQ_CST); }
inline unsigned atomicOr(unsigned *p, unsigned v) { return __atomic_fetch_or(p, v, __ATOMIC_SEQ_CST); }
inline unsigned long long atomicMax(unsigned long long *p, unsigned long long v)
{
	unsigned long long o = __atomic_load_n(p, __ATOMIC_SEQ_CST);
	while (o < v && !__atomic_compare_exchange_n(p, &o, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) {}
	return o;
}
void __syncthreads();
uint32_t *emu_dyn_smem();

// ---- runtime ----
typedef int cudaError_t;
enum { cudaSuccess = 0, cudaErrorInvalidValue = 1 };
enum cudaMemcpyKind { cudaMemcpyHostToHost, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost, cudaMemcpyDeviceToDevice };
enum cudaDeviceAttr { cudaDevAttrMultiProcessorCount };
enum cudaFuncAttribute { cudaFuncAttributeMaxDynamicSharedMemorySize };
typedef void *cudaStream_t;
typedef int *cudaEvent_t;
inline const char *cudaGetErrorString(cudaError_t) { return "emulated CUDA error"; }
inline cudaError_t cudaGetLastError() { return cudaSuccess; }
inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
inline cudaError_t cudaGetDevice(int *d) { *d = 0; return cudaSuccess; }
int emu_sms();
inline cudaError_t cudaDeviceGetAttribute(int *v, cudaDeviceAttr, int) { *v = emu_sms(); return cudaSuccess; }
template <class F> inline cudaError_t cudaFuncSetAttribute(F, cudaFuncAttribute, int) { return cudaSuccess; }
template <class T> inline cudaError_t cudaMalloc(T **p, size_t n)
{
	*p = (T *)malloc(n ? n : 1);
	if (*p) memset((void *)*p, 0xA5, n);   // device memory starts with garbage
	return *p ? cudaSuccess : cudaErrorInvalidValue;
}
inline cudaError_t cudaFree(void *p) { free(p); return cudaSuccess; }
inline cudaError_t cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind) { memcpy(d, s, n); return cudaSuccess; }
inline cudaError_t cudaMemset(void *p, int v, size_t n) { memset(p, v, n); return cudaSuccess; }
inline cudaError_t cudaEventCreate(cudaEvent_t *e) { *e = new int(0); return cudaSuccess; }
inline cudaError_t cudaEventDestroy(cudaEvent_t e) { delete e; return cudaSuccess; }
inline cudaError_t cudaEventRecord(cudaEvent_t, cudaStream_t = nullptr) { return cudaSuccess; }
inline cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
inline cudaError_t cudaEventElapsedTime(float *ms, cudaEvent_t, cudaEvent_t) { *ms = 1.0f; return cudaSuccess; }

// ---- launches: kernel<<<grid, block[, smem]>>>(args) -> emu_launch(kernel, EmuCfg{grid, block[, smem]})(args)
struct EmuCfg {
	dim3 grid, block;
	size_t smem = 0;
};
void emu_run_blocks(const EmuCfg &c, void (*body)(void *), void *ctx);
template <class K> struct EmuLaunch {
	K k;
	EmuCfg c;
	template <class... A> void operator()(A... a)
	{
		auto call = [&]() { k(a...); };
		emu_run_blocks(c, [](void *p) { (*static_cast<decltype(call) *>(p))(); }, &call);
	}
};
template <class K> EmuLaunch<K> emu_launch(K k, EmuCfg c) { return EmuLaunch<K>{ k, c }; }
