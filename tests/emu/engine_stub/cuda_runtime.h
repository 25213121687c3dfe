// Stand-in CUDA runtime for the host emulation of the PRP engine (test
// infrastructure: tests/test_kernels_emu_cpu.py).  Device memory is host
// memory, streams and events are synchronous no-ops, and every launch runs
// its CTAs on host threads (engine_emu.cpp): one cluster at a time, or the
// whole grid at once for a cooperative launch.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>

typedef int cudaError_t;
enum { cudaSuccess = 0, cudaErrorInvalidValue = 1, cudaErrorMemoryAllocation = 2 };
enum cudaMemcpyKind { cudaMemcpyHostToHost, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost, cudaMemcpyDeviceToDevice };
enum cudaDeviceAttr { cudaDevAttrMultiProcessorCount };
enum cudaFuncAttribute { cudaFuncAttributeMaxDynamicSharedMemorySize, cudaFuncAttributeNonPortableClusterSizeAllowed };
enum cudaLaunchAttributeID { cudaLaunchAttributeClusterDimension = 4, cudaLaunchAttributeCooperative = 2 };
enum { cudaStreamNonBlocking = 1 };
typedef void *cudaStream_t;
typedef int *cudaEvent_t;
struct cudaLaunchAttribute {
	cudaLaunchAttributeID id;
	struct {
		struct { unsigned x, y, z; } clusterDim;
		int cooperative;
	} val;
};
struct cudaLaunchConfig_t {
	dim3 gridDim, blockDim;
	size_t dynamicSmemBytes;
	cudaStream_t stream;
	cudaLaunchAttribute *attrs;
	unsigned numAttrs;
};

inline const char *cudaGetErrorString(cudaError_t) { return "emulated CUDA error"; }
inline cudaError_t cudaGetLastError() { return cudaSuccess; }
inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
inline cudaError_t cudaGetDevice(int *d) { *d = 0; return cudaSuccess; }
inline cudaError_t cudaGetDeviceCount(int *n) { *n = 1; return cudaSuccess; }
inline cudaError_t cudaDeviceGetAttribute(int *v, cudaDeviceAttr, int) { *v = 152; return cudaSuccess; }
template <class F> inline cudaError_t cudaFuncSetAttribute(F, cudaFuncAttribute, int) { return cudaSuccess; }
template <class F> inline cudaError_t cudaOccupancyMaxActiveBlocksPerMultiprocessor(int *n, F, int, size_t)
{
	*n = 1;
	return cudaSuccess;
}
template <class T> inline cudaError_t cudaMalloc(T **p, size_t n)
{
	*p = (T *)malloc(n ? n : 1);
	if (*p) memset((void *)*p, 0xA5, n);   // device memory starts with garbage
	return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
inline cudaError_t cudaFree(void *p) { free(p); return cudaSuccess; }
inline cudaError_t cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind) { memmove(d, s, n); return cudaSuccess; }
inline cudaError_t cudaMemcpyAsync(void *d, const void *s, size_t n, cudaMemcpyKind, cudaStream_t = nullptr)
{
	memmove(d, s, n);
	return cudaSuccess;
}
inline cudaError_t cudaMemcpy2DAsync(void *d, size_t dp, const void *s, size_t sp, size_t w, size_t h, cudaMemcpyKind,
                                     cudaStream_t = nullptr)
{
	for (size_t r = 0; r < h; ++r) memmove((char *)d + r * dp, (const char *)s + r * sp, w);
	return cudaSuccess;
}
inline cudaError_t cudaMemset(void *p, int v, size_t n) { memset(p, v, n); return cudaSuccess; }
inline cudaError_t cudaMemsetAsync(void *p, int v, size_t n, cudaStream_t = nullptr) { memset(p, v, n); return cudaSuccess; }
inline cudaError_t cudaStreamCreateWithFlags(cudaStream_t *s, unsigned) { *s = malloc(1); return cudaSuccess; }
inline cudaError_t cudaStreamDestroy(cudaStream_t s) { free(s); return cudaSuccess; }
inline cudaError_t cudaStreamSynchronize(cudaStream_t) { return cudaSuccess; }
inline cudaError_t cudaEventCreate(cudaEvent_t *e) { *e = new int(0); return cudaSuccess; }
inline cudaError_t cudaEventDestroy(cudaEvent_t e) { delete e; return cudaSuccess; }
inline cudaError_t cudaEventRecord(cudaEvent_t, cudaStream_t = nullptr) { return cudaSuccess; }
inline cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
inline cudaError_t cudaEventElapsedTime(float *ms, cudaEvent_t, cudaEvent_t) { *ms = 1.0f; return cudaSuccess; }

// launches
void emu_run_ctas(dim3 grid, dim3 block, size_t smem, int group, void (*body)(void *), void *ctx);
template <class... P, class... A> cudaError_t cudaLaunchKernelEx(const cudaLaunchConfig_t *c, void (*k)(P...), A... a)
{
	int group = 1;
	for (unsigned i = 0; i < c->numAttrs; ++i)
	{
		if (c->attrs[i].id == cudaLaunchAttributeClusterDimension) group = (int)c->attrs[i].val.clusterDim.x;
		if (c->attrs[i].id == cudaLaunchAttributeCooperative && c->attrs[i].val.cooperative) group = (int)c->gridDim.x;
	}
	auto call = [&]() { k(a...); };
	emu_run_ctas(c->gridDim, c->blockDim, c->dynamicSmemBytes, group, [](void *p) { (*static_cast<decltype(call) *>(p))(); },
	             &call);
	return cudaSuccess;
}
struct EmuCfg {
	dim3 grid, block;
	size_t smem = 0;
	cudaStream_t stream = nullptr;
};
template <class K> struct EmuLaunch {
	K k;
	EmuCfg c;
	template <class... A> void operator()(A... a)
	{
		auto call = [&]() { k(a...); };
		emu_run_ctas(c.grid, c.block, c.smem, 1, [](void *p) { (*static_cast<decltype(call) *>(p))(); }, &call);
	}
};
template <class K> EmuLaunch<K> emu_launch(K k, EmuCfg c) { return EmuLaunch<K>{ k, c }; }
