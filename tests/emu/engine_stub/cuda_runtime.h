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
#include <functional>
#include <utility>
#include <vector>

// Stream capture: while a capture is open, copies, sets and launches are
// recorded (their arguments by value) instead of run; a graph launch replays
// them in order.  Host memory behind a recorded copy is read at replay, as a
// captured host-to-device copy reads it when the graph runs.
extern std::vector<std::function<void()>> *emu_capture;
inline void emu_issue(std::function<void()> f)
{
	if (emu_capture) emu_capture->push_back(std::move(f));
	else f();
}
struct EmuGraph {
	std::vector<std::function<void()>> ops;
};
typedef EmuGraph *cudaGraph_t;
typedef EmuGraph *cudaGraphExec_t;
enum cudaStreamCaptureMode { cudaStreamCaptureModeRelaxed = 2 };
enum cudaStreamCaptureStatus { cudaStreamCaptureStatusNone = 0, cudaStreamCaptureStatusActive = 1 };
enum { cudaEventDisableTiming = 2 };

typedef int cudaError_t;
enum { cudaSuccess = 0, cudaErrorInvalidValue = 1, cudaErrorMemoryAllocation = 2, cudaErrorNotReady = 600 };
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
inline cudaError_t cudaSetDevice(int) { return cudaSuccess; }
template <class T> inline cudaError_t cudaGetSymbolAddress(void **p, const T &sym)
{
	*p = (void *)&sym;
	return cudaSuccess;
}
inline cudaError_t cudaMemGetInfo(size_t *fr, size_t *tot)
{
	*fr = (size_t)1 << 32;
	*tot = (size_t)1 << 33;
	return cudaSuccess;
}
inline cudaError_t cudaGetDeviceCount(int *n) { *n = 1; return cudaSuccess; }
inline cudaError_t cudaDeviceGetAttribute(int *v, cudaDeviceAttr, int) { *v = 152; return cudaSuccess; }
template <class F> inline cudaError_t cudaFuncSetAttribute(F, cudaFuncAttribute, int) { return cudaSuccess; }
template <class F> inline cudaError_t cudaOccupancyMaxActiveBlocksPerMultiprocessor(int *n, F, int, size_t)
{
	*n = 1;
	return cudaSuccess;
}
template <class F, class C> inline cudaError_t cudaOccupancyMaxActiveClusters(int *n, F, const C *)
{
	*n = 2;
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
	emu_issue([=]() { memmove(d, s, n); });
	return cudaSuccess;
}
template <class T> inline cudaError_t cudaMallocHost(T **p, size_t n)
{
	*p = (T *)malloc(n ? n : 1);
	return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
inline cudaError_t cudaFreeHost(void *p) { free(p); return cudaSuccess; }
inline cudaError_t cudaMemcpy2DAsync(void *d, size_t dp, const void *s, size_t sp, size_t w, size_t h, cudaMemcpyKind,
                                     cudaStream_t = nullptr)
{
	emu_issue([=]() {
		for (size_t r = 0; r < h; ++r) memmove((char *)d + r * dp, (const char *)s + r * sp, w);
	});
	return cudaSuccess;
}
inline cudaError_t cudaMemset(void *p, int v, size_t n) { memset(p, v, n); return cudaSuccess; }
inline cudaError_t cudaMemsetAsync(void *p, int v, size_t n, cudaStream_t = nullptr)
{
	emu_issue([=]() { memset(p, v, n); });
	return cudaSuccess;
}
inline cudaError_t cudaStreamCreateWithFlags(cudaStream_t *s, unsigned) { *s = malloc(1); return cudaSuccess; }
inline cudaError_t cudaStreamDestroy(cudaStream_t s) { free(s); return cudaSuccess; }
inline cudaError_t cudaStreamSynchronize(cudaStream_t) { return cudaSuccess; }
inline cudaError_t cudaEventCreate(cudaEvent_t *e) { *e = new int(0); return cudaSuccess; }
inline cudaError_t cudaEventCreateWithFlags(cudaEvent_t *e, unsigned) { *e = new int(0); return cudaSuccess; }
inline cudaError_t cudaEventQuery(cudaEvent_t) { return cudaSuccess; }
inline cudaError_t cudaStreamBeginCapture(cudaStream_t, cudaStreamCaptureMode)
{
	if (emu_capture) return cudaErrorInvalidValue;
	emu_capture = new std::vector<std::function<void()>>();
	return cudaSuccess;
}
inline cudaError_t cudaStreamIsCapturing(cudaStream_t, cudaStreamCaptureStatus *st)
{
	*st = emu_capture ? cudaStreamCaptureStatusActive : cudaStreamCaptureStatusNone;
	return cudaSuccess;
}
inline cudaError_t cudaStreamEndCapture(cudaStream_t, cudaGraph_t *g)
{
	if (!emu_capture) return cudaErrorInvalidValue;
	*g = new EmuGraph{ std::move(*emu_capture) };
	delete emu_capture;
	emu_capture = nullptr;
	return cudaSuccess;
}
inline cudaError_t cudaGraphInstantiate(cudaGraphExec_t *e, cudaGraph_t g, unsigned long long)
{
	*e = new EmuGraph(*g);
	return cudaSuccess;
}
inline cudaError_t cudaGraphDestroy(cudaGraph_t g) { delete g; return cudaSuccess; }
inline cudaError_t cudaGraphExecDestroy(cudaGraphExec_t e) { delete e; return cudaSuccess; }
inline cudaError_t cudaGraphLaunch(cudaGraphExec_t e, cudaStream_t)
{
	for (auto &f : e->ops) f();
	return cudaSuccess;
}
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
	const dim3 grid = c->gridDim, block = c->blockDim;
	const size_t smem = c->dynamicSmemBytes;
	emu_issue([=]() {
		auto call = [&]() { k(a...); };
		emu_run_ctas(grid, block, smem, group, [](void *p) { (*static_cast<decltype(call) *>(p))(); }, &call);
	});
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
		const K kk = k;
		const EmuCfg cc = c;
		emu_issue([=]() {
			auto call = [&]() { kk(a...); };
			emu_run_ctas(cc.grid, cc.block, cc.smem, 1, [](void *p) { (*static_cast<decltype(call) *>(p))(); }, &call);
		});
	}
};
template <class K> EmuLaunch<K> emu_launch(K k, EmuCfg c) { return EmuLaunch<K>{ k, c }; }
