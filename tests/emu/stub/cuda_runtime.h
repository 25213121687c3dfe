// Minimal stand-in for the CUDA runtime header (host emulation of the kernels).
#pragma once
#include <cstddef>
#include <cstdint>
typedef int cudaError_t;
typedef void *cudaStream_t;
enum { cudaSuccess = 0 };
