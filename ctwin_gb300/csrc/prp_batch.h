// Batch kernel interface (prp_batch.cu): several pools' launches of degrees
// 2^12..2^15 (4096 coefficients per CTA) in one persistent launch.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "prp_kernels.cuh"

namespace ctw {

// One class of work items: the launch a pool would make (its arguments, as for
// prp_launch over `items * (8 >> lg)` lanes), 2^lg CTAs per lane.
struct PrpBatchClass {
	PrpKernelArgs a;
	int lg;                     // 0..3: degree 2^(12 + lg)
	int items;                  // work items: lanes [i * (8 >> lg), (i + 1) * (8 >> lg))
	int pad[2];
};

// One persistent launch over ncls classes (largest degree first) of np NTT
// primes, built for occ (1 or 2) CTAs per SM; d_heads[ncls] must be zero (the
// per-class queue heads).
cudaError_t prp_batch_launch(int np, int occ, const PrpBatchClass *d_cls, int ncls, int total_items, unsigned *d_heads,
                             cudaStream_t stream);
// Clusters of 8 CTAs the device holds at once for that build.
int prp_batch_max_clusters(int np, int occ);

}  // namespace ctw
