// Batch kernel: the squaring (or multiply) launches of several pools of
// different degrees 2^12..2^15 in ONE persistent launch.
//
// Every CTA holds 4096 coefficients (the radix-16 path), so a candidate of
// degree 2^(12+lg) takes 2^lg CTAs.  The launch is made of clusters of 8 CTAs
// that stay resident and take work items from per-degree queues, largest
// degree first: an item of class c (one pool's launch) is 8 >> lg lanes of
// that pool, each on 2^lg CTAs of the cluster (a 2^15 candidate fills the
// cluster; eight 2^12 candidates take one CTA each).  The item runs the
// pool's own launch body (prp_body / cols_body of prp_kernel_impl.cuh, with
// the cluster ranks of its lane group) for the class's count of squarings, so
// every lane's registers are those of the pool's own launch.  A cluster whose
// queues are empty leaves.
#include "prp_kernel_impl.cuh"
#include "prp_batch.h"

namespace ctw {

namespace {

constexpr int BATCH_CLUSTER = 8;

__device__ __forceinline__ unsigned ld_volatile_u32(const unsigned *p)
{
	return *reinterpret_cast<const volatile unsigned *>(p);
}

// One item of lanes on 2^LGI CTAs each; not inlined, so that every body gets
// the build's registers to itself instead of sharing one allocation.
template <int NP, int LGI>
__device__ __noinline__ void batch_item(const PrpKernelArgs &a, uint32_t *sm, int lane, int g, int rbase)
{
	if constexpr (LGI == 0) prp_body<0, true, NP, true>(a, sm, lane, 0);
	else cols_body<LGI, true, NP, true>(a, sm, lane, g, rbase);
}

template <int NP> struct BatchBounds {
	static constexpr int threads = NP == 2 ? 512 : 384;    // the 4096-coefficient dense builds
};

// OCC: CTAs per SM the build is compiled for (2: 64 / 80 registers, some
// spills; 1: up to 128 registers), an autotuning choice.
template <int NP, int OCC>
__global__ void __launch_bounds__(BatchBounds<NP>::threads, OCC)
    prp_kernel_batch(const PrpBatchClass *__restrict__ cls, int ncls, unsigned *heads, int item_off)
{
	extern __shared__ __align__(16) uint32_t sm[];
	// class and index of the current item, written into every CTA by rank 0 of
	// the cluster, after the words the launch bodies use; then the class's
	// launch arguments, copied into shared memory for the item's bodies
	int *item = reinterpret_cast<int *>(sm + item_off);
	PrpKernelArgs *sa = reinterpret_cast<PrpKernelArgs *>(sm + item_off + 4);
	cg::cluster_group cl = cg::this_cluster();
	const int rank = (int)cl.block_rank();
	for (;;)
	{
		if (rank == 0 && threadIdx.x == 0)
		{
			int c = -1, idx = 0;
			for (int q = 0; q < ncls && c < 0; ++q)
			{
				const unsigned n = (unsigned)cls[q].items;
				if (ld_volatile_u32(heads + q) >= n) continue;     // queue empty: no atomic
				const unsigned i = atomicAdd(heads + q, 1u);
				if (i < n)
				{
					c = q;
					idx = (int)i;
				}
			}
			for (int r = 0; r < BATCH_CLUSTER; ++r)
			{
				int *dst = cl.map_shared_rank(item, r);
				dst[0] = c;
				dst[1] = idx;
			}
		}
		cl.sync();
		const int c = item[0], idx = item[1];
		if (c < 0) break;
		const PrpBatchClass &C = cls[c];
		{
			const uint32_t *src = reinterpret_cast<const uint32_t *>(&C.a);
			uint32_t *dst = reinterpret_cast<uint32_t *>(sa);
			for (int i = threadIdx.x; i < (int)(sizeof(PrpKernelArgs) / 4); i += blockDim.x) dst[i] = src[i];
		}
		__syncthreads();
		const int lg = C.lg;
		const int sub = rank >> lg, g = rank & ((1 << lg) - 1);
		const int lane = idx * (BATCH_CLUSTER >> lg) + sub;
		switch (lg)
		{
		case 0: batch_item<NP, 0>(*sa, sm, lane, 0, 0); break;
		case 1: batch_item<NP, 1>(*sa, sm, lane, g, sub << 1); break;
		case 2: batch_item<NP, 2>(*sa, sm, lane, g, sub << 2); break;
		default: batch_item<NP, 3>(*sa, sm, lane, g, 0); break;
		}
		cl.sync();                                   // every CTA done before the next item is posted
	}
}

// Bytes of shared memory the launch bodies use (the item words follow).
template <int NP>
size_t batch_body_smem()
{
	size_t m = 0;
	for (int lg = 0; lg <= 3; ++lg) m = std::max(m, prp_smem_bytes(12, lg, 0, NP));
	return NP == 3 ? m - prp_shoup_words(12, 3) * 4 : m;    // the three-prime build reads its Shoup roots from L2
}
template <int NP> size_t batch_smem() { return batch_body_smem<NP>() + 16 + (sizeof(PrpKernelArgs) + 15) / 16 * 16; }

template <int NP, int OCC>
cudaError_t batch_launch_t(const PrpBatchClass *d_cls, int ncls, int total_items, unsigned *d_heads,
                           cudaStream_t stream)
{
	void (*kern)(const PrpBatchClass *, int, unsigned *, int) = prp_kernel_batch<NP, OCC>;
	const size_t smem = batch_smem<NP>();
	cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e != cudaSuccess) return e;
	cudaLaunchConfig_t cfg = {};
	cfg.blockDim = dim3(BatchBounds<NP>::threads);
	cfg.dynamicSmemBytes = smem;
	cfg.stream = stream;
	cudaLaunchAttribute at[1];
	at[0].id = cudaLaunchAttributeClusterDimension;
	at[0].val.clusterDim.x = BATCH_CLUSTER;
	at[0].val.clusterDim.y = 1;
	at[0].val.clusterDim.z = 1;
	cfg.attrs = at;
	cfg.numAttrs = 1;
	static int max_clusters = 0;                 // per instance: resident clusters of this build
	if (max_clusters == 0)
	{
		cfg.gridDim = dim3(BATCH_CLUSTER);
		int n = 0;
		e = cudaOccupancyMaxActiveClusters(&n, kern, &cfg);
		if (e != cudaSuccess) return e;
		max_clusters = n > 0 ? n : 1;
	}
	const int clusters = std::max(1, std::min(total_items, max_clusters));
	cfg.gridDim = dim3(clusters * BATCH_CLUSTER);
	return cudaLaunchKernelEx(&cfg, kern, d_cls, ncls, d_heads, (int)(batch_body_smem<NP>() / 4));
}

}  // namespace

cudaError_t prp_batch_launch(int np, int occ, const PrpBatchClass *d_cls, int ncls, int total_items, unsigned *d_heads,
                             cudaStream_t stream)
{
	if (ncls <= 0 || total_items <= 0) return cudaSuccess;
	if (np == 2)
		return occ == 1 ? batch_launch_t<2, 1>(d_cls, ncls, total_items, d_heads, stream)
		                : batch_launch_t<2, 2>(d_cls, ncls, total_items, d_heads, stream);
	return occ == 1 ? batch_launch_t<3, 1>(d_cls, ncls, total_items, d_heads, stream)
	                : batch_launch_t<3, 2>(d_cls, ncls, total_items, d_heads, stream);
}

int prp_batch_max_clusters(int np, int occ)
{
	void (*kern)(const PrpBatchClass *, int, unsigned *, int) =
	    np == 2 ? (occ == 1 ? prp_kernel_batch<2, 1> : prp_kernel_batch<2, 2>)
	            : (occ == 1 ? prp_kernel_batch<3, 1> : prp_kernel_batch<3, 2>);
	const size_t smem = np == 2 ? batch_smem<2>() : batch_smem<3>();
	if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 0;
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3(BATCH_CLUSTER);
	cfg.blockDim = dim3(np == 2 ? 512 : 384);
	cfg.dynamicSmemBytes = smem;
	cudaLaunchAttribute at[1];
	at[0].id = cudaLaunchAttributeClusterDimension;
	at[0].val.clusterDim.x = BATCH_CLUSTER;
	at[0].val.clusterDim.y = 1;
	at[0].val.clusterDim.z = 1;
	cfg.attrs = at;
	cfg.numAttrs = 1;
	int n = 0;
	if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) != cudaSuccess) return 0;
	return n;
}

}  // namespace ctw
