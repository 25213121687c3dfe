// Launch dispatch of the two-prime PRP kernels (instantiated here, apart from
// the three-prime ones, so that both halves compile in parallel).
#include "prp_kernel_impl.cuh"

namespace ctw {

cudaError_t prp_launch_np2(const PrpKernelArgs &a, int lg, int lanes, cudaStream_t stream)
{
	if (!prp_two_prime_split(a.lm, lg)) return cudaErrorInvalidValue;
	PrpKernelArgs a2 = a;     // two planes of roots may fit where three do not
	a2.tw_smem = prp_smem_bytes(a.lm, lg, 1, 2) <= 227 * 1024 ? 1 : 0;
	if (a.lm == 13 && lg == 4) return launch_lg<4, false, true, 2>(a2, lanes, stream);   // 2^17 on 16 CTAs
	if (a.lm != 12) return launch_lg<0, false, false, 2>(a2, lanes, stream);
	// dense: two CTAs per SM once the launch fills the SMs at one per SM
	const bool dense = a.dense > 0 || (a.dense == 0 && lg > 0 && (lanes << lg) >= prp_device_sms());
	if (dense && lg > 0)
	{
		a2.tw_smem = 0;       // two CTAs per SM: roots from L1 / L2
		switch (lg)
		{
		case 1: return launch_lg<1, true, true, 2, true>(a2, lanes, stream);
		case 2: return launch_lg<2, true, true, 2, true>(a2, lanes, stream);
		case 3: return launch_lg<3, true, true, 2, true>(a2, lanes, stream);
		default: return launch_lg<4, true, true, 2, true>(a2, lanes, stream);
		}
	}
	switch (lg)
	{
	case 0: return launch_lg<0, true, false, 2>(a2, lanes, stream);
	case 1: return launch_lg<1, true, true, 2>(a2, lanes, stream);
	case 2: return launch_lg<2, true, true, 2>(a2, lanes, stream);
	case 3: return launch_lg<3, true, true, 2>(a2, lanes, stream);
	default: return launch_lg<4, true, true, 2>(a2, lanes, stream);
	}
}

}  // namespace ctw
