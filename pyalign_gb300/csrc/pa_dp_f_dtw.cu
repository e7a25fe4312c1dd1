// Instantiations of dp_kernel<float, GAP_DTW, *, *> (split per family for parallel builds).
#include "pa_dp.cuh"
#include "pa_launch.h"

namespace pa {

cudaError_t launch_dp_f_dtw(int loc, int tb, const DpParams<float> &p, int grid, size_t smem,
                                  cudaStream_t st) {
#define PA_CASE(L, T)                                                                       \
	if (loc == L && tb == T) {                                                          \
		auto k = dp_kernel<float, GAP_DTW, L, T>;                                         \
		if (smem > 48 * 1024)                                                           \
			cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)); \
		k<<<grid, BLOCK, smem, st>>>(p);                                                \
		return cudaGetLastError();                                                      \
	}
	PA_CASE(LOC_GLOBAL, TB_NONE)
	PA_CASE(LOC_GLOBAL, TB_ONE)
#undef PA_CASE
	return cudaErrorInvalidValue;
}

cudaError_t occupancy_dp_f_dtw(int loc, int tb, size_t smem, int *blocks_per_sm) {
	cudaError_t e = cudaErrorInvalidValue;
#define PA_OCC(L, T) \
	if (loc == L && tb == T) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, dp_kernel<float, GAP_DTW, L, T>, BLOCK, smem);
	PA_OCC(LOC_GLOBAL, TB_NONE) PA_OCC(LOC_GLOBAL, TB_ONE)
#undef PA_OCC
	return e;
}

}  // namespace pa
