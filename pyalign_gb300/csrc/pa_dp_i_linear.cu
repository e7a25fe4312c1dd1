// Instantiations of dp_kernel<int32_t, GAP_LINEAR, *, *> (split per family for parallel builds).
#include "pa_dp.cuh"
#include "pa_launch.h"

namespace pa {

cudaError_t launch_dp_i_linear(int loc, int tb, const DpParams<int32_t> &p, int grid, size_t smem,
                                  cudaStream_t st) {
#define PA_CASE(L, T)                                                                       \
	if (loc == L && tb == T) {                                                          \
		auto k = dp_kernel<int32_t, GAP_LINEAR, L, T>;                                         \
		if (smem > 48 * 1024)                                                           \
			cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)); \
		k<<<grid, BLOCK, smem, st>>>(p);                                                \
		return cudaGetLastError();                                                      \
	}
	PA_CASE(LOC_LOCAL, TB_NONE)
	PA_CASE(LOC_LOCAL, TB_ONE)
	PA_CASE(LOC_LOCAL, TB_ALL)
	PA_CASE(LOC_GLOBAL, TB_NONE)
	PA_CASE(LOC_GLOBAL, TB_ONE)
	PA_CASE(LOC_GLOBAL, TB_ALL)
	PA_CASE(LOC_SEMI, TB_NONE)
	PA_CASE(LOC_SEMI, TB_ONE)
	PA_CASE(LOC_SEMI, TB_ALL)
#undef PA_CASE
	return cudaErrorInvalidValue;
}

cudaError_t occupancy_dp_i_linear(int loc, int tb, size_t smem, int *blocks_per_sm) {
	cudaError_t e = cudaErrorInvalidValue;
#define PA_OCC(L, T) \
	if (loc == L && tb == T) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, dp_kernel<int32_t, GAP_LINEAR, L, T>, BLOCK, smem);
	PA_OCC(LOC_LOCAL, TB_NONE) PA_OCC(LOC_LOCAL, TB_ONE) PA_OCC(LOC_LOCAL, TB_ALL)
	PA_OCC(LOC_GLOBAL, TB_NONE) PA_OCC(LOC_GLOBAL, TB_ONE) PA_OCC(LOC_GLOBAL, TB_ALL)
	PA_OCC(LOC_SEMI, TB_NONE) PA_OCC(LOC_SEMI, TB_ONE) PA_OCC(LOC_SEMI, TB_ALL)
#undef PA_OCC
	return e;
}

}  // namespace pa
