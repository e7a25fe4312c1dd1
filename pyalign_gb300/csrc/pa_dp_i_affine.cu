// Instantiations of dp_kernel<int32_t, GAP_AFFINE, *, *> (split per family for parallel builds).
#include "pa_dp.cuh"
#include "pa_launch.h"

namespace pa {

cudaError_t launch_dp_i_affine(int loc, int tb, bool vals, const DpParams<int32_t> &p, int grid, size_t smem,
                                  cudaStream_t st) {
#define PA_CASE(L, T) PA_CASE2(L, T, false) PA_CASE2(L, T, true)
#define PA_CASE2(L, T, VA)                                                                   \
	if (loc == L && tb == T && vals == VA) {                                            \
		auto k = dp_kernel<int32_t, GAP_AFFINE, L, T, VA>;                                         \
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
#undef PA_CASE2
	return cudaErrorInvalidValue;
}

cudaError_t occupancy_dp_i_affine(int loc, int tb, bool vals, size_t smem, int *blocks_per_sm) {
	cudaError_t e = cudaErrorInvalidValue;
#define PA_OCC(L, T) PA_OCC2(L, T, false) PA_OCC2(L, T, true)
#define PA_OCC2(L, T, VA) \
	if (loc == L && tb == T && vals == VA) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, dp_kernel<int32_t, GAP_AFFINE, L, T, VA>, BLOCK, smem);
	PA_OCC(LOC_LOCAL, TB_NONE) PA_OCC(LOC_LOCAL, TB_ONE) PA_OCC(LOC_LOCAL, TB_ALL)
	PA_OCC(LOC_GLOBAL, TB_NONE) PA_OCC(LOC_GLOBAL, TB_ONE) PA_OCC(LOC_GLOBAL, TB_ALL)
	PA_OCC(LOC_SEMI, TB_NONE) PA_OCC(LOC_SEMI, TB_ONE) PA_OCC(LOC_SEMI, TB_ALL)
#undef PA_OCC
#undef PA_OCC2
	return e;
}

}  // namespace pa
