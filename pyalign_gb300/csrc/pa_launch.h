// Launch entry points of the DP kernel families (one translation unit each).
#pragma once
#include "pa_dp.cuh"

namespace pa {

#define PA_DECL(V, VT, GAP)                                                                      \
	cudaError_t launch_dp_##V##_##GAP(int loc, int tb, bool vals, const DpParams<VT> &p, int grid, size_t smem, \
	                                  cudaStream_t st);                                          \
	cudaError_t occupancy_dp_##V##_##GAP(int loc, int tb, bool vals, size_t smem, int *blocks_per_sm);
PA_DECL(i, int32_t, linear)
PA_DECL(i, int32_t, affine)
PA_DECL(i, int32_t, dtw)
PA_DECL(f, float, linear)
PA_DECL(f, float, affine)
PA_DECL(f, float, dtw)
PA_DECL(i, int32_t, linear_chain)
PA_DECL(i, int32_t, affine_chain)
PA_DECL(i, int32_t, dtw_chain)
PA_DECL(f, float, linear_chain)
PA_DECL(f, float, affine_chain)
PA_DECL(f, float, dtw_chain)
#undef PA_DECL

#define PA_DECL2(GAP)                                                                                      \
	cudaError_t launch_dp2_##GAP(int loc, int tb, bool chain, const DpParams<int32_t> &p, int grid, size_t smem, \
	                             cudaStream_t st);                                                     \
	cudaError_t occupancy_dp2_##GAP(int loc, int tb, bool chain, size_t smem, int *blocks_per_sm);
PA_DECL2(linear)
PA_DECL2(affine)
PA_DECL2(dtw)
#undef PA_DECL2

#define PA_DECL16(GAP)                                                                                  \
	cudaError_t launch_dp16_##GAP(int loc, int tb, int cols, const DpParams<int32_t> &p, int grid, size_t smem, \
	                              cudaStream_t st);                                                 \
	cudaError_t occupancy_dp16_##GAP(int loc, int tb, int cols, size_t smem, int *blocks_per_sm);
PA_DECL16(linear)
PA_DECL16(affine)
#undef PA_DECL16

#define PA_DECL16B(GAP)                                                                                 \
	cudaError_t launch_dp16b_##GAP(int loc, int tb, const DpParams<int32_t> &p, int grid, size_t smem,  \
	                               cudaStream_t st);                                                 \
	cudaError_t occupancy_dp16b_##GAP(int loc, int tb, size_t smem, int *blocks_per_sm);
PA_DECL16B(linear)
PA_DECL16B(affine)
#undef PA_DECL16B

}  // namespace pa
