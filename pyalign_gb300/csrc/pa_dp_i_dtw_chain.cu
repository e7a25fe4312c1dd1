// Instantiations of dp_kernel<int32_t, GAP_DTW, *, *, *, true>: stripe-chained mode.
#define PA_VT int32_t
#define PA_GAPK GAP_DTW
#define PA_DTW 1
#define PA_CHAIN true
#define PA_FN(x) x##_dp_i_dtw_chain
#include "pa_dp_inst.inc"
