// Instantiations of dp_kernel<int32_t, GAP_LINEAR, *, *, *, true>: stripe-chained mode.
#define PA_VT int32_t
#define PA_GAPK GAP_LINEAR
#define PA_DTW 0
#define PA_CHAIN true
#define PA_FN(x) x##_dp_i_linear_chain
#include "pa_dp_inst.inc"
