// Instantiations of dp_kernel<float, GAP_DTW, *, *, *, true>: stripe-chained mode.
#define PA_VT float
#define PA_GAPK GAP_DTW
#define PA_DTW 1
#define PA_CHAIN true
#define PA_FN(x) x##_dp_f_dtw_chain
#include "pa_dp_inst.inc"
