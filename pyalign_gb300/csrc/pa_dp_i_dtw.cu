// Instantiations of dp_kernel<int32_t, GAP_DTW, *, *, *, false>: group mode.
#define PA_VT int32_t
#define PA_GAPK GAP_DTW
#define PA_DTW 1
#define PA_CHAIN false
#define PA_FN(x) x##_dp_i_dtw
#include "pa_dp_inst.inc"
