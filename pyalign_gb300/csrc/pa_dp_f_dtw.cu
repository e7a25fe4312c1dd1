// Instantiations of dp_kernel<float, GAP_DTW, *, *, *, false>: group mode.
#define PA_VT float
#define PA_GAPK GAP_DTW
#define PA_DTW 1
#define PA_CHAIN false
#define PA_FN(x) x##_dp_f_dtw
#include "pa_dp_inst.inc"
