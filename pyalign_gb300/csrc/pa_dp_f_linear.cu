// Instantiations of dp_kernel<float, GAP_LINEAR, *, *, *, false>: group mode.
#define PA_VT float
#define PA_GAPK GAP_LINEAR
#define PA_DTW 0
#define PA_CHAIN false
#define PA_FN(x) x##_dp_f_linear
#include "pa_dp_inst.inc"
