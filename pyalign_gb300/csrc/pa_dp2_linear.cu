// Instantiations of dp2_kernel<GAP_LINEAR, *, *, *> (two columns per lane step, int32 tagged).
#define PA_GAPK GAP_LINEAR
#define PA_DTW 0
#define PA_FN(x) x##_dp2_linear
#include "pa_dp2_inst.inc"
