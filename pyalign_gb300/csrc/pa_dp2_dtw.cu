// Instantiations of dp2_kernel<GAP_DTW, *, *, *> (two columns per lane step, int32 tagged).
#define PA_GAPK GAP_DTW
#define PA_DTW 1
#define PA_FN(x) x##_dp2_dtw
#include "pa_dp2_inst.inc"
