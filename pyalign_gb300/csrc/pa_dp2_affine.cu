// Instantiations of dp2_kernel<GAP_AFFINE, *, *, *> (two columns per lane step, int32 tagged).
#define PA_GAPK GAP_AFFINE
#define PA_DTW 0
#define PA_FN(x) x##_dp2_affine
#include "pa_dp2_inst.inc"
