// Instantiations of dp_kernel<float, GAP_AFFINE, *, *, *, true>: stripe-chained mode.
#define PA_VT float
#define PA_GAPK GAP_AFFINE
#define PA_DTW 0
#define PA_CHAIN true
#define PA_FN(x) x##_dp_f_affine_chain
#include "pa_dp_inst.inc"
