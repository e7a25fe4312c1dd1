// Instantiations of dp16b_kernel<GAP_LINEAR, *, *> (packed 16-bit twin pairs, 4 x 4 blocks).
#define PA_GAPK GAP_LINEAR
#define PA_FN(x) x##_dp16b_linear
#include "pa_dp16b_inst.inc"
