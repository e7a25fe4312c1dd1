// Instantiations of dp16_kernel<GAP_LINEAR, *, *> (packed 16-bit twin pairs).
#define PA_GAPK GAP_LINEAR
#define PA_FN(x) x##_dp16_linear
#include "pa_dp16_inst.inc"
