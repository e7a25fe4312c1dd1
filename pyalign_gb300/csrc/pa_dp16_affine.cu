// Instantiations of dp16_kernel<GAP_AFFINE, *, *> (packed 16-bit twin pairs).
#define PA_GAPK GAP_AFFINE
#define PA_FN(x) x##_dp16_affine
#include "pa_dp16_inst.inc"
