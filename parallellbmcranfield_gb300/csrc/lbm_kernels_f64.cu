// Kernel instantiations for StF64 population storage.
// Compiled with --fmad=false: the FP64 mode keeps every rounding of the
// serial reference (no multiply-add contraction).
#include "lbm_kset.cuh"

LBM_DEFINE_KERNEL_SET(kernels_f64, StF64)
