// Kernel instantiations for StF16 population storage.
#include "lbm_kset.cuh"

LBM_DEFINE_KERNEL_SET(kernels_f16, StF16)
