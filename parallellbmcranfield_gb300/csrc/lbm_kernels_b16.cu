// Kernel instantiations for StB16 population storage.
#include "lbm_kset.cuh"

LBM_DEFINE_KERNEL_SET(kernels_b16, StB16)
