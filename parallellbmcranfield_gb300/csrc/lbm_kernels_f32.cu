// Kernel instantiations for StF32 population storage.
#include "lbm_kset.cuh"

LBM_DEFINE_KERNEL_SET(kernels_f32, StF32)
