// Instantiates the kernel templates for one storage policy and exposes them
// as a launch table (included once by each lbm_kernels_<precision>.cu).
#pragma once
#include "lbm_device.cuh"
#include "lbm_internal.h"

#define LBM_STEPS(ST, MODEL)                                                       \
  {(const void *)k_step<ST, MODEL, PH_AB>, (const void *)k_step<ST, MODEL, PH_AA_A>, \
   (const void *)k_step<ST, MODEL, PH_AA_B>}
#define LBM_INITS(ST, MODEL) \
  {(const void *)k_init<ST, MODEL, PH_AB>, (const void *)k_init<ST, MODEL, PH_AA_A>}

#define LBM_DEFINE_KERNEL_SET(FUNC, ST)                                                    \
  namespace lbm {                                                                          \
  const KernelSet &FUNC() {                                                                \
    static const KernelSet ks = {                                                          \
        {{nullptr, nullptr, nullptr}, LBM_STEPS(ST, 1), LBM_STEPS(ST, 2), LBM_STEPS(ST, 3)}, \
        {{nullptr, nullptr}, LBM_INITS(ST, 1), LBM_INITS(ST, 2), LBM_INITS(ST, 3)},        \
        {(const void *)k_finish<ST, PH_AB>, (const void *)k_finish<ST, PH_AA_A>,          \
         (const void *)k_finish<ST, PH_AA_B>},                                             \
        {(const void *)k_resid_ref<ST, PH_AB>, (const void *)k_resid_ref<ST, PH_AA_A>,    \
         (const void *)k_resid_ref<ST, PH_AA_B>},                                          \
        (const void *)k_reduce_partials, (int)sizeof(typename ST::T)};                                                      \
    return ks;                                                                             \
  }                                                                                        \
  }
