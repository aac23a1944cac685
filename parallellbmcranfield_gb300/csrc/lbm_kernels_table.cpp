// Assembles the per-precision launch tables from the separately compiled parts.
#include "lbm_internal.h"

namespace lbm {

#define LBM_DECL_PARTS(P)                 \
  const KernelPart &kernel_part_##P##_0(); \
  const KernelPart &kernel_part_##P##_1(); \
  const KernelPart &kernel_part_##P##_2(); \
  const KernelPart &kernel_part_##P##_3();
LBM_DECL_PARTS(0)
LBM_DECL_PARTS(1)
LBM_DECL_PARTS(2)
LBM_DECL_PARTS(3)

namespace {
KernelSet assemble(const KernelPart &io, const KernelPart &m1, const KernelPart &m2,
                   const KernelPart &m3) {
  KernelSet ks{};
  const KernelPart *mp[4] = {nullptr, &m1, &m2, &m3};
  for (int m = 1; m <= 3; m++) {
    for (int ph = 0; ph < 3; ph++)
      for (int v = 0; v < NVAR; v++) ks.step[m][ph][v] = mp[m]->step[ph][v];
    ks.init[m][0] = mp[m]->init[0];
    ks.init[m][1] = mp[m]->init[1];
  }
  for (int l = 0; l < 3; l++) {
    ks.finish[l] = io.finish[l];
    ks.resid[l] = io.resid[l];
  }
  ks.reduce = io.reduce;
  ks.elem_size = io.elem_size;
  return ks;
}
}  // namespace

#define LBM_SET(NAME, P)                                                                 \
  const KernelSet &NAME() {                                                              \
    static const KernelSet ks = assemble(kernel_part_##P##_0(), kernel_part_##P##_1(),   \
                                         kernel_part_##P##_2(), kernel_part_##P##_3());  \
    return ks;                                                                           \
  }
LBM_SET(kernels_f64, 0)
LBM_SET(kernels_f32, 1)
LBM_SET(kernels_f16, 2)
LBM_SET(kernels_b16, 3)

}  // namespace lbm
