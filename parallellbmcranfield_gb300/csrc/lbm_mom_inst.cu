// Launch table of the moment storage (lbm_mom.cuh): bulk step per collision
// model and tile, special-node step, first collision, finish and residual.
#include "lbm_internal.h"
#include "lbm_mom.cuh"

namespace lbm {

// The reference's residual line (serial/ComputeResiduals.c:6-51, cells
// 0..m-1 only) read through the moment accessor.
__global__ void __launch_bounds__(256) k_resid_mom(const __grid_constant__ StepArgs a,
                                                   double *out) {
  resid_body<AccMom<false>>(a, AccMom<false>(a, nullptr), out);
}

template <int MODEL>
void fill_mom_model(MomKernels &t) {
  t.step[MODEL][0] = (const void *)k_step_mom<MODEL, MOM_NPT[0], MOM_MINB[0], MOM_PFL[0], MOM_LD[0]>;
  t.step[MODEL][1] = (const void *)k_step_mom<MODEL, MOM_NPT[1], MOM_MINB[1], MOM_PFL[1], MOM_LD[1]>;
  t.step[MODEL][2] = (const void *)k_step_mom<MODEL, MOM_NPT[2], MOM_MINB[2], MOM_PFL[2], MOM_LD[2]>;
  t.step[MODEL][3] = (const void *)k_step_mom<MODEL, MOM_NPT[3], MOM_MINB[3], MOM_PFL[3], MOM_LD[3]>;
  static_assert(MOM_NVAR == 4, "moment tile table");
  t.special[MODEL] = (const void *)k_special_mom<MODEL>;
  t.init[MODEL] = (const void *)k_init_mom<MODEL>;
}

const MomKernels &kernels_mom() {
  static const MomKernels t = [] {
    MomKernels k{};
    fill_mom_model<1>(k);
    fill_mom_model<2>(k);
    fill_mom_model<3>(k);
    k.finish = (const void *)k_finish_mom;
    k.resid = (const void *)k_resid_mom;
    k.reduce = (const void *)k_reduce_partials;
    return k;
  }();
  return t;
}

}  // namespace lbm
