// Instantiates the kernel templates for one storage precision and one part
// (io kernels, or the step/init kernels of one collision model) as a launch
// table.  lbm_kernels_inst.cu includes this once per object; build.py
// compiles it with -DLBM_PREC=0..3 (FP64, FP32, FP16-dev, BF16-dev) and
// -DLBM_PART=0..3 (0: finish/residual/reduce, 1..3: collision model).
#pragma once
#include "lbm_device.cuh"
#include "lbm_internal.h"

namespace lbm {

template <class ST, int MODEL, int PH, int I>
const void *step_variant() {
  constexpr TileVariant V = VARS[I];
  if constexpr (V.kind == 0)
    return (const void *)k_step<ST, MODEL, PH, V.bx, V.npt>;
  else if constexpr (V.kind == 1)
    return (const void *)k_step_vec<ST, MODEL, PH, V.bx, V.v, V.npt>;
  else if constexpr (V.kind == 3) {
    if constexpr (sizeof(typename ST::T) == 2)
      return (const void *)k_step_h2<ST, MODEL, PH, V.npt>;
    else
      return (const void *)k_step<ST, MODEL, PH, 128, V.npt>;
  }
  else
    return (const void *)k_step_tma<ST, MODEL, PH, V.tx, V.ty, V.rpt>;
}

template <class ST, int MODEL, int PH>
void fill_variants(const void *out[NVAR]) {
  out[0] = step_variant<ST, MODEL, PH, 0>();
  out[1] = step_variant<ST, MODEL, PH, 1>();
  out[2] = step_variant<ST, MODEL, PH, 2>();
  out[3] = step_variant<ST, MODEL, PH, 3>();
  out[4] = step_variant<ST, MODEL, PH, 4>();
  out[5] = step_variant<ST, MODEL, PH, 5>();
  static_assert(NVAR == 6, "variant table");
}

template <class ST, int MODEL>
KernelPart make_model_part() {
  KernelPart p{};
  fill_variants<ST, MODEL, PH_AB>(p.step[PH_AB]);
  fill_variants<ST, MODEL, PH_AA_A>(p.step[PH_AA_A]);
  fill_variants<ST, MODEL, PH_AA_B>(p.step[PH_AA_B]);
  p.init[0] = (const void *)k_init<ST, MODEL, PH_AB>;
  p.init[1] = (const void *)k_init<ST, MODEL, PH_AA_A>;
  return p;
}

template <class ST>
KernelPart make_io_part() {
  KernelPart p{};
  p.finish[PH_AB] = (const void *)k_finish<ST, PH_AB>;
  p.finish[PH_AA_A] = (const void *)k_finish<ST, PH_AA_A>;
  p.finish[PH_AA_B] = (const void *)k_finish<ST, PH_AA_B>;
  p.resid[PH_AB] = (const void *)k_resid_ref<ST, PH_AB>;
  p.resid[PH_AA_A] = (const void *)k_resid_ref<ST, PH_AA_A>;
  p.resid[PH_AA_B] = (const void *)k_resid_ref<ST, PH_AA_B>;
  p.reduce = (const void *)k_reduce_partials;
  p.elem_size = (int)sizeof(typename ST::T);
  return p;
}

}  // namespace lbm
