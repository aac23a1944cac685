// One part of the kernel tables (see lbm_kset.cuh).  Compiled several times
// with -DLBM_PREC and -DLBM_PART; the FP64 objects are compiled with
// --fmad=false so that they keep the serial reference's roundings.
#include "lbm_kset.cuh"

#if !defined(LBM_PREC) || !defined(LBM_PART)
#error "compile with -DLBM_PREC=0..3 -DLBM_PART=0..3"
#endif

#if LBM_PREC == 0
#define LBM_ST StF64
#elif LBM_PREC == 1
#define LBM_ST StF32
#elif LBM_PREC == 2
#define LBM_ST StF16
#else
#define LBM_ST StB16
#endif

#define LBM_CAT3(a, b, c) a##b##_##c
#define LBM_PART_FN(p, q) LBM_CAT3(kernel_part_, p, q)

namespace lbm {
const KernelPart &LBM_PART_FN(LBM_PREC, LBM_PART)() {
#if LBM_PART == 0
  static const KernelPart part = make_io_part<LBM_ST>();
#else
  static const KernelPart part = make_model_part<LBM_ST, LBM_PART>();
#endif
  return part;
}
}  // namespace lbm
