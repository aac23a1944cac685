// Batched-step kernels for one storage precision (compiled with
// -DLBM_PREC=0 (FP64, --fmad=false), 1 (FP32) or 2 (FP16-dev)).
#include "lbm_batch.cuh"

#if !defined(LBM_PREC)
#error "compile with -DLBM_PREC=0..2"
#endif
#if LBM_PREC == 0
#define LBM_ST StF64
#elif LBM_PREC == 1
#define LBM_ST StF32
#else
#define LBM_ST StF16
#endif

#define LBM_CAT2(a, b) a##b
#define LBM_BATCH_FN(p) LBM_CAT2(batch_kernels_, p)

namespace lbm {

template <class ST, int MODEL>
void fill_batch_steps(const void *out[BVAR]) {
  out[0] = (const void *)k_batch_step<ST, MODEL, BVAR_BX[0], BVAR_NPT[0]>;
  out[1] = (const void *)k_batch_step<ST, MODEL, BVAR_BX[1], BVAR_NPT[1]>;
  out[2] = (const void *)k_batch_step<ST, MODEL, BVAR_BX[2], BVAR_NPT[2]>;
  out[3] = (const void *)k_batch_step<ST, MODEL, BVAR_BX[3], BVAR_NPT[3]>;
  static_assert(BVAR == 4, "batch tile table");
}

const BatchKernels &LBM_BATCH_FN(LBM_PREC)() {
  static const BatchKernels bk = [] {
    BatchKernels k{};
    fill_batch_steps<LBM_ST, 1>(k.step[1]);
    fill_batch_steps<LBM_ST, 2>(k.step[2]);
    fill_batch_steps<LBM_ST, 3>(k.step[3]);
    k.special[1] = (const void *)k_batch_special<LBM_ST, 1>;
    k.special[2] = (const void *)k_batch_special<LBM_ST, 2>;
    k.special[3] = (const void *)k_batch_special<LBM_ST, 3>;
    k.du = (const void *)k_batch_du<LBM_ST>;
    k.advance = (const void *)k_batch_advance;
    k.converge = (const void *)k_batch_converge;
    k.compact_tiles = (const void *)k_batch_compact<int4>;
    k.compact_special = (const void *)k_batch_compact<int2>;
    return k;
  }();
  return bk;
}

}  // namespace lbm
