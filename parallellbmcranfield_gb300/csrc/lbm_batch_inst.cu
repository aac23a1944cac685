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

// FP64 (the parity mode, whose MRT reads the full stmiv table) keeps the
// persistent kernel over full case arguments; FP32 and FP16-dev take the
// per-tile bulk kernel over compact arguments.
template <class ST, int MODEL, int V>
const void *batch_step_fn() {
  if constexpr (std::is_same<ST, StF64>::value)
    return (const void *)k_batch_step<ST, MODEL, BVAR_BX[V], BVAR_NPT[V]>;
  else
    return (const void *)k_batch_bulk<ST, MODEL, BVAR_BX[V], BVAR_NPT[V]>;
}

template <class ST, int MODEL>
void fill_batch_steps(const void *out[BVAR]) {
  out[0] = batch_step_fn<ST, MODEL, 0>();
  out[1] = batch_step_fn<ST, MODEL, 1>();
  out[2] = batch_step_fn<ST, MODEL, 2>();
  out[3] = batch_step_fn<ST, MODEL, 3>();
  static_assert(BVAR == 4, "batch tile table");
}

const BatchKernels &LBM_BATCH_FN(LBM_PREC)() {
  static const BatchKernels bk = [] {
    BatchKernels k{};
    k.per_tile = std::is_same<LBM_ST, StF64>::value ? 0 : 1;
    fill_batch_steps<LBM_ST, 1>(k.step[1]);
    fill_batch_steps<LBM_ST, 2>(k.step[2]);
    fill_batch_steps<LBM_ST, 3>(k.step[3]);
    if (k.per_tile) {
      k.side_fill = (const void *)k_batch_side_fill<LBM_ST>;
      k.side_sync = (const void *)k_batch_side_sync<LBM_ST>;
      k.special[1] = (const void *)k_batch_special_c<LBM_ST, 1>;
      k.special[2] = (const void *)k_batch_special_c<LBM_ST, 2>;
      k.special[3] = (const void *)k_batch_special_c<LBM_ST, 3>;
    } else {
      k.special[1] = (const void *)k_batch_special<LBM_ST, 1>;
      k.special[2] = (const void *)k_batch_special<LBM_ST, 2>;
      k.special[3] = (const void *)k_batch_special<LBM_ST, 3>;
    }
    k.du = (const void *)k_batch_du<LBM_ST>;
    k.advance = (const void *)k_batch_advance;
    k.converge = (const void *)k_batch_converge;
    k.compact_tiles = (const void *)k_batch_compact<int4>;
    return k;
  }();
  return bk;
}

}  // namespace lbm
