// Internal host-side declarations shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/lbm_gb300.h"
#include "lbm_types.h"

namespace lbm {

// Records `msg` as this thread's last error and returns `s`.
lbm_status fail(lbm_status s, const std::string &msg);

// Host result of the per-cell preprocessing (CellIni restated in O(N)).
struct Prep {
  int n = 0, m = 0, pitch = 0;
  long long plane = 0;
  double delta = 0, min_y = 0, max_y = 0;
  double omega = 0, omegaA = 0;
  double stmiv[81] = {};
  std::vector<uint8_t> cls;   // m * pitch
  std::vector<uint32_t> aux;  // m * pitch
  std::vector<BRec> rec;
  uint32_t nsb = 0;           // side-buffer slots (AA)
  long long nfluid = 0;
  std::vector<double> uo_cell; // Uo of every cell (n*m) with a parabolic inlet, CellIni's initial U
};

// Builds the per-node class/record tables of a mesh; for the AA pattern it
// also assigns the side-buffer slots.  Returns LBM_INVALID (with a message) for meshes
// the fused kernel cannot treat exactly.
lbm_status preprocess(const lbm_mesh *mesh, const lbm_params *p, Prep *out);

// Launch tables, one per storage precision, assembled (lbm_kernels_table.cpp)
// from parts compiled separately (lbm_kernels_inst.cu).
struct KernelPart {
  const void *step[3][NVAR];  // [Phase][tile variant] of one collision model
  const void *init[2];        // [0: AB, 1: AA]
  const void *finish[3];
  const void *resid[3];
  const void *reduce;
  int elem_size;
};
typedef void (*StepFn)(StepArgs);
struct KernelSet {
  const void *step[4][3][NVAR];  // [model 1..3][Phase][tile variant]
  const void *init[4][2];    // [model 1..3][0: AB, 1: AA]
  const void *finish[3];     // [layout]
  const void *resid[3];      // [layout]
  const void *reduce;        // k_reduce_partials
  int elem_size;
};
// Launch table of the moment storage (LBM_FP16NEQ, lbm_mom_inst.cu).
struct MomKernels {
  const void *step[4][MOM_NVAR];  // [model 1..3][tile variant: MOM_NPT rows per thread]
  const void *special[4];  // [model] class-3 / class-2 nodes from the compact list
  const void *init[4];     // [model]
  const void *finish;
  const void *resid;
  const void *reduce;
};
const MomKernels &kernels_mom();

const KernelSet &kernels_f64();
const KernelSet &kernels_f32();
const KernelSet &kernels_f16();
const KernelSet &kernels_b16();

}  // namespace lbm

namespace lbm {
// Diagnostics reduction with the library's fixed device scratch array
// (lbm_noalloc.cu); performs no device allocation.
lbm_status check_noalloc(const void *finish, const void *reduce, const StepArgs &a, dim3 grid,
                         cudaStream_t stream, double sums[NSUM]);
}  // namespace lbm
