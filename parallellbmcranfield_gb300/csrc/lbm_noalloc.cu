// lbm_check_noalloc: the full-field diagnostics of lbm_check computed with
// no device allocation at all.
//
// Who needs it: callers that cannot call cudaMalloc at the moment they want
// the diagnostics, e.g. a host that hands all device memory to its own pool
// up front and forbids further driver allocations, or a monitoring loop that
// must not allocate between time steps (an allocation can block on the
// device and can fail under memory pressure).  lbm_check allocates its
// per-block scratch in lbm_create and its du_rel fields on first use; this
// variant writes the per-block partial sums into one fixed array that lives
// in the library image instead.
//
// The array: kNoallocMaxBlocks blocks x NSUM doubles (5 MiB), held by every
// GPU that loads the library until the process exits.  The reduction grid is
// lbm_check's: one block column per 128 grid columns, block rows striding
// over the grid rows so that at most 8192 blocks result when the columns
// allow.  Only a domain wider than 65536 x 128 = 8.4 M grid columns needs
// more blocks than the array holds; it is rejected with LBM_INVALID.
//
// Sharing: every call uses the same array, which keeps the last call's
// contents.  Each call writes every slot it later reads (one slot row per
// block of its own grid), so nothing has to start at zero; but two calls
// whose kernels overlap on the GPU (different streams, or different host
// threads) race on the array.  Serialise such calls.
//
// Set-up: the first call on a device looks up the array's device address
// with cudaGetSymbolAddress (with that device current) and caches it; in host
// code the symbol itself is only a host-side stand-in and must never be
// handed to a kernel.  Make that first call before any stream capture.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "lbm_internal.h"

namespace {

constexpr int kNoallocMaxBlocks = 65536;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_scratch[kNoallocMaxBlocks * lbm::NSUM + 64];

std::mutex g_mu;
double *g_scratch_dev[kMaxDevices] = {};

lbm_status scratch_for_current_device(double **out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return lbm::fail(LBM_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return lbm::fail(LBM_INVALID, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_dev[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return lbm::fail(LBM_CUDA, std::string("cudaGetSymbolAddress(scratch): ") +
                                     cudaGetErrorString(e));
    g_scratch_dev[dev] = (double *)p;
  }
  *out = g_scratch_dev[dev];
  return LBM_OK;
}

}  // namespace

namespace lbm {

lbm_status check_noalloc(const void *finish, const void *reduce, const StepArgs &a, dim3 grid,
                         cudaStream_t stream, double sums[NSUM]) {
  const long long nblk = (long long)grid.x * grid.y;
  if (nblk > kNoallocMaxBlocks)
    return fail(LBM_INVALID, "lbm_check_noalloc: the domain needs " + std::to_string(nblk) +
                                 " reduction blocks; the fixed scratch holds " +
                                 std::to_string(kNoallocMaxBlocks) + " (domains up to " +
                                 std::to_string((long long)kNoallocMaxBlocks * 128) +
                                 " grid columns)");
  double *scratch = nullptr;
  lbm_status s = scratch_for_current_device(&scratch);
  if (s != LBM_OK) return s;
  double *partial = scratch;
  double *total = scratch + (size_t)kNoallocMaxBlocks * NSUM;
  FinishOut o{};
  o.partial = partial;
  StepArgs args = a;
  void *fargs[] = {&args, &o};
  cudaError_t e = cudaLaunchKernel(finish, grid, dim3(128), fargs, 0, stream);
  if (e != cudaSuccess) return fail(LBM_CUDA, std::string("finish launch: ") + cudaGetErrorString(e));
  int nb = (int)nblk;
  void *rargs[] = {&partial, &nb, &total};
  e = cudaLaunchKernel(reduce, dim3(1), dim3(32 * NSUM), rargs, 0, stream);
  if (e != cudaSuccess) return fail(LBM_CUDA, std::string("reduce launch: ") + cudaGetErrorString(e));
  e = cudaMemcpyAsync(sums, total, NSUM * sizeof(double), cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return fail(LBM_CUDA, std::string("read-back: ") + cudaGetErrorString(e));
  return LBM_OK;
}

}  // namespace lbm
