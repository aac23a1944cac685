// C ABI of the D2Q9 step library (include/lbm_gb300.h): context lifetime,
// state upload, the stepping loop and field / diagnostic read-back.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "lbm_internal.h"

namespace lbm {
namespace {
thread_local std::string g_err;
}
lbm_status fail(lbm_status s, const std::string &msg) {
  g_err = msg;
  return s;
}
}  // namespace lbm

using lbm::fail;

#define LBM_CK(call)                                                                     \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return fail(e_ == cudaErrorMemoryAllocation ? LBM_NOMEM : LBM_CUDA,                \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                   \
  } while (0)

struct lbm_ctx {
  lbm::Prep P;
  lbm_params p{};
  const lbm::KernelSet *ks = nullptr;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  void *pop[2] = {nullptr, nullptr};
  double *sb[2] = {nullptr, nullptr};
  uint8_t *d_cls = nullptr;
  uint32_t *d_aux = nullptr;
  lbm::BRec *d_rec = nullptr;
  double *d_rho0 = nullptr, *d_u0 = nullptr, *d_v0 = nullptr;
  float *d_uprev = nullptr, *d_vprev = nullptr;
  bool have_prev = false;
  int64_t prev_iter = 0;     // iteration of the previous lbm_check (du_rel interval)
  double *d_partial = nullptr, *d_sums = nullptr;
  double *d_hist = nullptr;
  int hist_cap = 0;
  int nblk = 0;              // blocks of a node-grid launch
  int64_t iter = 0;          // completed iterations
  int64_t g = 0;             // index of the METAF generation held on the device
  bool have_state = false;
  int64_t dev_bytes = 0;
  int variant = 0;           // tile variant of the fused step
  int pf_blocks[lbm::NVAR] = {};  // per variant: resident blocks of one wave (-1: not known yet)
  void *pop_raw[2] = {nullptr, nullptr};  // allocations behind pop[] (guard elements in front)
  int *d_err = nullptr;      // [0] error word of bounded waits, [1] NaN flag of the step
  // moment storage (LBM_FP16NEQ)
  const lbm::MomKernels *mk = nullptr;
  float *ss[2] = {nullptr, nullptr};  // FP32 side arrays of the class-3 nodes (A-B parities)
  uint32_t *d_mlist = nullptr;        // class-3 and class-2 nodes
  int mlist_n = 0;
  std::vector<uint32_t> mlist_host;
  lbm::StepArgs base{};
};

namespace {

constexpr int kBlock = 128;
constexpr unsigned kFinishBlocks = 8192;  // partial rows of the diagnostics reduction

template <class T>
lbm_status dalloc(lbm_ctx *c, T **p, size_t count) {
  size_t bytes = count * sizeof(T);
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc((void **)p, bytes);
  if (e != cudaSuccess)
    return fail(LBM_NOMEM, "cudaMalloc of " + std::to_string(bytes) + " bytes: " +
                               cudaGetErrorString(e));
  c->dev_bytes += (int64_t)bytes;
  return LBM_OK;
}

void release(lbm_ctx *c) {
  void *ptrs[] = {c->pop_raw[0], c->pop_raw[1], c->sb[0], c->sb[1], c->d_cls, c->d_err,
                  c->d_aux,  c->d_rec,  c->d_rho0,   c->d_u0,       c->d_v0,
                  c->d_uprev, c->d_vprev, c->d_partial, c->d_sums, c->d_hist,
                  c->ss[0], c->ss[1], c->d_mlist};
  for (void *q : ptrs)
    if (q) cudaFree(q);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
}

dim3 node_grid(const lbm_ctx *c) {
  return dim3((unsigned)((c->P.n + kBlock - 1) / kBlock), (unsigned)c->P.m);
}

int layout_of(const lbm_ctx *c) {
  if (c->p.pattern == LBM_AB) return lbm::PH_AB;
  return (c->g & 1) ? lbm::PH_AA_B : lbm::PH_AA_A;
}

// Arguments for a launch that reads generation g (and writes g+1).
lbm::StepArgs args_now(const lbm_ctx *c) {
  lbm::StepArgs a = c->base;
  a.gen = (unsigned)(c->g + 1);
  if (c->p.pattern == LBM_AB) {
    a.src = c->pop[c->g & 1];
    a.dst = c->pop[(c->g + 1) & 1];
    a.ss_src = c->ss[c->g & 1];
    a.ss_dst = c->ss[(c->g + 1) & 1];
  } else {
    a.src = a.dst = c->pop[0];
    a.sb_src = c->sb[c->g & 1];
    a.sb_dst = c->sb[(c->g + 1) & 1];
  }
  return a;
}

lbm_status launch(const void *fn, dim3 grid, dim3 block, void **args, cudaStream_t s) {
  cudaError_t e = cudaLaunchKernel(fn, grid, block, args, 0, s);
  if (e != cudaSuccess) return fail(LBM_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  return LBM_OK;
}

// Launch shape of tile variant `var` (grid, block, dynamic shared memory).
// Returns false when the variant cannot run for this storage (TMA ring too
// large for the shared-memory budget).
bool step_config(lbm_ctx *c, int var, dim3 *grid, dim3 *block, size_t *smem) {
  const lbm::TileVariant &V = lbm::VARS[var];
  *smem = 0;
  if (V.kind == 3 && c->ks->elem_size != 2) {  // runs as the scalar tile (bx 128)
    *grid = dim3((unsigned)((c->P.n + 127) / 128), (unsigned)((c->P.m + V.npt - 1) / V.npt));
    *block = dim3(128);
    return true;
  }
  if (V.kind == 0 || V.kind == 1 || V.kind == 3) {
    const int span = V.kind == 0 ? c->P.n : c->P.pitch;  // vector tiles cover whole padded rows
    *grid = dim3((unsigned)((span + V.bx * V.v - 1) / (V.bx * V.v)),
                 (unsigned)((c->P.m + V.npt - 1) / V.npt));
    *block = dim3(V.bx);
    // L2 prefetch distance of the paired kernel: a quarter of a wave of resident
    // blocks (measured at 16384^2: 1/4-1/3 wave 1.79 ms/step, 1 wave 1.82, 2 waves 2.08,
    // none 2.02), looked up once per variant
    if (V.kind == 3 && c->pf_blocks[var] == 0) {
      const void *fn = c->ks->step[c->p.collision_model][layout_of(c)][var];
      int per_sm = 0, sms = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, V.bx, 0) != cudaSuccess)
        per_sm = 0;
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->p.device);
      c->pf_blocks[var] = per_sm > 0 ? std::max(1, per_sm * sms / 4) : -1;
    }
    return true;
  }
  // stage layout of k_step_tma: 9 population planes of ty rows of
  // tx + 2 granules, then ty rows of tx class bytes, rounded to 128 bytes
  const int es = c->ks->elem_size;
  const int W = V.tx + 2 * (16 / es);
  const size_t stage = ((size_t)9 * V.ty * W * es + (size_t)V.ty * V.tx + 127) / 128 * 128;
  // ring depth: up to 4 stages within ~75 KB so that 3 blocks share an SM;
  // a larger stage gets 2 stages within the 200 KB budget
  int S = (int)((75 * 1024 - 128) / stage);
  if (S > lbm::TMA_MAX_STAGES) S = lbm::TMA_MAX_STAGES;
  if (S < 2) S = (128 + 2 * stage <= (size_t)lbm::TMA_MAX_SMEM) ? 2 : 0;
  if (S < 2) return false;
  *smem = 128 + (size_t)S * stage;
  const int threads = V.tx * V.ty / V.rpt;
  const void *fn = c->ks->step[c->p.collision_model][layout_of(c)][var];
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)*smem) !=
      cudaSuccess)
    return false;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, *smem) != cudaSuccess ||
      per_sm < 1)
    return false;
  int dev = c->p.device, sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int tiles_x = (c->P.pitch + V.tx - 1) / V.tx;
  const int tiles_y = (c->P.m - 2 + V.ty - 1) / V.ty;
  long long tiles = (long long)tiles_x * tiles_y;
  long long blocks = (long long)sms * per_sm;
  if (blocks > tiles) blocks = tiles;
  *grid = dim3((unsigned)(blocks > 0 ? blocks : 1));
  *block = dim3(threads);
  c->base.tma_stages = S;
  c->base.tma_tiles_x = tiles_x;
  c->base.tma_tiles_y = tiles_y;
  return true;
}

// Moment storage: the bulk kernel (blocks of 4 warps x 60 columns, NPT rows
// per thread) and the special-node kernel over the compact list, both
// reading the same generation (they write disjoint nodes).
lbm_status launch_step_mom(lbm_ctx *c) {
  const int npt = lbm::MOM_NPT[c->variant];
  lbm::StepArgs a = args_now(c);
  void *args[] = {&a};
  const dim3 grid((unsigned)((c->P.n + 239) / 240), (unsigned)((c->P.m + npt - 1) / npt));
  cudaError_t e = cudaLaunchKernel(c->mk->step[c->p.collision_model][c->variant], grid, dim3(128),
                                   args, 0, c->stream);
  if (e == cudaSuccess && c->mlist_n > 0)
    e = cudaLaunchKernel(c->mk->special[c->p.collision_model],
                         dim3((unsigned)((c->mlist_n + 127) / 128)), dim3(128), args, 0, c->stream);
  if (e != cudaSuccess) return fail(LBM_CUDA, std::string("step launch: ") + cudaGetErrorString(e));
  c->g++;
  return LBM_OK;
}

lbm_status launch_step(lbm_ctx *c) {
  if (c->mk) return launch_step_mom(c);
  const int var = c->variant;
  dim3 grid, block;
  size_t smem;
  if (!step_config(c, var, &grid, &block, &smem))
    return fail(LBM_INVALID, "tile variant " + std::to_string(var + 1) + " cannot run here");
  lbm::StepArgs a = args_now(c);
  a.pf_blocks = c->pf_blocks[var] > 0 ? c->pf_blocks[var] : 0;
  void *args[] = {&a};
  const void *fn = c->ks->step[c->p.collision_model][layout_of(c)][var];
  cudaError_t e = cudaLaunchKernel(fn, grid, block, args, smem, c->stream);
  if (e != cudaSuccess) return fail(LBM_CUDA, std::string("step launch: ") + cudaGetErrorString(e));
  c->g++;
  return LBM_OK;
}

// A bounded device wait that gave up sets the error word; report and clear
// it.  A reduced-precision step that produced a NaN or infinity sets the NaN
// flag, which stays set until the next lbm_set_state (the state is lost).
lbm_status check_device_error(lbm_ctx *c) {
  int h[2] = {0, 0};
  LBM_CK(cudaMemcpyAsync(h, c->d_err, sizeof h, cudaMemcpyDeviceToHost, c->stream));
  LBM_CK(cudaStreamSynchronize(c->stream));
  if (h[0] != 0) {
    cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream);
    return fail(LBM_TIMEOUT, "a bounded device wait (TMA stage barrier) gave up");
  }
  if (h[1] == 2)
    return fail(LBM_DIVERGED,
                "moment storage out of range (|rho - rho0| >= 0.5 rho0 or |j| >= 0.25 rho0)");
  if (h[1] != 0) return fail(LBM_DIVERGED, "DIVERGENCE! (NaN or infinity in the populations)");
  return LBM_OK;
}

lbm_status launch_resid(lbm_ctx *c, double *out) {
  lbm::StepArgs a = args_now(c);
  void *args[] = {&a, &out};
  return launch(c->mk ? c->mk->resid : c->ks->resid[layout_of(c)], dim3(1), dim3(256), args,
                c->stream);
}

// Finish and reduction kernels of the context's storage.
const void *finish_fn(const lbm_ctx *c) { return c->mk ? c->mk->finish : c->ks->finish[layout_of(c)]; }
const void *reduce_fn(const lbm_ctx *c) { return c->mk ? c->mk->reduce : c->ks->reduce; }

// Grid of the finish kernel: one block column per 128 x positions, block rows
// striding over the grid so that at most kFinishBlocks partial rows result.
dim3 finish_grid(const lbm_ctx *c) {
  dim3 g = node_grid(c);
  unsigned rows = kFinishBlocks / g.x;
  if (rows < 1) rows = 1;
  if (rows < g.y) g.y = rows;
  return g;
}

lbm_status launch_finish(lbm_ctx *c, lbm::FinishOut &o) {
  lbm::StepArgs a = args_now(c);
  o.partial = c->d_partial;
  void *args[] = {&a, &o};
  const dim3 g = finish_grid(c);
  int nb = (int)(g.x * g.y);
  lbm_status s = launch(finish_fn(c), g, dim3(kBlock), args, c->stream);
  if (s != LBM_OK) return s;
  void *rargs[] = {&c->d_partial, &nb, &c->d_sums};
  return launch(reduce_fn(c), dim3(1), dim3(32 * lbm::NSUM), rargs, c->stream);
}

// Host copy of a per-cell default field.
std::vector<double> default_field(const lbm_ctx *c, int which) {
  const size_t N = (size_t)c->P.n * c->P.m;
  if (which == 0) return std::vector<double>(N, (double)c->p.rho_ini);
  if (which == 2) return std::vector<double>(N, 0.0);
  if (!c->P.uo_cell.empty()) return c->P.uo_cell;
  return std::vector<double>(N, (double)c->p.uavg);
}

lbm_status set_state_impl(lbm_ctx *c, const double *f, const double *rho, const double *u,
                          const double *v, bool zero_f) {
  const size_t N = (size_t)c->P.n * c->P.m;
  const double *src[3] = {rho, u, v};
  double *dst[3] = {c->d_rho0, c->d_u0, c->d_v0};
  for (int i = 0; i < 3; i++) {
    if (src[i]) {
      LBM_CK(cudaMemcpyAsync(dst[i], src[i], N * sizeof(double), cudaMemcpyHostToDevice,
                             c->stream));
    } else {
      std::vector<double> h = default_field(c, i);
      LBM_CK(cudaMemcpyAsync(dst[i], h.data(), N * sizeof(double), cudaMemcpyHostToDevice,
                             c->stream));
      LBM_CK(cudaStreamSynchronize(c->stream));
    }
  }
  double *d_f = nullptr;
  if (f || zero_f) {
    LBM_CK(cudaMallocAsync((void **)&d_f, N * 9 * sizeof(double), c->stream));
    if (f)
      LBM_CK(cudaMemcpyAsync(d_f, f, N * 9 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    else
      LBM_CK(cudaMemsetAsync(d_f, 0, N * 9 * sizeof(double), c->stream));
  }
  LBM_CK(cudaMemsetAsync(c->d_err + 1, 0, sizeof(int), c->stream));  // the first collision may set it
  c->g = 0;
  lbm::StepArgs a = args_now(c);
  a.dst = c->pop[0];
  a.sb_dst = c->sb[0];
  a.ss_dst = c->ss[0];
  a.gen = 0;
  void *args[] = {&a, &d_f, &c->d_rho0, &c->d_u0, &c->d_v0};
  int which = c->p.pattern == LBM_AB ? 0 : 1;
  lbm_status s = launch(c->mk ? c->mk->init[c->p.collision_model]
                              : c->ks->init[c->p.collision_model][which],
                        node_grid(c), dim3(kBlock), args, c->stream);
  if (d_f) cudaFreeAsync(d_f, c->stream);
  if (s != LBM_OK) return s;
  LBM_CK(cudaStreamSynchronize(c->stream));
  LBM_CK(cudaGetLastError());
  c->iter = 0;
  c->have_state = true;
  c->have_prev = false;
  return LBM_OK;
}

}  // namespace

extern "C" {

const char *lbm_status_string(lbm_status s) {
  switch (s) {
    case LBM_OK: return "ok";
    case LBM_DIVERGED: return "diverged";
    case LBM_IO: return "file i/o error";
    case LBM_CUDA: return "cuda error";
    case LBM_TIMEOUT: return "device wait timed out";
    case LBM_INVALID: return "invalid argument";
    case LBM_NOMEM: return "out of memory";
  }
  return "unknown status";
}

const char *lbm_last_error(void) { return lbm::g_err.c_str(); }

lbm_status lbm_create(const lbm_mesh *mesh, const lbm_params *params, lbm_ctx **out) {
  if (!out || !params) return fail(LBM_INVALID, "null argument");
  *out = nullptr;
  if (params->precision < LBM_FP64 || params->precision > LBM_FP16NEQ)
    return fail(LBM_INVALID, "unknown precision");
  if (params->pattern != LBM_AB && params->pattern != LBM_AA)
    return fail(LBM_INVALID, "unknown pattern");
  const bool mom = params->precision == LBM_FP16NEQ;
  if (mom && params->pattern != LBM_AB)
    return fail(LBM_INVALID, "moment storage (LBM_FP16NEQ) runs the A-B pattern only");
  if (mom && params->tile_variant > lbm::MOM_NVAR)
    return fail(LBM_INVALID, "tile_variant must be 0 (default/tuned) or 1.." +
                                 std::to_string(lbm::MOM_NVAR) + " for moment storage");
  lbm_ctx *c = new lbm_ctx();
  c->p = *params;
  lbm_status s = lbm::preprocess(mesh, params, &c->P);
  if (s != LBM_OK) {
    delete c;
    return s;
  }
  if (params->tile_variant < 0 || params->tile_variant > lbm::NVAR) {
    delete c;
    return fail(LBM_INVALID, "tile_variant must be 0 (default/tuned) or 1.." + std::to_string(lbm::NVAR));
  }
  c->variant = params->tile_variant > 0 ? params->tile_variant - 1 : 0;
  if (mom && (long long)c->P.pitch * 21 > INT32_MAX) {
    delete c;
    return fail(LBM_INVALID, "moment storage: rows of more than 102 M nodes are not supported");
  }
  if (c->P.m > 65535) {
    delete c;
    return fail(LBM_INVALID, "grid taller than 65535 rows");
  }
  switch (params->precision) {
    case LBM_FP64: c->ks = &lbm::kernels_f64(); break;
    case LBM_FP32: c->ks = &lbm::kernels_f32(); break;
    case LBM_FP16DEV: c->ks = &lbm::kernels_f16(); break;
    case LBM_FP16NEQ: c->mk = &lbm::kernels_mom(); break;
    default: c->ks = &lbm::kernels_b16(); break;
  }
  if (mom) {
    // fluid nodes next to a class-3 node become class 2: the special-node
    // kernel updates both, so the bulk kernel never reads the side array
    lbm::Prep &Pm = c->P;
    std::vector<uint32_t> list;
    for (const lbm::BRec &r : Pm.rec) {
      for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++) {
          const long long z = (long long)r.node + dx + (long long)dy * Pm.pitch;
          if (z >= 0 && z < Pm.plane && Pm.cls[z] == lbm::CLS_BULK) Pm.cls[z] = lbm::CLS_BULK_REC;
        }
    }
    for (long long z = 0; z < Pm.plane; z++)
      if (Pm.cls[z] == lbm::CLS_BULK_REC || Pm.cls[z] == lbm::CLS_SPECIAL) list.push_back((uint32_t)z);
    c->mlist_n = (int)list.size();
    c->mlist_host.swap(list);
  }
  auto bail = [&](lbm_status st) {
    release(c);
    delete c;
    return st;
  };
  if (cudaSetDevice(params->device) != cudaSuccess)
    return bail(fail(LBM_CUDA, "cudaSetDevice failed (no GPU?)"));
  if (params->stream) {
    c->stream = (cudaStream_t)params->stream;
  } else {
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
      return bail(fail(LBM_CUDA, "cudaStreamCreate failed"));
    c->own_stream = true;
  }
  const lbm::Prep &P = c->P;
  const size_t N = (size_t)P.n * P.m;
  // guard elements before the first and after the last plane: the 16-byte
  // halo granules of the TMA row copies and the edge reads of the vector
  // tiles reach up to 16 bytes (plus one row for the last tile) outside
  const size_t guard = 1024;
  // moment storage: 21 bytes per node (nine 16-bit planes, three byte planes)
  const size_t es = mom ? 1 : (size_t)c->ks->elem_size;
  const size_t pop_elems =
      mom ? (size_t)P.plane * 21 + 2 * guard : (size_t)P.plane * 9 + 2 * guard + (size_t)P.pitch;
  const int npop = params->pattern == LBM_AB ? 2 : 1;
  for (int i = 0; i < npop; i++) {
    if ((s = dalloc(c, (char **)&c->pop_raw[i], pop_elems * es)) != LBM_OK)
      return bail(s);
    if (cudaMemset(c->pop_raw[i], 0, pop_elems * es) != cudaSuccess)
      return bail(fail(LBM_CUDA, "cudaMemset failed"));
    c->pop[i] = (char *)c->pop_raw[i] + guard * es;
  }
  if (mom) {
    for (int i = 0; i < 2; i++) {
      if ((s = dalloc(c, &c->ss[i], P.rec.size() * 9)) != LBM_OK) return bail(s);
      if (cudaMemset(c->ss[i], 0, std::max<size_t>(16, P.rec.size() * 9 * 4)) != cudaSuccess)
        return bail(fail(LBM_CUDA, "cudaMemset failed"));
    }
    if ((s = dalloc(c, &c->d_mlist, c->mlist_host.size())) != LBM_OK) return bail(s);
    if (!c->mlist_host.empty() &&
        cudaMemcpy(c->d_mlist, c->mlist_host.data(), c->mlist_host.size() * 4,
                   cudaMemcpyHostToDevice) != cudaSuccess)
      return bail(fail(LBM_CUDA, "upload of the special-node list failed"));
  }
  if ((s = dalloc(c, &c->d_err, 2)) != LBM_OK) return bail(s);
  if (cudaMemset(c->d_err, 0, 2 * sizeof(int)) != cudaSuccess)
    return bail(fail(LBM_CUDA, "cudaMemset failed"));
  if (params->pattern == LBM_AA)
    for (int i = 0; i < 2; i++)
      if ((s = dalloc(c, &c->sb[i], (size_t)P.nsb * 9)) != LBM_OK) return bail(s);
  if ((s = dalloc(c, &c->d_cls, P.cls.size())) != LBM_OK) return bail(s);
  if ((s = dalloc(c, &c->d_aux, P.aux.size())) != LBM_OK) return bail(s);
  if ((s = dalloc(c, &c->d_rec, P.rec.size())) != LBM_OK) return bail(s);
  if ((s = dalloc(c, &c->d_rho0, N)) != LBM_OK) return bail(s);
  if ((s = dalloc(c, &c->d_u0, N)) != LBM_OK) return bail(s);
  if ((s = dalloc(c, &c->d_v0, N)) != LBM_OK) return bail(s);
  c->nblk = (int)(finish_grid(c).x * finish_grid(c).y);
  if ((s = dalloc(c, &c->d_partial, (size_t)c->nblk * lbm::NSUM)) != LBM_OK) return bail(s);
  if ((s = dalloc(c, &c->d_sums, lbm::NSUM)) != LBM_OK) return bail(s);
  if (cudaMemcpy(c->d_cls, P.cls.data(), P.cls.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(c->d_aux, P.aux.data(), P.aux.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      (!P.rec.empty() && cudaMemcpy(c->d_rec, P.rec.data(), P.rec.size() * sizeof(lbm::BRec),
                                    cudaMemcpyHostToDevice) != cudaSuccess))
    return bail(fail(LBM_CUDA, "upload of node tables failed"));
  lbm::StepArgs &a = c->base;
  std::memset(&a, 0, sizeof a);
  a.n = P.n;
  a.m = P.m;
  a.pitch = P.pitch;
  a.model = params->collision_model;
  a.curved = params->curved_boundaries;
  a.outlet = params->outlet_profile;
  a.plane = P.plane;
  a.cls = c->d_cls;
  a.aux = c->d_aux;
  a.rec = c->d_rec;
  a.omega = P.omega;
  a.omegaA = P.omegaA;
  a.rho_out = params->rho_out;
  a.rho0 = params->rho_ini;
  const double w[9] = {4. / 9., 1. / 9., 1. / 9., 1. / 9., 1. / 9., 1. / 36., 1. / 36., 1. / 36., 1. / 36.};
  for (int k = 0; k < 9; k++) {
    // 16-bit storage keeps (f_k - w_k rho0) / (w_k rho0) * S: S = 4096 keeps
    // FP16 normal down to relative deviations of 1.5e-8; BF16 has FP32 range.
    double S = params->precision == LBM_FP16DEV ? 4096.0 : 1.0;
    double sc = S / (w[k] * (params->rho_ini > 0 ? params->rho_ini : 1.0));
    a.scale[k] = (float)sc;
    a.inv_scale[k] = (float)(1.0 / sc);
  }
  std::memcpy(a.stmiv, P.stmiv, sizeof a.stmiv);
  a.err = c->d_err;
  // FP64 is the parity mode: its divergence report stays the reference's
  // (a NaN residual line); the other storages flag any NaN in the step
  a.nanflag = params->precision == LBM_FP64 ? nullptr : c->d_err + 1;
  if (mom) {
    // 24-bit fixed point: rho - rho0 within +-0.5 rho0, j within +-0.25 rho0
    const double r0 = params->rho_ini > 0 ? params->rho_ini : 1.0;
    const double qmax = (double)((1 << 23) - 1);
    a.fx_rho = (float)(0.5 * r0 / qmax);
    a.fx_irho = (float)(qmax / (0.5 * r0));
    a.fx_j = (float)(0.25 * r0 / qmax);
    a.fx_ij = (float)(qmax / (0.25 * r0));
    a.fx_irho0 = (float)(1.0 / r0);
    a.neq_s = lbm::MOM_NEQ_S;
    a.neq_is = 1.f / lbm::MOM_NEQ_S;
    a.f_i4rho0 = (float)(0.25 / r0);
    const double hr = 0.5 * r0 / qmax, hj = 0.25 * r0 / qmax, S = lbm::MOM_NEQ_S;
    a.fx_enc[0] = (float)(64.0 / hr);
    a.fx_enc[1] = (float)(32.0 / hj);
    // two codes of margin: the rounding of v / step and the dither stay inside +-qmax
    a.fx_rlim = (float)((qmax - 2.0) * hr);
    a.fx_jlim = (float)((qmax - 2.0) * hj);
    a.enc_c[0] = (float)(2.0 * S * hr);
    a.enc_c[1] = (float)(-3.0 * S * hj * hj);
    a.enc_c[2] = (float)(-S * hr);
    a.enc_c[3] = (float)(3.0 * S * hj * hj);
    a.enc_c[4] = (float)(S * hj);
    a.enc_c[5] = (float)(-S * hj * hj / r0);
    // relaxation rates of the moment collision (collide_mom): MRT 1.4, 1.2,
    // omega (serial/CellFunctions.c:401-438); TRT omega, omegaA, omega; BGK omega
    const int model = params->collision_model;
    const double s12 = model == 3 ? 1.4 : P.omega;
    const double s46 = model == 3 ? 1.2 : (model == 2 ? P.omegaA : P.omega);
    const double es[9] = {3.0 * S * s12, -2.0 * S * s12, S * s12, -3.0 * S * s12, S * (1.0 - s12),
                          -S * s46, S * (1.0 - s46), S * P.omega, S * (1.0 - P.omega)};
    for (int k = 0; k < 9; k++) a.enc_s[k] = (float)es[k];
    a.f_rho0 = (float)a.rho0;
    a.f_om = (float)a.omega;
    a.f_omA = (float)a.omegaA;
    a.mlist = c->d_mlist;
    a.mlist_n = c->mlist_n;
  }
  *out = c;
  return LBM_OK;
}

void lbm_destroy(lbm_ctx *ctx) {
  if (!ctx) return;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  release(ctx);
  delete ctx;
}

lbm_status lbm_get_dims(const lbm_ctx *ctx, int32_t *n, int32_t *m) {
  if (!ctx || !n || !m) return fail(LBM_INVALID, "null argument");
  *n = ctx->P.n;
  *m = ctx->P.m;
  return LBM_OK;
}

lbm_status lbm_get_info(const lbm_ctx *ctx, int64_t *iteration, int64_t *device_bytes,
                        int32_t *bytes_per_node_step) {
  if (!ctx) return fail(LBM_INVALID, "null argument");
  if (iteration) *iteration = ctx->iter;
  if (device_bytes) *device_bytes = ctx->dev_bytes;
  if (bytes_per_node_step) *bytes_per_node_step = ctx->mk ? 42 : 18 * ctx->ks->elem_size;
  return LBM_OK;
}

lbm_status lbm_set_state(lbm_ctx *ctx, const double *f, const double *rho, const double *u,
                         const double *v) {
  if (!ctx) return fail(LBM_INVALID, "null argument");
  LBM_CK(cudaSetDevice(ctx->p.device));
  return set_state_impl(ctx, f, rho, u, v, false);
}

lbm_status lbm_step(lbm_ctx *ctx, int32_t nsteps, int32_t check_every, double *residuals) {
  if (!ctx || nsteps < 0) return fail(LBM_INVALID, "bad argument");
  LBM_CK(cudaSetDevice(ctx->p.device));
  lbm_status s;
  if (!ctx->have_state) {
    // the reference's own start: F = 0, Rho = rho_ini, U = Uo, V = 0
    // (serial/CellFunctions.c:147-150, 252-267 and the calloc of serial/Iterate.c:193)
    if ((s = set_state_impl(ctx, nullptr, nullptr, nullptr, nullptr, true)) != LBM_OK) return s;
  }
  const int rows = check_every > 0 ? nsteps / check_every : 0;
  if (rows > ctx->hist_cap) {
    if (ctx->d_hist) cudaFree(ctx->d_hist);
    ctx->d_hist = nullptr;
    ctx->hist_cap = 0;
    if ((s = dalloc(ctx, &ctx->d_hist, (size_t)rows * 4)) != LBM_OK) return s;
    ctx->hist_cap = rows;
  }
  int row = 0;
  for (int st = 1; st <= nsteps; st++) {
    if (ctx->iter > 0)
      if ((s = launch_step(ctx)) != LBM_OK) return s;
    ctx->iter++;
    if (check_every > 0 && st % check_every == 0) {
      if ((s = launch_resid(ctx, ctx->d_hist + (size_t)row * 4)) != LBM_OK) return s;
      row++;
    }
  }
  if (rows > 0 && residuals)
    LBM_CK(cudaMemcpyAsync(residuals, ctx->d_hist, (size_t)rows * 4 * sizeof(double),
                           cudaMemcpyDeviceToHost, ctx->stream));
  LBM_CK(cudaStreamSynchronize(ctx->stream));
  LBM_CK(cudaGetLastError());
  if ((s = check_device_error(ctx)) != LBM_OK) return s;
  if (residuals)
    for (int r = 0; r < rows; r++)
      if (residuals[4 * r] != residuals[4 * r])
        return fail(LBM_DIVERGED, "DIVERGENCE! (NaN residual)");
  return LBM_OK;
}

lbm_status lbm_get_fields(lbm_ctx *ctx, double *rho, double *u, double *v, double *f,
                          double *metaf) {
  if (!ctx) return fail(LBM_INVALID, "null argument");
  LBM_CK(cudaSetDevice(ctx->p.device));
  const size_t N = (size_t)ctx->P.n * ctx->P.m;
  if (!ctx->have_state || ctx->iter == 0) {
    if (f || metaf) return fail(LBM_INVALID, "F/METAF exist only after the first iteration");
    if (!ctx->have_state) {
      double *dst[3] = {rho, u, v};
      for (int i = 0; i < 3; i++)
        if (dst[i]) {
          std::vector<double> h = default_field(ctx, i);
          std::memcpy(dst[i], h.data(), N * sizeof(double));
        }
      return LBM_OK;
    }
    if (rho) LBM_CK(cudaMemcpy(rho, ctx->d_rho0, N * 8, cudaMemcpyDeviceToHost));
    if (u) LBM_CK(cudaMemcpy(u, ctx->d_u0, N * 8, cudaMemcpyDeviceToHost));
    if (v) LBM_CK(cudaMemcpy(v, ctx->d_v0, N * 8, cudaMemcpyDeviceToHost));
    return LBM_OK;
  }
  lbm::FinishOut o;
  std::memset(&o, 0, sizeof o);
  o.rho_solid = ctx->d_rho0;
  o.u_solid = ctx->d_u0;
  o.v_solid = ctx->d_v0;
  double *host[5] = {rho, u, v, f, metaf};
  double **dev[5] = {&o.rho, &o.u, &o.v, &o.f, &o.metaf};
  size_t cnt[5] = {N, N, N, 9 * N, 9 * N};
  lbm_status s = LBM_OK;
  // rho, u, v go through the set_state field buffers, in place: the finish
  // kernel reads a solid cell's reported value and writes the same element,
  // and the fluid cells' entries are not read again before the next
  // lbm_set_state refills them.  F and METAF need device temporaries.
  double *fields[3] = {ctx->d_rho0, ctx->d_u0, ctx->d_v0};
  for (int i = 0; i < 5 && s == LBM_OK; i++) {
    if (!host[i]) continue;
    if (i < 3)
      *dev[i] = fields[i];
    else if (cudaMallocAsync((void **)dev[i], cnt[i] * 8, ctx->stream) != cudaSuccess)
      s = fail(LBM_NOMEM, "device temporary for field read-back");
  }
  if (s == LBM_OK) s = launch_finish(ctx, o);
  for (int i = 0; i < 5 && s == LBM_OK; i++)
    if (host[i] && cudaMemcpyAsync(host[i], *dev[i], cnt[i] * 8, cudaMemcpyDeviceToHost,
                                   ctx->stream) != cudaSuccess)
      s = fail(LBM_CUDA, "field read-back failed");
  for (int i = 3; i < 5; i++)
    if (*dev[i]) cudaFreeAsync(*dev[i], ctx->stream);
  LBM_CK(cudaStreamSynchronize(ctx->stream));
  return s;
}

lbm_status lbm_check(lbm_ctx *ctx, lbm_diagnostics *out) {
  if (!ctx || !out) return fail(LBM_INVALID, "null argument");
  if (!ctx->have_state || ctx->iter == 0)
    return fail(LBM_INVALID, "no completed iteration to check");
  LBM_CK(cudaSetDevice(ctx->p.device));
  const size_t N = (size_t)ctx->P.n * ctx->P.m;
  lbm_status s;
  if (!ctx->d_uprev) {
    if ((s = dalloc(ctx, &ctx->d_uprev, N)) != LBM_OK) return s;
    if ((s = dalloc(ctx, &ctx->d_vprev, N)) != LBM_OK) return s;
  }
  lbm::FinishOut o;
  std::memset(&o, 0, sizeof o);
  o.uprev = ctx->d_uprev;
  o.vprev = ctx->d_vprev;
  if ((s = launch_finish(ctx, o)) != LBM_OK) return s;
  double h[lbm::NSUM];
  LBM_CK(cudaMemcpyAsync(h, ctx->d_sums, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
  LBM_CK(cudaStreamSynchronize(ctx->stream));
  out->iteration = ctx->iter;
  out->l2_full = std::sqrt(h[lbm::S_L2]);
  out->mass = h[lbm::S_MASS];
  out->momentum[0] = h[lbm::S_MX];
  out->momentum[1] = h[lbm::S_MY];
  out->force[0] = h[lbm::S_FX];
  out->force[1] = h[lbm::S_FY];
  out->max_speed = h[lbm::S_VMAX];
  const int64_t span = std::max<int64_t>(1, ctx->iter - ctx->prev_iter);
  out->du_rel = ctx->have_prev ? std::sqrt(h[lbm::S_DU] / h[lbm::S_UU]) / (double)span : INFINITY;
  ctx->have_prev = true;
  ctx->prev_iter = ctx->iter;
  if (h[lbm::S_NAN] > 0 || h[lbm::S_MASS] != h[lbm::S_MASS])
    return fail(LBM_DIVERGED, "NaN in the macroscopic fields");
  return LBM_OK;
}

}  // extern "C"

// Allocation-free variant of lbm_check (see lbm_noalloc.cu for the fixed
// scratch array it uses and its limits).
extern "C" lbm_status lbm_check_noalloc(lbm_ctx *ctx, lbm_diagnostics *out) {
  if (!ctx || !out) return fail(LBM_INVALID, "null argument");
  if (!ctx->have_state || ctx->iter == 0)
    return fail(LBM_INVALID, "no completed iteration to check");
  LBM_CK(cudaSetDevice(ctx->p.device));
  double h[lbm::NSUM];
  // the launch shape of lbm_check (block rows capped at kFinishBlocks
  // partial rows), so both reduce the same partial sums in the same order
  lbm_status s = lbm::check_noalloc(finish_fn(ctx), reduce_fn(ctx), args_now(ctx),
                                    finish_grid(ctx), ctx->stream, h);
  if (s != LBM_OK) return s;
  out->iteration = ctx->iter;
  out->l2_full = std::sqrt(h[lbm::S_L2]);
  out->mass = h[lbm::S_MASS];
  out->momentum[0] = h[lbm::S_MX];
  out->momentum[1] = h[lbm::S_MY];
  out->force[0] = h[lbm::S_FX];
  out->force[1] = h[lbm::S_FY];
  out->max_speed = h[lbm::S_VMAX];
  out->du_rel = NAN;  // needs per-cell reference fields, which this variant cannot allocate
  if (h[lbm::S_NAN] > 0 || h[lbm::S_MASS] != h[lbm::S_MASS])
    return fail(LBM_DIVERGED, "NaN in the macroscopic fields");
  return LBM_OK;
}

// ------------------------------------------------------------------ autotuner

namespace {

std::string tune_key(const lbm_ctx *c) {
  cudaDeviceProp prop;
  std::string gpu = "gpu";
  if (cudaGetDeviceProperties(&prop, c->p.device) == cudaSuccess) gpu = prop.name;
  const char *prec[] = {"fp64", "fp32", "fp16dev", "bf16dev", "fp16neq"};
  return gpu + "|" + prec[c->p.precision] + "|" + (c->p.pattern == LBM_AB ? "ab" : "aa") + "|m" +
         std::to_string(c->p.collision_model) + "|" + std::to_string(c->P.n) + "x" +
         std::to_string(c->P.m);
}

// Cache lines: {"key": "<key>", "variant": <v>, "ms": [..]} -- last line for a key wins.
int cache_lookup(const char *path, const std::string &key, int nvar) {
  if (!path) return -1;
  FILE *f = std::fopen(path, "r");
  if (!f) return -1;
  char line[1024];
  int found = -1;
  const std::string pat = "\"key\": \"" + key + "\"";
  while (std::fgets(line, sizeof line, f)) {
    const char *k = std::strstr(line, pat.c_str());
    const char *v = std::strstr(line, "\"variant\": ");
    if (k && v) {
      int var = std::atoi(v + 11);
      if (var >= 0 && var < nvar) found = var;
    }
  }
  std::fclose(f);
  return found;
}

}  // namespace

extern "C" lbm_status lbm_autotune(lbm_ctx *ctx, int32_t steps_per_trial, const char *cache_path,
                                   char *report, size_t report_cap) {
  if (!ctx) return fail(LBM_INVALID, "null argument");
  if (ctx->have_state) return fail(LBM_INVALID, "lbm_autotune must run before lbm_set_state");
  LBM_CK(cudaSetDevice(ctx->p.device));
  const std::string key = tune_key(ctx);
  std::string rep = "{\"key\": \"" + key + "\"";
  const int nvar = ctx->mk ? lbm::MOM_NVAR : lbm::NVAR;
  int best = cache_lookup(cache_path, key, nvar);
  if (best >= 0) {
    ctx->variant = best;
    rep += ", \"variant\": " + std::to_string(best) + ", \"cached\": true}";
  } else {
    if (steps_per_trial < 1) steps_per_trial = 1;
    const size_t N = (size_t)ctx->P.n * ctx->P.m;
    std::vector<double> rho(N, (double)ctx->p.rho_ini), zero(N, 0.0);
    lbm_status s = set_state_impl(ctx, nullptr, rho.data(), zero.data(), zero.data(), false);
    if (s != LBM_OK) return s;
    cudaEvent_t e0, e1;
    LBM_CK(cudaEventCreate(&e0));
    LBM_CK(cudaEventCreate(&e1));
    double ms[lbm::NVAR];
    best = 0;
    for (int v = 0; v < nvar && s == LBM_OK; v++) {
      dim3 g_, b_;
      size_t sm_;
      if (!ctx->mk && !step_config(ctx, v, &g_, &b_, &sm_)) {
        ms[v] = INFINITY;
        continue;
      }
      ctx->variant = v;
      for (int i = 0; i < 2 && s == LBM_OK; i++) s = launch_step(ctx);
      // median of three timed runs: one slow run (a clock change, another
      // process) must not decide the pick
      double rep[3];
      for (int r = 0; r < 3; r++) {
        cudaEventRecord(e0, ctx->stream);
        for (int i = 0; i < steps_per_trial && s == LBM_OK; i++) s = launch_step(ctx);
        cudaEventRecord(e1, ctx->stream);
        cudaEventSynchronize(e1);
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        rep[r] = (double)t / steps_per_trial;
      }
      std::sort(rep, rep + 3);
      ms[v] = rep[1];
      if (ms[v] < ms[best]) best = v;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (s == LBM_OK) s = check_device_error(ctx);
    ctx->have_state = false;  // the trial state is discarded
    ctx->iter = 0;
    ctx->g = 0;
    if (s != LBM_OK) return s;
    LBM_CK(cudaGetLastError());
    ctx->variant = best;
    std::string arr = "[";
    char buf[64];
    for (int v = 0; v < nvar; v++) {
      if (std::isinf(ms[v])) std::snprintf(buf, sizeof buf, "%snull", v ? ", " : "");
      else std::snprintf(buf, sizeof buf, "%s%.5f", v ? ", " : "", ms[v]);
      arr += buf;
    }
    arr += "]";
    rep += ", \"variant\": " + std::to_string(best) + ", \"ms\": " + arr + "}";
    if (cache_path) {
      FILE *f = std::fopen(cache_path, "a");
      if (f) {
        std::fprintf(f, "%s\n", rep.c_str());
        std::fclose(f);
      }
    }
  }
  if (report && report_cap > 0) {
    std::strncpy(report, rep.c_str(), report_cap - 1);
    report[report_cap - 1] = '\0';
  }
  return LBM_OK;
}
