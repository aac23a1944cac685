// C ABI of batched stepping (lbm_batch_*): many independent domains advanced
// by one persistent launch per step over a device-side (case, tile) work
// list, per-case du_rel checks and convergence flags on the device, and each
// run segment (check_every steps + one check) replayed as one CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "lbm_batch.cuh"
#include "lbm_internal.h"

namespace lbm {
const BatchKernels &batch_kernels_0();
const BatchKernels &batch_kernels_1();
const BatchKernels &batch_kernels_2();
}  // namespace lbm

using lbm::fail;

#define LBM_BCK(call)                                                                    \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return fail(e_ == cudaErrorMemoryAllocation ? LBM_NOMEM : LBM_CUDA,                \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                   \
  } while (0)

namespace {

struct CaseDev {
  void *raw[2] = {nullptr, nullptr};
  void *pop[2] = {nullptr, nullptr};
  uint8_t *cls = nullptr;
  uint32_t *aux = nullptr;
  lbm::BRec *rec = nullptr;
  lbm::WRec *wrec = nullptr;  // FP32 copies of rec (boundary-node pass of per-tile batches)
  float *side[2] = {nullptr, nullptr};  // per-tile batches: METAF of the records, per buffer
  int nrec = 0;
  float *uprev = nullptr, *vprev = nullptr;
  int n = 0, m = 0;
  long long fluid = 0;
};

constexpr size_t kGuard = 1024;

}  // namespace

struct lbm_batch {
  int nc = 0, model = 1, precision = LBM_FP32, device = 0;
  std::vector<lbm_params> params;
  std::vector<CaseDev> cases;
  std::vector<lbm::BatchCase> hcases;
  lbm::BatchCase *d_cases = nullptr;
  lbm::BulkArgs *d_bulk = nullptr;  // per case and parity: the bulk pass's arguments
  lbm::SpecExtra *d_extra = nullptr;  // per case: the rest of the boundary-node pass's arguments
  lbm::BatchState s{};
  int4 *d_tiles[lbm::BVAR] = {};
  int ntiles[lbm::BVAR] = {};
  int4 *d_rows = nullptr;
  int nrows = 0;
  int4 *d_special = nullptr;  // (case, node, record, flags) of every node with boundary work, sorted by kind
  int nspecial = 0;
  int2 *d_allrec = nullptr;  // per-tile kinds: (case, record) of every record (side-array sync)
  int nallrec = 0;
  int *d_nspecial = nullptr;  // nspecial on the device (the boundary-node kernel's count)
  int4 *d_live_tiles = nullptr;   // compacted work lists of the cases still stepping
  int *d_live_n = nullptr;        // [0]: live tiles
  int variant = 1;
  int special_bps = 0;        // boundary-node pass: blocks per SM (0: one thread per entry)
  bool bulk_pf = false;       // bulk pass: L2 prefetch a quarter of a wave of blocks ahead
  int bulk_pf_blocks[lbm::BVAR] = {};  // that distance per tile variant (0: not known yet)
  int sms = 152;              // multiprocessors of the device
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;  // boundary-node pass, concurrent with the bulk pass
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  const lbm::KernelSet *ks = nullptr;
  const lbm::BatchKernels *bk = nullptr;
  int *d_err = nullptr;
  cudaGraphExec_t graph = nullptr;
  int graph_k = -1, graph_var = -1, graph_bps = -1, graph_pf = -1;
  double graph_tol = -1;
  int64_t dev_bytes = 0;
  long long nodes = 0, fluid = 0;
  bool have_state = false;
  std::vector<void *> allocs;
};

namespace {

template <class T>
lbm_status balloc(lbm_batch *b, T **p, size_t count) {
  size_t bytes = std::max<size_t>(count * sizeof(T), 16);
  cudaError_t e = cudaMalloc((void **)p, bytes);
  if (e != cudaSuccess)
    return fail(LBM_NOMEM, "cudaMalloc of " + std::to_string(bytes) + " bytes: " +
                               cudaGetErrorString(e));
  b->dev_bytes += (int64_t)bytes;
  b->allocs.push_back((void *)*p);
  return LBM_OK;
}

void bfree(lbm_batch *b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  for (void *p : b->allocs) cudaFree(p);
  b->allocs.clear();
  if (b->ev_fork) cudaEventDestroy(b->ev_fork);
  if (b->ev_join) cudaEventDestroy(b->ev_join);
  if (b->side) cudaStreamDestroy(b->side);
  if (b->stream) cudaStreamDestroy(b->stream);
}

// The boundary-node pass's stream, at the highest priority the device
// offers: its blocks are latency-bound and few, so the block scheduler should
// place them as soon as a slot frees instead of after the bulk pass's
// remaining blocks (graphs keep the priority: see ensure_graph).
bool create_side_stream(cudaStream_t *s) {
  int lo = 0, hi = 0;
  if (cudaDeviceGetStreamPriorityRange(&lo, &hi) != cudaSuccess) return false;
  return cudaStreamCreateWithPriority(s, cudaStreamNonBlocking, hi) == cudaSuccess;
}

int persistent_blocks(const void *fn, int threads, int device) {
  int per_sm = 0, sms = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  return std::max(1, per_sm) * std::max(1, sms);
}

lbm_status reset_state(lbm_batch *b) {
  std::vector<int> ones(b->nc, 1);
  std::vector<long long> neg(b->nc, -1);
  LBM_BCK(cudaMemcpyAsync(b->s.active, ones.data(), b->nc * sizeof(int), cudaMemcpyHostToDevice, b->stream));
  LBM_BCK(cudaMemsetAsync(b->s.gpar, 0, b->nc * sizeof(int), b->stream));
  LBM_BCK(cudaMemsetAsync(b->s.steps, 0, b->nc * sizeof(long long), b->stream));
  LBM_BCK(cudaMemsetAsync(b->s.bad, 0, b->nc * sizeof(int), b->stream));
  LBM_BCK(cudaMemsetAsync(b->s.du_last, 0, b->nc * sizeof(double), b->stream));
  LBM_BCK(cudaMemsetAsync(b->s.have_prev, 0, b->nc * sizeof(int), b->stream));
  LBM_BCK(cudaMemcpyAsync(b->s.conv_at, neg.data(), b->nc * sizeof(long long), cudaMemcpyHostToDevice, b->stream));
  LBM_BCK(cudaStreamSynchronize(b->stream));
  return LBM_OK;
}

// Side arrays of buffer 0 from the planes, after case c was (re)initialised.
lbm_status fill_side(lbm_batch *b, int c) {
  const CaseDev &d = b->cases[c];
  if (!b->bk->per_tile || d.nrec == 0) return LBM_OK;
  lbm::StepArgs a = b->hcases[c].args[0];  // reads buffer 0
  const lbm::BRec *rec = d.rec;
  int nrec = d.nrec;
  float *side0 = d.side[0];
  void *args[] = {&a, (void *)&rec, &nrec, &side0};
  cudaError_t e = cudaLaunchKernel(b->bk->side_fill, dim3((unsigned)((nrec + 127) / 128)), dim3(128),
                                   args, 0, b->stream);
  if (e != cudaSuccess) return fail(LBM_CUDA, std::string("side fill: ") + cudaGetErrorString(e));
  return LBM_OK;
}

// f = f_eq(rho_ini, 0, 0) and its first collision, for every case.
lbm_status set_rest(lbm_batch *b) {
  for (int c = 0; c < b->nc; c++) {
    const CaseDev &d = b->cases[c];
    const size_t N = (size_t)d.n * d.m;
    std::vector<double> rho(N, (double)b->params[c].rho_ini);
    double *dr = nullptr, *dz = nullptr;
    LBM_BCK(cudaMallocAsync((void **)&dr, N * 8, b->stream));
    LBM_BCK(cudaMallocAsync((void **)&dz, N * 8, b->stream));
    LBM_BCK(cudaMemcpyAsync(dr, rho.data(), N * 8, cudaMemcpyHostToDevice, b->stream));
    LBM_BCK(cudaMemsetAsync(dz, 0, N * 8, b->stream));
    lbm::StepArgs a = b->hcases[c].args[1];  // writes buffer 0
    a.dst = d.pop[0];
    const double *f0 = nullptr;
    void *args[] = {&a, (void *)&f0, &dr, &dz, &dz};
    dim3 grid((unsigned)((d.n + 127) / 128), (unsigned)d.m);
    cudaError_t e = cudaLaunchKernel(b->ks->init[b->model][0], grid, dim3(128), args, 0, b->stream);
    cudaFreeAsync(dr, b->stream);
    cudaFreeAsync(dz, b->stream);
    if (e != cudaSuccess) return fail(LBM_CUDA, std::string("init launch: ") + cudaGetErrorString(e));
    lbm_status fs = fill_side(b, c);
    if (fs != LBM_OK) return fs;
    LBM_BCK(cudaStreamSynchronize(b->stream));  // host vectors go out of scope
  }
  lbm_status s = reset_state(b);
  if (s != LBM_OK) return s;
  b->have_state = true;
  return LBM_OK;
}

// The work lists of the cases still stepping (start of every run segment).
lbm_status launch_compact(lbm_batch *b) {
  LBM_BCK(cudaMemsetAsync(b->d_live_n, 0, 2 * sizeof(int), b->stream));
  int *cnt_t = b->d_live_n;
  int nt = b->ntiles[b->variant];
  void *targs[] = {&b->d_tiles[b->variant], &nt, &b->s.active, &b->d_live_tiles, &cnt_t};
  cudaError_t e = cudaLaunchKernel(b->bk->compact_tiles, dim3(std::min((nt + 255) / 256, 152 * 8)),
                                   dim3(256), targs, 0, b->stream);
  // the boundary-node list is not compacted: an atomic compaction would
  // scatter its sorted order; entries of converged cases return at once
  if (e != cudaSuccess) return fail(LBM_CUDA, std::string("batch compact: ") + cudaGetErrorString(e));
  return LBM_OK;
}

lbm_status launch_steps(lbm_batch *b, int k) {
  const void *fn = b->bk->step[b->model][b->variant];
  const int bx = lbm::BVAR_BX[b->variant];
  // per-tile kernels: one block per tile of the full list (blocks past the
  // live count return); persistent kernels: one wave of resident blocks
  const int grid = b->bk->per_tile ? b->ntiles[b->variant]
                                   : std::min(b->ntiles[b->variant], persistent_blocks(fn, bx, b->device));
  void *step_args0 = b->bk->per_tile ? (void *)b->d_bulk : (void *)b->d_cases;
  // prefetch distance of the per-tile bulk pass: a quarter of a wave of
  // resident blocks (the distance that served the single-domain 16-bit step)
  int pf = 0;
  if (b->bk->per_tile && b->bulk_pf) {
    int &d = b->bulk_pf_blocks[b->variant];
    if (d == 0) {
      int per_sm = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, bx, 0) != cudaSuccess)
        per_sm = 0;
      d = per_sm > 0 ? std::max(1, per_sm * b->sms / 4) : -1;
    }
    pf = d > 0 ? d : 0;
  }
  lbm_status st = launch_compact(b);
  if (st != LBM_OK) return st;
  int *cnt_t = b->d_live_n;
  for (int i = 0; i < k; i++) {
    // the boundary-node pass writes other nodes than the bulk pass and both
    // only read the source state, so it runs on a second stream alongside
    // (fork and join by events: two parallel branches when captured)
    if (b->nspecial > 0) {
      LBM_BCK(cudaEventRecord(b->ev_fork, b->stream));
      LBM_BCK(cudaStreamWaitEvent(b->side, b->ev_fork, 0));
    }
    // (k_batch_bulk's parameters; the persistent FP64 k_batch_step takes the first five)
    void *args[] = {&step_args0, &b->d_live_tiles, &cnt_t, &b->s.active, &b->s.gpar, &pf};
    cudaError_t e = cudaLaunchKernel(fn, dim3(grid), dim3(bx), args, 0, b->stream);
    if (e != cudaSuccess) return fail(LBM_CUDA, std::string("batch step: ") + cudaGetErrorString(e));
    if (b->nspecial > 0) {
      void *sargs[] = {&b->d_cases, &b->d_special, &b->d_nspecial, &b->s.active, &b->s.gpar};
      void *cargs[] = {&b->d_bulk,     &b->d_extra,    &b->d_cases, &b->d_special,
                       &b->d_nspecial, &b->s.active, &b->s.gpar};
      // both grid-stride; k_batch_special_c one thread per entry unless
      // special_bps caps its blocks per SM (lbm_batch_autotune's choice)
      const int need = (b->nspecial + 127) / 128;
      const int sg = b->bk->per_tile
                         ? (b->special_bps > 0 ? std::min(need, b->sms * b->special_bps) : need)
                         : std::min(need, b->sms * 16);
      e = cudaLaunchKernel(b->bk->special[b->model], dim3(sg), dim3(128),
                           b->bk->per_tile ? cargs : sargs, 0, b->side);
      if (e != cudaSuccess) return fail(LBM_CUDA, std::string("batch special: ") + cudaGetErrorString(e));
      LBM_BCK(cudaEventRecord(b->ev_join, b->side));
      LBM_BCK(cudaStreamWaitEvent(b->stream, b->ev_join, 0));
    }
    void *aargs[] = {&b->nc, &b->s};
    e = cudaLaunchKernel(b->bk->advance, dim3((b->nc + 255) / 256), dim3(256), aargs, 0, b->stream);
    if (e != cudaSuccess) return fail(LBM_CUDA, std::string("batch advance: ") + cudaGetErrorString(e));
  }
  return LBM_OK;
}

// Planes of the boundary records the boundary-node pass left to the side
// arrays, before anything reads whole states (per-tile kinds).
lbm_status launch_side_sync(lbm_batch *b) {
  if (!b->bk->per_tile || b->nallrec == 0) return LBM_OK;
  void *args[] = {&b->d_bulk, &b->d_extra, &b->d_allrec, &b->nallrec, &b->s.gpar};
  cudaError_t e = cudaLaunchKernel(b->bk->side_sync, dim3((unsigned)((b->nallrec + 127) / 128)),
                                   dim3(128), args, 0, b->stream);
  if (e != cudaSuccess) return fail(LBM_CUDA, std::string("side sync: ") + cudaGetErrorString(e));
  return LBM_OK;
}

lbm_status launch_check(lbm_batch *b, int k, double tol) {
  lbm_status ss = launch_side_sync(b);
  if (ss != LBM_OK) return ss;
  const int grid = b->nrows;  // one block per row tile
  void *args[] = {&b->d_cases, &b->d_rows, &b->nrows, &b->s};
  cudaError_t e = cudaLaunchKernel(b->bk->du, dim3(grid), dim3(128), args, 0, b->stream);
  if (e != cudaSuccess) return fail(LBM_CUDA, std::string("batch du: ") + cudaGetErrorString(e));
  double inv_span = 1.0 / k;
  void *cargs[] = {&b->nc, &b->s, &tol, &inv_span};
  e = cudaLaunchKernel(b->bk->converge, dim3((unsigned)((b->nc * 32 + 255) / 256)), dim3(256), cargs,
                       0, b->stream);
  if (e != cudaSuccess) return fail(LBM_CUDA, std::string("batch converge: ") + cudaGetErrorString(e));
  return LBM_OK;
}

// One graph = check_every steps followed by one convergence check.
lbm_status ensure_graph(lbm_batch *b, int k, double tol) {
  if (b->graph && b->graph_k == k && b->graph_var == b->variant && b->graph_bps == b->special_bps &&
      b->graph_pf == (int)b->bulk_pf &&
      b->graph_tol == tol)
    return LBM_OK;
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  cudaGraph_t g;
  LBM_BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  lbm_status s = launch_steps(b, k);
  if (s == LBM_OK) s = launch_check(b, k, tol);
  cudaError_t e = cudaStreamEndCapture(b->stream, &g);
  if (s != LBM_OK) return s;
  if (e != cudaSuccess) return fail(LBM_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&b->graph, g, cudaGraphInstantiateFlagUseNodePriority);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(LBM_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  b->graph_k = k;
  b->graph_var = b->variant;
  b->graph_bps = b->special_bps;
  b->graph_pf = (int)b->bulk_pf;
  b->graph_tol = tol;
  return LBM_OK;
}

}  // namespace

extern "C" {

lbm_status lbm_batch_create(const lbm_mesh *meshes, const lbm_params *params, int32_t ncases,
                            lbm_batch **out) {
  if (!meshes || !params || !out || ncases < 1) return fail(LBM_INVALID, "bad batch arguments");
  *out = nullptr;
  const lbm_params &p0 = params[0];
  for (int c = 0; c < ncases; c++) {
    if (params[c].precision != p0.precision || params[c].collision_model != p0.collision_model ||
        params[c].device != p0.device)
      return fail(LBM_INVALID, "all cases of a batch share precision, model and device");
    if (params[c].pattern != LBM_AB) return fail(LBM_INVALID, "batches use the A-B pattern");
  }
  if (p0.precision != LBM_FP64 && p0.precision != LBM_FP32 && p0.precision != LBM_FP16DEV)
    return fail(LBM_INVALID, "batch precision must be FP64, FP32 or FP16-dev");
  lbm_batch *b = new lbm_batch();
  auto bail = [&](lbm_status st) {
    bfree(b);
    delete b;
    return st;
  };
  b->nc = ncases;
  b->model = p0.collision_model;
  b->precision = p0.precision;
  b->device = p0.device;
  b->params.assign(params, params + ncases);
  switch (p0.precision) {
    case LBM_FP64: b->ks = &lbm::kernels_f64(); b->bk = &lbm::batch_kernels_0(); break;
    case LBM_FP32: b->ks = &lbm::kernels_f32(); b->bk = &lbm::batch_kernels_1(); break;
    default: b->ks = &lbm::kernels_f16(); b->bk = &lbm::batch_kernels_2(); break;
  }
  if (cudaSetDevice(p0.device) != cudaSuccess) return bail(fail(LBM_CUDA, "cudaSetDevice failed"));
  if (cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, p0.device) != cudaSuccess ||
      b->sms < 1)
    b->sms = 152;
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      !create_side_stream(&b->side) ||
      cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming) != cudaSuccess)
    return bail(fail(LBM_CUDA, "cudaStreamCreate failed"));
  lbm_status st;
  if ((st = balloc(b, &b->d_err, 1)) != LBM_OK) return bail(st);
  cudaMemset(b->d_err, 0, sizeof(int));
  b->cases.resize(ncases);
  b->hcases.resize(ncases);
  std::vector<std::vector<int4>> tiles(lbm::BVAR);
  std::vector<int4> rows;
  std::vector<int4> specials;
  std::vector<int> rbeg;  // first row tile of each case (then the total)
  std::vector<int2> allrec;  // (case, record) of every boundary record (per-tile kinds)
  std::vector<uint32_t> special_key;
  const size_t es = (size_t)b->ks->elem_size;
  const double w[9] = {4. / 9., 1. / 9., 1. / 9., 1. / 9., 1. / 9., 1. / 36., 1. / 36., 1. / 36., 1. / 36.};
  for (int c = 0; c < ncases; c++) {
    lbm::Prep P;
    if ((st = lbm::preprocess(&meshes[c], &params[c], &P)) != LBM_OK)
      return bail(fail(st, "case " + std::to_string(c) + ": " + lbm_last_error()));
    if (P.m > 65535 * 4) return bail(fail(LBM_INVALID, "case grid too tall"));
    CaseDev &d = b->cases[c];
    d.n = P.n;
    d.m = P.m;
    d.fluid = P.nfluid;
    b->nodes += (long long)P.n * P.m;
    b->fluid += P.nfluid;
    const size_t elems = (size_t)P.plane * 9 + 2 * kGuard + (size_t)P.pitch;
    for (int i = 0; i < 2; i++) {
      if ((st = balloc(b, (char **)&d.raw[i], elems * es)) != LBM_OK) return bail(st);
      cudaMemset(d.raw[i], 0, elems * es);
      d.pop[i] = (char *)d.raw[i] + kGuard * es;
    }
    if ((st = balloc(b, &d.cls, P.cls.size())) != LBM_OK) return bail(st);
    if ((st = balloc(b, &d.aux, P.aux.size())) != LBM_OK) return bail(st);
    if ((st = balloc(b, &d.rec, P.rec.size())) != LBM_OK) return bail(st);
    if ((st = balloc(b, &d.uprev, (size_t)P.n * P.m)) != LBM_OK) return bail(st);
    if ((st = balloc(b, &d.vprev, (size_t)P.n * P.m)) != LBM_OK) return bail(st);
    cudaMemcpy(d.cls, P.cls.data(), P.cls.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(d.aux, P.aux.data(), P.aux.size() * 4, cudaMemcpyHostToDevice);
    if (!P.rec.empty())
      cudaMemcpy(d.rec, P.rec.data(), P.rec.size() * sizeof(lbm::BRec), cudaMemcpyHostToDevice);
    {
      // FP32 records and, per link, the record of the node it is pulled from
      // when that node's METAF is in the side arrays (every special node but
      // the outlet ones, which take the full treatment from the planes)
      std::vector<lbm::WRec> wr(P.rec.size());
      const int D[9][2] = {{0, 0}, {1, 0}, {0, 1}, {-1, 0}, {0, -1}, {1, 1}, {-1, 1}, {-1, -1}, {1, -1}};
      // an extrapolating outlet reads its neighbours' planes through the full
      // treatment: such cases keep every plane of every record written
      bool all_planes = false;
      if (params[c].outlet_profile == 2)
        for (const lbm::BRec &r : P.rec) all_planes = all_planes || (r.flags & lbm::FL_EAST);
      for (size_t ri = 0; ri < P.rec.size(); ri++) {
        lbm::WRec &w = wr[ri];
        std::memset(&w, 0, sizeof w);
        w.flags = P.rec[ri].flags;
        w.uo = (float)P.rec[ri].uo;
        const long long node = P.rec[ri].node;
        const bool east = (P.rec[ri].flags & lbm::FL_EAST) != 0;
        const int x = (int)(node % P.pitch), y = (int)(node / P.pitch);
        for (int k = 0; k < 9; k++) {
          w.q[k] = (float)P.rec[ri].q[k];
          w.nrec[k] = -1;
          // the source of link k: node - c_k
          const int xs = x - D[k][0], ys = y - D[k][1];
          if (xs >= 0 && xs < P.n && ys >= 0 && ys < P.m) {
            const long long z = (long long)ys * P.pitch + xs;
            if (P.cls[z] == lbm::CLS_SPECIAL && !(P.rec[P.aux[z]].flags & lbm::FL_EAST))
              w.nrec[k] = (int32_t)P.aux[z];
          }
          // the reader of plane k at this node: node + c_k
          const int xt = x + D[k][0], yt = y + D[k][1];
          if (k == 0 || xt < 0 || xt >= P.n || yt < 0 || yt >= P.m) continue;
          const uint8_t ct = P.cls[(long long)yt * P.pitch + xt];
          if (ct == lbm::CLS_SOLID) continue;
          if (ct != lbm::CLS_SPECIAL || east) w.exported |= 1u << k;
        }
        if (all_planes) w.exported = 0x1FFu;
      }
      if ((st = balloc(b, &d.wrec, wr.size())) != LBM_OK) return bail(st);
      if (!wr.empty())
        cudaMemcpy(d.wrec, wr.data(), wr.size() * sizeof(lbm::WRec), cudaMemcpyHostToDevice);
      d.nrec = (int)P.rec.size();
      for (int i = 0; i < 2; i++) {
        if ((st = balloc(b, &d.side[i], P.rec.size() * 9)) != LBM_OK) return bail(st);
        cudaMemset(d.side[i], 0, std::max<size_t>(P.rec.size() * 9 * sizeof(float), 16));
      }
    }
    lbm::StepArgs a;
    std::memset(&a, 0, sizeof a);
    a.n = P.n;
    a.m = P.m;
    a.pitch = P.pitch;
    a.model = params[c].collision_model;
    a.curved = params[c].curved_boundaries;
    a.outlet = params[c].outlet_profile;
    a.plane = P.plane;
    a.cls = d.cls;
    a.aux = d.aux;
    a.rec = d.rec;
    a.omega = P.omega;
    a.omegaA = P.omegaA;
    a.rho_out = params[c].rho_out;
    a.rho0 = params[c].rho_ini;
    a.err = b->d_err;
    for (int k = 0; k < 9; k++) {
      double S = p0.precision == LBM_FP16DEV ? 4096.0 : 1.0;
      double sc = S / (w[k] * (params[c].rho_ini > 0 ? params[c].rho_ini : 1.0));
      a.scale[k] = (float)sc;
      a.inv_scale[k] = (float)(1.0 / sc);
    }
    std::memcpy(a.stmiv, P.stmiv, sizeof a.stmiv);
    for (int par = 0; par < 2; par++) {
      b->hcases[c].args[par] = a;
      b->hcases[c].args[par].src = d.pop[par];
      b->hcases[c].args[par].dst = d.pop[par ^ 1];
    }
    b->hcases[c].uprev = d.uprev;
    b->hcases[c].vprev = d.vprev;
    for (int v = 0; v < lbm::BVAR; v++) {
      const int bx = lbm::BVAR_BX[v], npt = lbm::BVAR_NPT[v];
      for (int by = 0; by < (P.m + npt - 1) / npt; by++)
        for (int tx = 0; tx < (P.n + bx - 1) / bx; tx++) tiles[v].push_back(make_int4(c, tx, by, 0));
    }
    rbeg.push_back((int)rows.size());
    for (int yb = 0; yb < (P.m + lbm::DU_NPT - 1) / lbm::DU_NPT; yb++)
      for (int tx = 0; tx < (P.n + 127) / 128; tx++) rows.push_back(make_int4(c, tx, yb, 0));
    if (b->bk->per_tile)
      for (size_t ri = 0; ri < P.rec.size(); ri++) allrec.push_back(make_int2(c, (int)ri));
    for (size_t ri = 0; ri < P.rec.size(); ri++) {
      const lbm::BRec &r = P.rec[ri];
      specials.push_back(make_int4(c, (int)r.node, (int)ri, (int)r.flags));
      special_key.push_back(r.flags);
    }
  }
  {
    // nodes of the same boundary kind (equal flags: streamed links, walls,
    // lid / inlet / outlet) next to each other, so that the warps of the
    // boundary-node pass take one path through the treatment instead of all
    std::vector<size_t> ord(specials.size());
    for (size_t i = 0; i < ord.size(); i++) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(),
                     [&](size_t x, size_t y) { return special_key[x] < special_key[y]; });
    std::vector<int4> sorted(specials.size());
    for (size_t i = 0; i < ord.size(); i++) sorted[i] = specials[ord[i]];
    specials.swap(sorted);
  }
  if ((st = balloc(b, &b->d_cases, (size_t)ncases)) != LBM_OK) return bail(st);
  cudaMemcpy(b->d_cases, b->hcases.data(), ncases * sizeof(lbm::BatchCase), cudaMemcpyHostToDevice);
  {
    std::vector<lbm::BulkArgs> bulk(2 * (size_t)ncases);
    for (int c = 0; c < ncases; c++)
      for (int par = 0; par < 2; par++) {
        const lbm::StepArgs &a = b->hcases[c].args[par];
        lbm::BulkArgs &q = bulk[2 * c + par];
        std::memset(&q, 0, sizeof q);
        q.src = a.src;
        q.dst = a.dst;
        q.cls = a.cls;
        q.plane = a.plane;
        q.pitch = a.pitch;
        q.n = a.n;
        q.m = a.m;
        q.omega = (float)a.omega;
        q.omegaA = (float)a.omegaA;
        q.rho0 = (float)a.rho0;
        for (int k = 0; k < 9; k++) {
          q.scale[k] = a.scale[k];
          q.inv_scale[k] = a.inv_scale[k];
        }
      }
    if ((st = balloc(b, &b->d_bulk, bulk.size())) != LBM_OK) return bail(st);
    cudaMemcpy(b->d_bulk, bulk.data(), bulk.size() * sizeof(lbm::BulkArgs), cudaMemcpyHostToDevice);
    std::vector<lbm::SpecExtra> extra((size_t)ncases);
    for (int c = 0; c < ncases; c++) {
      const lbm::StepArgs &a = b->hcases[c].args[0];
      lbm::SpecExtra &x = extra[c];
      std::memset(&x, 0, sizeof x);
      x.rec = a.rec;
      x.wrec = b->cases[c].wrec;
      x.side[0] = b->cases[c].side[0];
      x.side[1] = b->cases[c].side[1];
      x.aux = a.aux;
      x.nanflag = a.nanflag;
      x.curved = a.curved;
      x.outlet = a.outlet;
      x.rho_out = a.rho_out;
    }
    if ((st = balloc(b, &b->d_extra, extra.size())) != LBM_OK) return bail(st);
    cudaMemcpy(b->d_extra, extra.data(), extra.size() * sizeof(lbm::SpecExtra), cudaMemcpyHostToDevice);
  }
  for (int v = 0; v < lbm::BVAR; v++) {
    b->ntiles[v] = (int)tiles[v].size();
    if ((st = balloc(b, &b->d_tiles[v], tiles[v].size())) != LBM_OK) return bail(st);
    cudaMemcpy(b->d_tiles[v], tiles[v].data(), tiles[v].size() * sizeof(int4), cudaMemcpyHostToDevice);
  }
  size_t max_tiles = 0;
  for (int v = 0; v < lbm::BVAR; v++) max_tiles = std::max(max_tiles, tiles[v].size());
  if ((st = balloc(b, &b->d_live_tiles, max_tiles)) != LBM_OK ||
      (st = balloc(b, &b->d_live_n, 2)) != LBM_OK)
    return bail(st);
  b->nallrec = (int)allrec.size();
  if ((st = balloc(b, &b->d_allrec, allrec.size())) != LBM_OK) return bail(st);
  if (!allrec.empty())
    cudaMemcpy(b->d_allrec, allrec.data(), allrec.size() * sizeof(int2), cudaMemcpyHostToDevice);
  b->nspecial = (int)specials.size();
  if ((st = balloc(b, &b->d_special, specials.size())) != LBM_OK) return bail(st);
  if ((st = balloc(b, &b->d_nspecial, 1)) != LBM_OK) return bail(st);
  cudaMemcpy(b->d_nspecial, &b->nspecial, sizeof(int), cudaMemcpyHostToDevice);
  if (!specials.empty())
    cudaMemcpy(b->d_special, specials.data(), specials.size() * sizeof(int4), cudaMemcpyHostToDevice);
  b->nrows = (int)rows.size();
  if ((st = balloc(b, &b->d_rows, rows.size())) != LBM_OK) return bail(st);
  cudaMemcpy(b->d_rows, rows.data(), rows.size() * sizeof(int4), cudaMemcpyHostToDevice);
  rbeg.push_back((int)rows.size());
  {
    int *d_rbeg = nullptr;
    if ((st = balloc(b, &d_rbeg, rbeg.size())) != LBM_OK ||
        (st = balloc(b, &b->s.part, rows.size())) != LBM_OK)
      return bail(st);
    cudaMemcpy(d_rbeg, rbeg.data(), rbeg.size() * sizeof(int), cudaMemcpyHostToDevice);
    b->s.rbeg = d_rbeg;
  }
  lbm::BatchState &s = b->s;
  if ((st = balloc(b, &s.active, ncases)) != LBM_OK || (st = balloc(b, &s.gpar, ncases)) != LBM_OK ||
      (st = balloc(b, &s.steps, ncases)) != LBM_OK ||
      (st = balloc(b, &s.bad, ncases)) != LBM_OK || (st = balloc(b, &s.du_last, ncases)) != LBM_OK ||
      (st = balloc(b, &s.have_prev, ncases)) != LBM_OK ||
      (st = balloc(b, &s.conv_at, ncases)) != LBM_OK)
    return bail(st);
  if (cudaGetLastError() != cudaSuccess) return bail(fail(LBM_CUDA, "batch upload failed"));
  if ((st = reset_state(b)) != LBM_OK) return bail(st);
  *out = b;
  return LBM_OK;
}

void lbm_batch_destroy(lbm_batch *b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  bfree(b);
  delete b;
}

lbm_status lbm_batch_info(const lbm_batch *b, int64_t *nodes, int64_t *fluid_nodes,
                          int32_t *tile_variant, int64_t *device_bytes) {
  if (!b) return fail(LBM_INVALID, "null argument");
  if (nodes) *nodes = b->nodes;
  if (fluid_nodes) *fluid_nodes = b->fluid;
  if (tile_variant) *tile_variant = b->variant;
  if (device_bytes) *device_bytes = b->dev_bytes;
  return LBM_OK;
}

lbm_status lbm_batch_set_tile(lbm_batch *b, int32_t tile_variant) {
  if (!b || tile_variant < 0 || tile_variant >= lbm::BVAR)
    return fail(LBM_INVALID, "tile variant must be 0.." + std::to_string(lbm::BVAR - 1));
  b->variant = tile_variant;
  return LBM_OK;
}

lbm_status lbm_batch_set_launch(lbm_batch *b, int32_t special_blocks_per_sm,
                                int32_t bulk_prefetch) {
  if (!b || special_blocks_per_sm < 0 || special_blocks_per_sm > 16)
    return fail(LBM_INVALID, "blocks per SM must be 0 (one thread per entry) .. 16");
  if (bulk_prefetch != 0 && bulk_prefetch != 1) return fail(LBM_INVALID, "bulk_prefetch is 0 or 1");
  b->special_bps = special_blocks_per_sm;
  b->bulk_pf = bulk_prefetch != 0;
  return LBM_OK;
}

lbm_status lbm_batch_set_rest(lbm_batch *b) {
  if (!b) return fail(LBM_INVALID, "null argument");
  LBM_BCK(cudaSetDevice(b->device));
  return set_rest(b);
}

lbm_status lbm_batch_set_state(lbm_batch *b, int32_t c, const double *rho, const double *u,
                               const double *v) {
  if (!b || c < 0 || c >= b->nc || !rho || !u || !v) return fail(LBM_INVALID, "bad argument");
  LBM_BCK(cudaSetDevice(b->device));
  lbm_status st;
  if (!b->have_state && (st = set_rest(b)) != LBM_OK) return st;
  const CaseDev &d = b->cases[c];
  const size_t N = (size_t)d.n * d.m;
  double *dm = nullptr;
  LBM_BCK(cudaMallocAsync((void **)&dm, 3 * N * 8, b->stream));
  LBM_BCK(cudaMemcpyAsync(dm, rho, N * 8, cudaMemcpyHostToDevice, b->stream));
  LBM_BCK(cudaMemcpyAsync(dm + N, u, N * 8, cudaMemcpyHostToDevice, b->stream));
  LBM_BCK(cudaMemcpyAsync(dm + 2 * N, v, N * 8, cudaMemcpyHostToDevice, b->stream));
  // f = f_eq(rho, u, v), first collision into buffer 0; the case restarts
  lbm::StepArgs a = b->hcases[c].args[1];
  a.dst = d.pop[0];
  const double *f0 = nullptr, *pr = dm, *pu = dm + N, *pv = dm + 2 * N;
  void *args[] = {&a, (void *)&f0, (void *)&pr, (void *)&pu, (void *)&pv};
  dim3 grid((unsigned)((d.n + 127) / 128), (unsigned)d.m);
  cudaError_t e = cudaLaunchKernel(b->ks->init[b->model][0], grid, dim3(128), args, 0, b->stream);
  cudaFreeAsync(dm, b->stream);
  if (e != cudaSuccess) return fail(LBM_CUDA, std::string("init launch: ") + cudaGetErrorString(e));
  lbm_status fs = fill_side(b, c);
  if (fs != LBM_OK) return fs;
  const int one = 1, zero = 0;
  const long long zl = 0, neg = -1;
  LBM_BCK(cudaMemcpyAsync(b->s.active + c, &one, sizeof one, cudaMemcpyHostToDevice, b->stream));
  LBM_BCK(cudaMemcpyAsync(b->s.gpar + c, &zero, sizeof zero, cudaMemcpyHostToDevice, b->stream));
  LBM_BCK(cudaMemcpyAsync(b->s.steps + c, &zl, sizeof zl, cudaMemcpyHostToDevice, b->stream));
  LBM_BCK(cudaMemcpyAsync(b->s.have_prev + c, &zero, sizeof zero, cudaMemcpyHostToDevice, b->stream));
  LBM_BCK(cudaMemcpyAsync(b->s.bad + c, &zero, sizeof zero, cudaMemcpyHostToDevice, b->stream));
  LBM_BCK(cudaMemcpyAsync(b->s.conv_at + c, &neg, sizeof neg, cudaMemcpyHostToDevice, b->stream));
  LBM_BCK(cudaStreamSynchronize(b->stream));
  return LBM_OK;
}

lbm_status lbm_batch_autotune(lbm_batch *b, int32_t steps_per_trial, char *report,
                              size_t report_cap) {
  if (!b) return fail(LBM_INVALID, "null argument");
  if (b->have_state) return fail(LBM_INVALID, "lbm_batch_autotune must run before stepping");
  LBM_BCK(cudaSetDevice(b->device));
  if (steps_per_trial < 1) steps_per_trial = 1;
  lbm_status s = set_rest(b);
  if (s != LBM_OK) return s;
  cudaEvent_t e0, e1;
  LBM_BCK(cudaEventCreate(&e0));
  LBM_BCK(cudaEventCreate(&e1));
  auto trial = [&](double *out) {
    s = launch_steps(b, 2);
    cudaEventRecord(e0, b->stream);
    if (s == LBM_OK) s = launch_steps(b, steps_per_trial);
    cudaEventRecord(e1, b->stream);
    cudaEventSynchronize(e1);
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    *out = (double)t / steps_per_trial;
  };
  // bulk tiles first (boundary pass one thread per entry), then the
  // boundary pass's blocks per SM with the chosen tile: fewer blocks leave
  // block slots to the bulk pass that runs alongside
  constexpr int kBps[4] = {0, 2, 4, 8};
  double ms[lbm::BVAR], bms[4] = {0, 0, 0, 0}, pms[2] = {0, 0};
  int best = 0, best_bps = 0;
  b->special_bps = 0;
  b->bulk_pf = false;
  for (int v = 0; v < lbm::BVAR && s == LBM_OK; v++) {
    b->variant = v;
    trial(&ms[v]);
    if (ms[v] < ms[best]) best = v;
  }
  b->variant = best;
  const bool tune_bps = b->bk->per_tile && b->nspecial > 0;
  for (int i = 0; i < 4 && tune_bps && s == LBM_OK; i++) {
    b->special_bps = kBps[i];
    trial(&bms[i]);
    if (bms[i] < bms[best_bps]) best_bps = i;
  }
  // then the bulk pass's L2 prefetch of the tile a quarter of a wave ahead
  b->special_bps = kBps[best_bps];
  bool pf = false;
  for (int i = 0; i < 2 && b->bk->per_tile && s == LBM_OK; i++) {
    b->bulk_pf = i == 1;
    trial(&pms[i]);
    if (i == 1 && pms[1] < pms[0]) pf = true;
  }
  b->bulk_pf = pf;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->have_state = false;
  if (s != LBM_OK) return s;
  b->special_bps = kBps[best_bps];
  if (report && report_cap > 0) {
    std::string r = "{\"variant\": " + std::to_string(best) + ", \"ms\": [";
    char buf[32];
    for (int v = 0; v < lbm::BVAR; v++) {
      std::snprintf(buf, sizeof buf, "%s%.5f", v ? ", " : "", ms[v]);
      r += buf;
    }
    r += "], \"special_blocks_per_sm\": " + std::to_string(b->special_bps) + ", \"special_ms\": [";
    for (int i = 0; i < 4; i++) {
      std::snprintf(buf, sizeof buf, "%s%.5f", i ? ", " : "", bms[i]);
      r += buf;
    }
    r += "], \"bulk_prefetch\": " + std::to_string((int)b->bulk_pf) + ", \"prefetch_ms\": [";
    for (int i = 0; i < 2; i++) {
      std::snprintf(buf, sizeof buf, "%s%.5f", i ? ", " : "", pms[i]);
      r += buf;
    }
    r += "]}";
    std::strncpy(report, r.c_str(), report_cap - 1);
    report[report_cap - 1] = '\0';
  }
  return LBM_OK;
}

lbm_status lbm_batch_run(lbm_batch *b, int64_t max_steps, int32_t check_every, double tol,
                         int64_t *steps, double *du_rel, int32_t *converged, double *seconds) {
  if (!b || max_steps < 0 || check_every < 1) return fail(LBM_INVALID, "bad argument");
  LBM_BCK(cudaSetDevice(b->device));
  lbm_status s;
  if (!b->have_state && (s = set_rest(b)) != LBM_OK) return s;
  if ((s = ensure_graph(b, check_every, tol)) != LBM_OK) return s;
  std::vector<int> act(b->nc);
  LBM_BCK(cudaStreamSynchronize(b->stream));
  const auto t0 = std::chrono::steady_clock::now();
  int64_t done = 0;
  while (done < max_steps) {
    LBM_BCK(cudaGraphLaunch(b->graph, b->stream));
    done += check_every;
    LBM_BCK(cudaMemcpyAsync(act.data(), b->s.active, b->nc * sizeof(int), cudaMemcpyDeviceToHost,
                            b->stream));
    LBM_BCK(cudaStreamSynchronize(b->stream));
    if (std::none_of(act.begin(), act.end(), [](int v) { return v != 0; })) break;
  }
  const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  LBM_BCK(cudaGetLastError());
  if (seconds) *seconds = el;
  std::vector<long long> st(b->nc), ca(b->nc);
  std::vector<int> bad(b->nc);
  LBM_BCK(cudaMemcpy(st.data(), b->s.steps, b->nc * 8, cudaMemcpyDeviceToHost));
  LBM_BCK(cudaMemcpy(ca.data(), b->s.conv_at, b->nc * 8, cudaMemcpyDeviceToHost));
  LBM_BCK(cudaMemcpy(bad.data(), b->s.bad, b->nc * 4, cudaMemcpyDeviceToHost));
  if (du_rel) LBM_BCK(cudaMemcpy(du_rel, b->s.du_last, b->nc * 8, cudaMemcpyDeviceToHost));
  bool any_bad = false;
  for (int c = 0; c < b->nc; c++) {
    if (steps) steps[c] = st[c];
    if (converged) converged[c] = bad[c] ? -1 : (ca[c] >= 0 ? 1 : 0);
    any_bad = any_bad || bad[c];
  }
  if (any_bad) return fail(LBM_DIVERGED, "NaN in at least one case (converged[c] = -1)");
  return LBM_OK;
}

lbm_status lbm_batch_get_fields(lbm_batch *b, int32_t c, double *rho, double *u, double *v) {
  if (!b || c < 0 || c >= b->nc) return fail(LBM_INVALID, "bad case index");
  if (!b->have_state) return fail(LBM_INVALID, "no state yet");
  LBM_BCK(cudaSetDevice(b->device));
  const CaseDev &d = b->cases[c];
  const size_t N = (size_t)d.n * d.m;
  int par = 0;
  LBM_BCK(cudaMemcpy(&par, b->s.gpar + c, sizeof(int), cudaMemcpyDeviceToHost));
  lbm::StepArgs a = b->hcases[c].args[par & 1];
  const dim3 grid((unsigned)((d.n + 127) / 128), (unsigned)std::min(d.m, 64));
  lbm::FinishOut o;
  std::memset(&o, 0, sizeof o);
  std::vector<double> rho0(N, (double)b->params[c].rho_ini);
  double *tmp = nullptr;
  LBM_BCK(cudaMalloc((void **)&tmp, (N * 6 + (size_t)grid.x * grid.y * lbm::NSUM) * 8));
  o.rho = tmp;
  o.u = tmp + N;
  o.v = tmp + 2 * N;
  o.rho_solid = tmp + 3 * N;
  o.u_solid = tmp + 4 * N;
  o.v_solid = tmp + 5 * N;
  o.partial = tmp + 6 * N;
  cudaMemcpy((void *)o.rho_solid, rho0.data(), N * 8, cudaMemcpyHostToDevice);
  cudaMemset((void *)o.u_solid, 0, 2 * N * 8);
  void *args[] = {&a, &o};
  lbm_status ss = launch_side_sync(b);
  if (ss != LBM_OK) {
    cudaFree(tmp);
    return ss;
  }
  cudaError_t e = cudaLaunchKernel(b->ks->finish[lbm::PH_AB], grid, dim3(128), args, 0, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e == cudaSuccess && rho) e = cudaMemcpy(rho, o.rho, N * 8, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && u) e = cudaMemcpy(u, o.u, N * 8, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && v) e = cudaMemcpy(v, o.v, N * 8, cudaMemcpyDeviceToHost);
  cudaFree(tmp);
  if (e != cudaSuccess) return fail(LBM_CUDA, std::string("batch fields: ") + cudaGetErrorString(e));
  return LBM_OK;
}

lbm_status lbm_batch_dims(const lbm_batch *b, int32_t c, int32_t *n, int32_t *m) {
  if (!b || c < 0 || c >= b->nc) return fail(LBM_INVALID, "bad case index");
  if (n) *n = b->cases[c].n;
  if (m) *m = b->cases[c].m;
  return LBM_OK;
}

}  // extern "C"
