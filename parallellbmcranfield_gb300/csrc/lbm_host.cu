// C ABI of the D2Q9 step library (include/lbm_gb300.h): context lifetime,
// state upload, the stepping loop and field / diagnostic read-back.
#include <cuda_runtime.h>

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
  double *d_partial = nullptr, *d_sums = nullptr;
  double *d_hist = nullptr;
  int hist_cap = 0;
  int nblk = 0;              // blocks of a node-grid launch
  int64_t iter = 0;          // completed iterations
  int64_t g = 0;             // index of the METAF generation held on the device
  bool have_state = false;
  int64_t dev_bytes = 0;
  lbm::StepArgs base{};
};

namespace {

constexpr int kBlock = 128;

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
  void *ptrs[] = {c->pop[0], c->pop[1], c->sb[0],    c->sb[1],      c->d_cls,
                  c->d_aux,  c->d_rec,  c->d_rho0,   c->d_u0,       c->d_v0,
                  c->d_uprev, c->d_vprev, c->d_partial, c->d_sums, c->d_hist};
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
  if (c->p.pattern == LBM_AB) {
    a.src = c->pop[c->g & 1];
    a.dst = c->pop[(c->g + 1) & 1];
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

lbm_status launch_step(lbm_ctx *c) {
  lbm::StepArgs a = args_now(c);
  void *args[] = {&a};
  int ph = layout_of(c);
  lbm_status s = launch(c->ks->step[c->p.collision_model][ph], node_grid(c), dim3(kBlock), args,
                        c->stream);
  if (s != LBM_OK) return s;
  c->g++;
  return LBM_OK;
}

lbm_status launch_resid(lbm_ctx *c, double *out) {
  lbm::StepArgs a = args_now(c);
  void *args[] = {&a, &out};
  return launch(c->ks->resid[layout_of(c)], dim3(1), dim3(256), args, c->stream);
}

lbm_status launch_finish(lbm_ctx *c, lbm::FinishOut &o) {
  lbm::StepArgs a = args_now(c);
  o.partial = c->d_partial;
  void *args[] = {&a, &o};
  lbm_status s = launch(c->ks->finish[layout_of(c)], node_grid(c), dim3(kBlock), args, c->stream);
  if (s != LBM_OK) return s;
  void *rargs[] = {&c->d_partial, &c->nblk, &c->d_sums};
  return launch(c->ks->reduce, dim3(1), dim3(32 * lbm::NSUM), rargs,
                c->stream);
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
  c->g = 0;
  lbm::StepArgs a = args_now(c);
  a.dst = c->pop[0];
  a.sb_dst = c->sb[0];
  void *args[] = {&a, &d_f, &c->d_rho0, &c->d_u0, &c->d_v0};
  int which = c->p.pattern == LBM_AB ? 0 : 1;
  lbm_status s = launch(c->ks->init[c->p.collision_model][which], node_grid(c), dim3(kBlock),
                        args, c->stream);
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
  if (params->precision < LBM_FP64 || params->precision > LBM_BF16DEV)
    return fail(LBM_INVALID, "unknown precision");
  if (params->pattern != LBM_AB && params->pattern != LBM_AA)
    return fail(LBM_INVALID, "unknown pattern");
  lbm_ctx *c = new lbm_ctx();
  c->p = *params;
  lbm_status s = lbm::preprocess(mesh, params, &c->P);
  if (s != LBM_OK) {
    delete c;
    return s;
  }
  if (c->P.m > 65535) {
    delete c;
    return fail(LBM_INVALID, "grid taller than 65535 rows");
  }
  switch (params->precision) {
    case LBM_FP64: c->ks = &lbm::kernels_f64(); break;
    case LBM_FP32: c->ks = &lbm::kernels_f32(); break;
    case LBM_FP16DEV: c->ks = &lbm::kernels_f16(); break;
    default: c->ks = &lbm::kernels_b16(); break;
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
  const size_t pop_elems = (size_t)P.plane * 9;
  const int npop = params->pattern == LBM_AB ? 2 : 1;
  for (int i = 0; i < npop; i++) {
    if ((s = dalloc(c, (char **)&c->pop[i], pop_elems * c->ks->elem_size)) != LBM_OK) return bail(s);
    if (cudaMemset(c->pop[i], 0, pop_elems * c->ks->elem_size) != cudaSuccess)
      return bail(fail(LBM_CUDA, "cudaMemset failed"));
  }
  if (params->pattern == LBM_AA)
    for (int i = 0; i < 2; i++)
      if ((s = dalloc(c, &c->sb[i], (size_t)P.nsb * 9)) != LBM_OK) return bail(s);
  if ((s = dalloc(c, &c->d_cls, P.cls.size())) != LBM_OK) return bail(s);
  if ((s = dalloc(c, &c->d_aux, P.aux.size())) != LBM_OK) return bail(s);
  if ((s = dalloc(c, &c->d_rec, P.rec.size())) != LBM_OK) return bail(s);
  if ((s = dalloc(c, &c->d_rho0, N)) != LBM_OK) return bail(s);
  if ((s = dalloc(c, &c->d_u0, N)) != LBM_OK) return bail(s);
  if ((s = dalloc(c, &c->d_v0, N)) != LBM_OK) return bail(s);
  c->nblk = (int)(node_grid(c).x * node_grid(c).y);
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
  if (bytes_per_node_step) *bytes_per_node_step = 18 * ctx->ks->elem_size;
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
  for (int i = 0; i < 5 && s == LBM_OK; i++)
    if (host[i] && cudaMallocAsync((void **)dev[i], cnt[i] * 8, ctx->stream) != cudaSuccess)
      s = fail(LBM_NOMEM, "device temporary for field read-back");
  if (s == LBM_OK) s = launch_finish(ctx, o);
  for (int i = 0; i < 5 && s == LBM_OK; i++)
    if (host[i] && cudaMemcpyAsync(host[i], *dev[i], cnt[i] * 8, cudaMemcpyDeviceToHost,
                                   ctx->stream) != cudaSuccess)
      s = fail(LBM_CUDA, "field read-back failed");
  for (int i = 0; i < 5; i++)
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
  out->du_rel = ctx->have_prev ? std::sqrt(h[lbm::S_DU] / h[lbm::S_UU]) : INFINITY;
  ctx->have_prev = true;
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
  lbm_status s = lbm::check_noalloc(ctx->ks, args_now(ctx), layout_of(ctx), node_grid(ctx),
                                    ctx->stream, h);
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
