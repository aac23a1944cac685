// Batched stepping of many independent domains (cavities, channels): per step
// one bulk launch covers a device-side work list of (case, tile) (one block
// per tile; FP64 walks it with a persistent grid), and a second launch,
// alongside it, the list of (case, node) with boundary work; per-case parity, step counters and convergence flags live on the
// device so that a whole run segment (steps + check) can be captured in one
// CUDA graph.
#pragma once
#include "lbm_device.cuh"

namespace lbm {

// Per-case launch arguments for both A-B parities (args[p] reads buffer p).
struct BatchCase {
  StepArgs args[2];
  float *uprev, *vprev;  // du_rel reference fields, n*m
};

// Tile shapes of the batched step (threads along x, rows per thread).
constexpr int BVAR = 4;
constexpr int BVAR_BX[BVAR] = {128, 64, 128, 128};
constexpr int BVAR_NPT[BVAR] = {1, 4, 2, 4};

constexpr int DU_NPT = 4;  // rows per thread of the du check

struct BatchState {
  int *active;        // 1 while the case still steps
  int *gpar;          // METAF generation parity of each case
  long long *steps;   // iterations completed by each case
  double2 *part;      // per row tile of the last check: sum |du|^2, sum |u|^2
  const int *rbeg;    // row tiles of case c: [rbeg[c], rbeg[c + 1])
  int *bad;           // per case: NaN seen
  double *du_last;    // per case: du_rel of the last check
  int *have_prev;     // per case: reference fields valid
  long long *conv_at; // per case: iteration at which du_rel <= tol was first seen (-1)
};

// Work-list compaction: the entries (x = case) of cases still stepping, in
// any order, and their count (zeroed before the launch).  Run at the start of
// every run segment, so that the step kernels walk only live work once cases
// have converged.
template <class E>
__global__ void k_batch_compact(const E *in, int n, const int *active, E *out, int *count) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const E e = in[i];
    if (active[e.x]) out[atomicAdd(count, 1)] = e;
  }
}

template <class ST, int MODEL, int BX, int NPT>
__global__ void __launch_bounds__(BX) k_batch_step(const BatchCase *cases, const int4 *tiles,
                                                   const int *ntiles_live, const int *active,
                                                   const int *gpar) {
  // The tile's case arguments are copied to shared memory once per tile: read
  // through a pointer to global memory they could alias the population
  // stores, and every node would reload them.
  __shared__ __align__(16) StepArgs sa;
  static_assert(sizeof(StepArgs) % 4 == 0, "word copy");
  const int ntiles = *ntiles_live;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int4 tl = tiles[t];
    if (!active[tl.x]) continue;  // uniform over the block
    const int *from = (const int *)&cases[tl.x].args[gpar[tl.x] & 1];
    __syncthreads();  // the previous tile is done with sa
    for (int i = threadIdx.x; i < (int)(sizeof(StepArgs) / 4); i += BX) ((int *)&sa)[i] = from[i];
    __syncthreads();
    step_column<ST, MODEL, PH_AB, NPT, true>(sa, tl.y * BX + threadIdx.x, tl.z * NPT);
  }
}

// One special node whose boundary record is known: the special branch of
// step_one (the same treatment and collision) without the class, index and
// record lookups that find it.
template <class ST, int MODEL, bool EXTRAP = true, class REC = BRec,
          class ACC = AccMain<ST, PH_AB, ST::SHIFT>>
__device__ __forceinline__ void step_special_rec(const StepArgs &a, long long node,
                                                 const REC &r) {
  using R = typename ST::R;
  constexpr bool SH = ST::SHIFT;
  R F[9], mac[3];
  special_node_rec<R, ACC, EXTRAP, REC>(a, ACC(a, a.src), node, r, F, mac);
  if constexpr (SH) {
    R M[9];
    collide_dev<MODEL>(F, mac[0], mac[1], mac[2], a, M);
    store_node_dev<ST, PH_AB>(a, node, (uint8_t)CLS_SPECIAL, M);
  } else {
    collide_store<ST, MODEL, PH_AB>(a, node, (uint8_t)CLS_SPECIAL, F, mac[0], mac[1], mac[2]);
  }
}

// The nodes with boundary work of every case, one thread each, from a list
// of (case, linear node index, boundary record, record flags) sorted by the
// flags: consecutive threads take the same path through the treatment, and
// the record comes with the entry (no class or index lookups on the node).
// The case arguments are read through restrict pointers: they do not alias
// the population stores, so the compiler may keep them in registers across
// the node's stores instead of reloading them.
template <class ST, int MODEL>
__global__ void __launch_bounds__(128) k_batch_special(const BatchCase *__restrict__ cases,
                                                       const int4 *__restrict__ list,
                                                       const int *__restrict__ nlist_live,
                                                       const int *__restrict__ active,
                                                       const int *__restrict__ gpar) {
  const int nlist = *nlist_live;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nlist; i += gridDim.x * blockDim.x) {
    const int4 e = list[i];
    if (!active[e.x]) continue;
    const StepArgs &a = cases[e.x].args[gpar[e.x] & 1];
    step_special_rec<ST, MODEL>(a, (long long)e.y, a.rec[e.z]);
  }
}

// The fields of one case's StepArgs that the bulk update reads, per A-B
// parity (k_batch_bulk): 128 bytes instead of the full argument record.
struct BulkArgs {
  const void *src;
  void *dst;
  const uint8_t *cls;
  long long plane;
  int pitch, n, m;
  float omega, omegaA, rho0;
  float scale[9], inv_scale[9];
};
static_assert(sizeof(BulkArgs) == 128, "BulkArgs layout");

// Bulk nodes (class 1) of one column of NPT rows; every other class is left
// to the boundary-node pass.  The loads of all NPT nodes go out first.
template <class ST, int MODEL, int NPT>
__device__ __forceinline__ void bulk_column(const StepArgs &a, int x, int y0) {
  using R = typename ST::R;
  using T = typename ST::T;
  if (x >= a.n) return;
  uint8_t c[NPT];
#pragma unroll
  for (int j = 0; j < NPT; j++)
    c[j] = (y0 + j < a.m) ? a.cls[(long long)(y0 + j) * a.pitch + x] : (uint8_t)CLS_SOLID;
  const T *s = (const T *)a.src;
  R F[NPT][9];
#pragma unroll
  for (int j = 0; j < NPT; j++) {
    const long long node = (long long)(y0 + j) * a.pitch + x;
#pragma unroll
    for (int k = 0; k < 9; k++)
      F[j][k] = (c[j] == CLS_BULK) ? ld_dev<ST>(s + pull_index<PH_AB>(k, node, a), k, a) : R(0);
  }
#pragma unroll
  for (int j = 0; j < NPT; j++)
    if (c[j] == CLS_BULK)
      bulk_store<ST, MODEL, PH_AB>(a, (long long)(y0 + j) * a.pitch + x, c[j], F[j]);
}

// Batched bulk pass with one block per live (case, tile): no persistent loop
// and no shared-memory copy of the case arguments, so a block's loads go out
// as soon as it starts and the hardware keeps every SM filled with blocks.
// Blocks past the live count (the grid is sized for all tiles when the
// graph is captured) return at once.  With pf > 0 the first 10 x NPT threads
// first prefetch into L2 the tile pf positions further down the live list
// (a fraction of a wave of blocks later): its NPT rows of the nine planes
// and of the class bytes, one bulk prefetch each (a hint, nothing waits for
// it; rows inside the case, x + BX <= pitch since the pitch is a multiple of
// 256, and every address 16-byte aligned).
template <class ST, int MODEL, int BX, int NPT>
__global__ void __launch_bounds__(BX) k_batch_bulk(const BulkArgs *__restrict__ args,
                                                   const int4 *__restrict__ tiles,
                                                   const int *__restrict__ ntiles_live,
                                                   const int *__restrict__ active,
                                                   const int *__restrict__ gpar, int pf) {
  static_assert(10 * NPT <= BX, "prefetch threads");
  const int t = blockIdx.x;
  const int nlive = __ldg(ntiles_live);
  if (t >= nlive) return;
  if (pf > 0 && threadIdx.x < 10 * NPT && t + pf < nlive) {
    const int4 u = __ldg(&tiles[t + pf]);
    const BulkArgs &q = args[2 * u.x + (__ldg(&gpar[u.x]) & 1)];
    const int k = threadIdx.x / NPT, y = u.z * NPT + threadIdx.x % NPT;
    if (y < q.m) {
      const long long node = (long long)y * q.pitch + (long long)u.y * BX;
      using T = typename ST::T;
      if (k < 9) {
        const T *p = (const T *)q.src + (long long)k * q.plane + node;
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "n"(BX * (int)sizeof(T))
                     : "memory");
      } else {
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(q.cls + node), "n"(BX)
                     : "memory");
      }
    }
  }
  const int4 tl = __ldg(&tiles[t]);
  if (!__ldg(&active[tl.x])) return;
  const BulkArgs &b = args[2 * tl.x + (__ldg(&gpar[tl.x]) & 1)];
  StepArgs a;
  a.src = const_cast<void *>(b.src);
  a.dst = b.dst;
  a.cls = b.cls;
  a.plane = b.plane;
  a.pitch = b.pitch;
  a.n = b.n;
  a.m = b.m;
  a.omega = b.omega;
  a.omegaA = b.omegaA;
  a.rho0 = b.rho0;
  a.nanflag = nullptr;
  if constexpr (sizeof(typename ST::T) == 2) {
#pragma unroll
    for (int k = 0; k < 9; k++) {
      a.scale[k] = b.scale[k];
      a.inv_scale[k] = b.inv_scale[k];
    }
  }
  bulk_column<ST, MODEL, NPT>(a, tl.y * BX + threadIdx.x, tl.z * NPT);
}

// Boundary record of the per-tile batches: the fields of BRec the treatment
// reads, in FP32 (the single-domain FP32 and FP16-dev paths convert the same
// doubles to FP32), 48 bytes instead of 112.
// nrec[k]: the record of the node the link k is pulled from (node - c_k)
// when that node's METAF is kept in the side arrays, else -1.  exported:
// the planes k another update reads from the planes at this node (a bulk
// neighbour at node + c_k, or one that reads it without the side arrays);
// the boundary-node pass writes only those planes, k_batch_side_sync the
// others before anything else reads the whole state.
struct WRec {
  uint32_t flags;
  float uo;
  float q[9];
  int32_t nrec[9];
  uint32_t exported;
};
static_assert(sizeof(WRec) == 84, "WRec layout");

// METAF of a special node's own links and of its special neighbours from
// the node-major side array of the current parity (9 values per record,
// written by the boundary-node pass next to the planes, equal to what a
// plane read returns: FP16-dev values pass through the storage's rounding),
// every other read from the planes as AccMain reads it.  A wall node's own
// values and its neighbours along the wall then come from a few contiguous
// sectors instead of one sector per value and row.
template <class ST>
struct AccSideB {
  using R = typename ST::R;
  static constexpr bool dev = ST::SHIFT;
  const StepArgs &a;
  const typename ST::T *s;
  const float *side;
  long long node;
  int ri;
  const int32_t *nrec;
  __device__ AccSideB(const StepArgs &a_, const float *side_, long long node_, int ri_,
                      const int32_t *nrec_)
      : a(a_), s((const typename ST::T *)a_.src), side(side_), node(node_), ri(ri_), nrec(nrec_) {}
  __device__ __forceinline__ R meta(long long z, int k) const {
    if (z == node) return side[(size_t)ri * 9 + k];
    if (z == node - nb(k, a.pitch)) {
      const int r = nrec[k];
      if (r >= 0) return side[(size_t)r * 9 + k];
    }
    if (a.cls[z] == CLS_SOLID) return dev ? -wgt<R>(k) * (R)a.rho0 : R(0);
    const typename ST::T *p = s + slot_of<PH_AB>(k, z, a);
    return dev ? ST::cvt_dev(__ldg(p), k, a) : ST::ld(p, k, a);
  }
};

// Per-case fields the boundary-node pass needs beyond BulkArgs.
struct SpecExtra {
  const BRec *rec;
  const WRec *wrec;
  float *side[2];  // side arrays of buffer 0 / 1 (9 values per record)
  const uint32_t *aux;
  int *nanflag;
  int curved, outlet;
  double rho_out;
};

// A case's arguments for the boundary treatment, in registers: the 128-byte
// BulkArgs of its parity and its SpecExtra.
template <class ST>
__device__ __forceinline__ void spec_args(const BulkArgs &b, const SpecExtra &x, StepArgs &a) {
  a.src = const_cast<void *>(b.src);
  a.dst = b.dst;
  a.cls = b.cls;
  a.plane = b.plane;
  a.pitch = b.pitch;
  a.n = b.n;
  a.m = b.m;
  a.omega = b.omega;
  a.omegaA = b.omegaA;
  a.rho0 = b.rho0;
  a.rec = x.rec;
  a.aux = x.aux;
  a.nanflag = x.nanflag;
  a.curved = x.curved;
  a.outlet = x.outlet;
  a.rho_out = x.rho_out;
  if constexpr (sizeof(typename ST::T) == 2) {
#pragma unroll
    for (int k = 0; k < 9; k++) {
      a.scale[k] = b.scale[k];
      a.inv_scale[k] = b.inv_scale[k];
    }
  }
}

// A node of an extrapolating outlet: the full treatment with the case's
// arguments in global memory (it treats the two nodes upstream as well).
template <class ST, int MODEL>
__device__ __noinline__ void batch_special_full(const StepArgs &a, long long node, int rec) {
  step_special_rec<ST, MODEL>(a, node, a.rec[rec]);
}

// One entry (case, node, record, flags) of the boundary-node pass of the
// per-tile batches (FP32, FP16-dev).  The case arguments are assembled in
// registers from the 128-byte BulkArgs of the case's parity and its
// SpecExtra, both read once, so the chain of dependent loads per node is
// entry -> (parity, arguments, record) -> populations, and no argument is
// reloaded after the node's stores.  Nodes of an extrapolating outlet take
// the full path with the arguments in global memory.
template <class ST, int MODEL>
__device__ __forceinline__ void batch_special_entry(const BulkArgs *__restrict__ args,
                                                    const SpecExtra *__restrict__ extra,
                                                    const BatchCase *__restrict__ cases,
                                                    const int4 e, const int *__restrict__ active,
                                                    const int *__restrict__ gpar) {
  if (!__ldg(&active[e.x])) return;
  const int par = __ldg(&gpar[e.x]) & 1;
  const SpecExtra &x = extra[e.x];
  if (x.outlet == 2 && ((uint32_t)e.w & FL_EAST)) {
    batch_special_full<ST, MODEL>(cases[e.x].args[par], (long long)e.y, e.z);
    return;
  }
  StepArgs a;
  spec_args<ST>(args[2 * e.x + par], x, a);
  using R = typename ST::R;
  const long long node = e.y;
  const WRec &w = x.wrec[e.z];
  const AccSideB<ST> acc(a, x.side[par], node, e.z, w.nrec);
  R F[9], mac[3], M[9];
  special_node_rec<R, AccSideB<ST>, false, WRec>(a, acc, node, w, F, mac);
  float *out = x.side[par ^ 1] + (size_t)e.z * 9;
  typename ST::T *d = (typename ST::T *)a.dst;
  if constexpr (ST::SHIFT) {
    collide_dev<MODEL>(F, mac[0], mac[1], mac[2], a, M);
#pragma unroll
    for (int k = 0; k < 9; k++) {
      if ((w.exported >> k) & 1u) st_dev<ST>(d + slot_of<PH_AB>(k, node, a), k, M[k], a);
      out[k] = ST::cvt_dev(ST::pack_dev(M[k], k, a), k, a);
    }
  } else {
    collide<MODEL, R>(F, mac[0], mac[1], mac[2], a, M);
#pragma unroll
    for (int k = 0; k < 9; k++) {
      if ((w.exported >> k) & 1u) ST::st(d + slot_of<PH_AB>(k, node, a), k, M[k], a);
      out[k] = M[k];
    }
  }
}

// Boundary-node pass of the per-tile batches over the whole list.
template <class ST, int MODEL>
__global__ void __launch_bounds__(128) k_batch_special_c(const BulkArgs *__restrict__ args,
                                                         const SpecExtra *__restrict__ extra,
                                                         const BatchCase *__restrict__ cases,
                                                         const int4 *__restrict__ list,
                                                         const int *__restrict__ nlist_live,
                                                         const int *__restrict__ active,
                                                         const int *__restrict__ gpar) {
  const int nlist = __ldg(nlist_live);
  // grid-stride: the host may launch fewer blocks than entries, so that this
  // latency-bound pass holds a few block slots per SM and the bulk pass,
  // launched alongside, keeps the rest
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nlist; i += gridDim.x * blockDim.x)
    batch_special_entry<ST, MODEL>(args, extra, cases, __ldg(&list[i]), active, gpar);
}

// The planes the boundary-node pass did not write (WRec::exported clear),
// from the side arrays of the current parity, for every record of every
// case: run before the du check and the read-back, which read whole states
// from the planes.  One thread per (case, record) entry.
template <class ST>
__global__ void __launch_bounds__(128) k_batch_side_sync(const BulkArgs *__restrict__ args,
                                                         const SpecExtra *__restrict__ extra,
                                                         const int2 *__restrict__ recs, int n,
                                                         const int *__restrict__ gpar) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int2 e = __ldg(&recs[i]);
  const int par = __ldg(&gpar[e.x]) & 1;
  const SpecExtra &x = extra[e.x];
  const WRec &w = x.wrec[e.y];
  const uint32_t todo = ~w.exported & 0x1FFu;
  if (!todo) return;
  StepArgs a;
  spec_args<ST>(args[2 * e.x + par], x, a);
  const long long node = x.rec[e.y].node;
  typename ST::T *p = (typename ST::T *)a.src;  // the state the next step reads
  const float *v = x.side[par] + (size_t)e.y * 9;
#pragma unroll
  for (int k = 0; k < 9; k++) {
    if (!((todo >> k) & 1u)) continue;
    if constexpr (ST::SHIFT) st_dev<ST>(p + slot_of<PH_AB>(k, node, a), k, v[k], a);
    else ST::st(p + slot_of<PH_AB>(k, node, a), k, v[k], a);
  }
}

// Side arrays of buffer 0 after a (re)initialisation of one case: every
// record's nine METAF as the planes hold them.
template <class ST>
__global__ void __launch_bounds__(128) k_batch_side_fill(const StepArgs a, const BRec *rec,
                                                         int nrec, float *side0) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrec) return;
  const AccMain<ST, PH_AB, ST::SHIFT> acc(a, a.src);
  const long long node = rec[i].node;
#pragma unroll
  for (int k = 0; k < 9; k++) side0[(size_t)i * 9 + k] = acc.meta(node, k);
}

// After a step: active cases advance their parity and counters.
static __global__ void k_batch_advance(int ncases, BatchState s) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < ncases && s.active[c]) {
    s.gpar[c]++;
    s.steps[c]++;
  }
}

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// du_rel sums of every active case: one block per tile of 128 positions of
// DU_NPT rows.  The velocity of a node is that of its post-collision METAF (the
// state the next step streams).  Per node and warp the sums are in the
// storage's arithmetic type (FP32 outside FP64 batches), per block in FP64,
// per case in k_batch_converge.
template <class ST>
__global__ void __launch_bounds__(128) k_batch_du(const BatchCase *cases, const int4 *rows,
                                                  int nrows, BatchState s) {
  using R = typename ST::R;
  using T = typename ST::T;
  using A = R;  // per-node and per-warp sums
  __shared__ double sh[2][4];
  const int t = blockIdx.x;
  if (t >= nrows) return;
  const int4 tl = rows[t];
  const int c = tl.x;
  if (!s.active[c]) return;  // uniform per block
  const BatchCase &bc = cases[c];
  const StepArgs &a = bc.args[s.gpar[c] & 1];
  const int x = tl.y * 128 + threadIdx.x, y0 = tl.z * DU_NPT;
  const int n = a.n, m = a.m, pitch = a.pitch;
  const T *src = (const T *)a.src;
  float *up = bc.uprev, *vp = bc.vprev;
  // every load of the DU_NPT rows first (more bytes in flight per thread)
  uint8_t cl[DU_NPT];
  R F[DU_NPT][9];
  float pu[DU_NPT], pv[DU_NPT];
#pragma unroll
  for (int j = 0; j < DU_NPT; j++) {
    const bool in = x < n && y0 + j < m;
    const long long node = (long long)(y0 + j) * pitch + x;
    cl[j] = in ? a.cls[node] : (uint8_t)CLS_SOLID;
    const bool fl = cl[j] != CLS_SOLID;
#pragma unroll
    for (int k = 0; k < 9; k++) F[j][k] = fl ? ld_dev<ST>(src + slot_of<PH_AB>(k, node, a), k, a) : R(0);
    const long long cell = (long long)(y0 + j) * n + x;
    pu[j] = fl ? up[cell] : 0.f;
    pv[j] = fl ? vp[cell] : 0.f;
  }
  A du = A(0), uu = A(0);
  int bad = 0;
#pragma unroll
  for (int j = 0; j < DU_NPT; j++) {
    if (cl[j] == CLS_SOLID) continue;
    // the node's own post-collision METAF: the collision conserves rho and
    // j, so their moments are the macroscopic fields of the step just taken
    R rho, u, v;
    moments_form<ST>(F[j], a, rho, u, v);
    du += ((A)u - (A)pu[j]) * ((A)u - (A)pu[j]) + ((A)v - (A)pv[j]) * ((A)v - (A)pv[j]);
    uu += (A)u * (A)u + (A)v * (A)v;
    const long long cell = (long long)(y0 + j) * n + x;
    up[cell] = (float)u;
    vp[cell] = (float)v;
    bad |= (rho != rho || u != u || v != v);
  }
  if constexpr (sizeof(A) == 8) {
    du = warp_sum(du);
    uu = warp_sum(uu);
  } else {
    du = warp_sum_f(du);
    uu = warp_sum_f(uu);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    sh[0][wid] = (double)du;
    sh[1][wid] = (double)uu;
  }
  const int anybad = __syncthreads_or(bad);
  if (threadIdx.x == 0) {
    s.part[t] = make_double2(sh[0][0] + sh[0][1] + sh[0][2] + sh[0][3],
                             sh[1][0] + sh[1][1] + sh[1][2] + sh[1][3]);
    if (anybad) s.bad[c] = 1;
  }
}

// Per-case convergence decision after k_batch_du, one warp per case summing
// its row tiles' partial sums in a fixed order (the result does not depend on
// block scheduling).  du_rel is the relative change per step:
// ||(u,v) - (u,v)_prev|| / ||(u,v)|| over the check interval, times
// inv_span = 1 / (steps in the interval).
static __global__ void k_batch_converge(int ncases, BatchState s, double tol, double inv_span) {
  const int c = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (c >= ncases || !s.active[c]) return;  // uniform per warp
  double a0 = 0.0, a1 = 0.0;
  for (int r = s.rbeg[c] + lane; r < s.rbeg[c + 1]; r += 32) {
    const double2 q = s.part[r];
    a0 += q.x;
    a1 += q.y;
  }
  a0 = warp_sum(a0);
  a1 = warp_sum(a1);
  if (lane != 0) return;
  const double du = a1 > 0 ? sqrt(a0 / a1) * inv_span : INFINITY;
  s.du_last[c] = s.have_prev[c] ? du : INFINITY;
  if (s.bad[c]) {
    s.active[c] = 0;  // diverged: frozen, reported by the host
  } else if (s.have_prev[c] && du <= tol) {
    s.active[c] = 0;
    s.conv_at[c] = s.steps[c];
  }
  s.have_prev[c] = 1;
}

struct BatchKernels {
  const void *step[4][BVAR];  // [model 1..3][tile shape]
  int per_tile;               // 1: step kernels take BulkArgs and one block per tile
                              // (k_batch_bulk); 0: BatchCase and a persistent grid
  const void *special[4];     // [model 1..3]: k_batch_special (persistent kinds) or
                              // k_batch_special_c (per-tile kinds)
  const void *side_fill;      // k_batch_side_fill (per-tile kinds)
  const void *side_sync;      // k_batch_side_sync (per-tile kinds)
  const void *du;
  const void *advance;
  const void *converge;
  const void *compact_tiles;    // k_batch_compact<int4>
};

}  // namespace lbm
