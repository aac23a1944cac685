/*
 * lbm_gb300.h -- C ABI of the GB300-native D2Q9 lattice-Boltzmann time step.
 *
 * Drop-in for the time loop of the serial solver of
 * mate-szoke/ParallelLbmCranfield.  One context owns one domain resident on
 * one GPU; the caller owns every host buffer.  No C++ types and no
 * exceptions cross this boundary; every entry point returns an lbm_status.
 *
 * Reference interfaces replaced (file:line in the reference project):
 *   lbm_create        CellIni + D2Q9Vars + MRTInitializer + the calloc of the
 *                     cell array          serial/Iterate.c:176-228,
 *                                         serial/include/CellFunctions.h:8-15
 *   lbm_set_state     the initial F / U / V / Rho of the cells
 *                                         serial/CellFunctions.c:147-150,252-267
 *   lbm_step          one loop body per step: CollisionStep, UpdateF,
 *                     StreamingStep, HandleBoundariesStep,
 *                     UpdateMacroscopicStep, ComputeResiduals
 *                                         serial/Iterate.c:263-307,
 *                                         serial/include/Iterate.h:8-19,
 *                                         serial/include/ComputeResiduals.h:6-7
 *   lbm_get_fields    reads of Cells[i].Rho/U/V/F/METAF by the writers
 *                                         serial/FileIO.c:298-427
 *   lbm_destroy       free(Cells)         serial/Iterate.c:407
 *   status codes      0 ok / 1 diverged / 2 file error of
 *                                         cuda/cuda_step3/include/Iterate.h:59-64
 */
#ifndef LBM_GB300_H
#define LBM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum lbm_status {
  LBM_OK = 0,
  LBM_DIVERGED = 1, /* NaN met by a residual/diagnostic (serial/ComputeResiduals.c:47-51) */
  LBM_IO = 2,       /* file could not be read or written */
  LBM_CUDA = 3,     /* a CUDA runtime call failed */
  LBM_TIMEOUT = 4,  /* a bounded device wait gave up */
  LBM_INVALID = 5,  /* bad argument or unsupported mesh */
  LBM_NOMEM = 6     /* device or host allocation failed */
} lbm_status;

typedef enum lbm_precision {
  LBM_FP64 = 0,    /* FP64 storage and arithmetic in the reference's order (parity mode) */
  LBM_FP32 = 1,    /* FP32 storage and arithmetic */
  LBM_FP16DEV = 2, /* FP16 storage of scaled (f_k - w_k rho0), FP32 arithmetic */
  LBM_BF16DEV = 3, /* BF16 storage of scaled (f_k - w_k rho0), FP32 arithmetic */
  LBM_FP16NEQ = 4  /* moment storage, A-B pattern only: rho - rho0 and j in 24-bit fixed
                      point (|rho - rho0| < 0.5 rho0, |j| < 0.25 rho0, else LBM_DIVERGED), the six
                      non-equilibrium moments in FP16, nodes with boundary work in FP32;
                      21 bytes per node, FP32 arithmetic */
} lbm_precision;

typedef enum lbm_pattern {
  LBM_AB = 0, /* two population buffers, pull streaming */
  LBM_AA = 1  /* one population buffer, in-place AA streaming */
} lbm_pattern;

/* Mesh in the reference's file format, already parsed:
 *   nodes: num_nodes x 5 floats  (i, j, x, y, fluid)            Mesh/D2node.dat
 *   conns: num_conns x 7 floats  (i, j, dir, type, x, y, id)    Mesh/BCconnectors.dat
 * (serial/FileIO.c:39-44 and :116-133). */
typedef struct lbm_mesh {
  const float *nodes;
  int32_t num_nodes;
  const float *conns;
  int32_t num_conns;
} lbm_mesh;

/* The SetUpData.ini switches of the time step (serial/FileIO.c:263-289) plus
 * the GB300 storage choices. */
typedef struct lbm_params {
  float uavg, vavg, rho_ini, viscosity; /* ini lines 1-4 (parsed as float) */
  int32_t inlet_profile;     /* 1 parabolic, 2 uniform Uavg */
  int32_t collision_model;   /* 1 BGKW, 2 TRT, 3 MRT */
  int32_t curved_boundaries; /* 1 curved (Bouzidi), 2 bounce-back of the streamed-in value */
  int32_t outlet_profile;    /* 1 Zou-He velocity, 2 2nd-order extrapolation,
                                3 none (as the serial code), 4 constant pressure rho_out */
  int32_t drag_lift_id;      /* CalculateDragLift: boundary ID of the force surface, 0 = none */
  int32_t precision;         /* lbm_precision */
  int32_t pattern;           /* lbm_pattern */
  int32_t device;            /* CUDA device ordinal */
  double rho_out;            /* outlet density for outlet_profile 4 */
  void *stream;              /* cudaStream_t to run on; NULL = a stream owned by the context */
  int32_t tile_variant;      /* fused-step tile: 0 = default or lbm_autotune's choice, 1..6 fixed
                                (1..4 for LBM_FP16NEQ) */
} lbm_params;

typedef struct lbm_ctx lbm_ctx;

/* Full-field diagnostics (FP64 reductions on the GPU), none of which the
 * serial code computes correctly (its residual only visits cells 0..m-1). */
typedef struct lbm_diagnostics {
  int64_t iteration;   /* completed iterations */
  double l2_full;      /* ||F - METAF||_2 over fluid cells (the CUDA/UPC variants' residual) */
  double du_rel;       /* relative change per step: ||(u,v) - (u,v)_prev|| / ||(u,v)|| since
                          the previous lbm_check, divided by the iterations in between */
  double mass;         /* sum rho over fluid cells */
  double momentum[2];  /* sum rho u, sum rho v */
  double force[2];     /* momentum-exchange force on wall links of drag_lift_id cells */
  double max_speed;    /* max |u| over fluid cells */
} lbm_diagnostics;

/* Library / status helpers. */
const char *lbm_status_string(lbm_status s);
/* Text of the last error seen by this thread, or "" */
const char *lbm_last_error(void);

lbm_status lbm_create(const lbm_mesh *mesh, const lbm_params *params, lbm_ctx **out);
void lbm_destroy(lbm_ctx *ctx);
/* Grid size n (x) and m (y) as CompDataNode derives them (serial/FileIO.c:193-194). */
lbm_status lbm_get_dims(const lbm_ctx *ctx, int32_t *n, int32_t *m);

/* State at the current iteration.  Arrays are cell-major, cells row-major
 * (j * n + i), length n*m (f: 9*n*m).  f == NULL sets f = f_eq(rho, u, v);
 * rho/u/v == NULL keep the values CellIni gave (rho_ini, Uo, 0).  The next
 * collision uses rho/u/v as given, like the reference's first step. */
lbm_status lbm_set_state(lbm_ctx *ctx, const double *f, const double *rho, const double *u,
                         const double *v);

/* Advance nsteps iterations.  For every step s (1-based within this call)
 * with check_every > 0 and s % check_every == 0, 4 doubles are appended to
 * residuals (may be NULL): the reference's L2_norm, L2_norm_weighted, Drag,
 * Lift (serial/ComputeResiduals.c:6-51, including its index quirk).  The
 * buffer must hold 4 * (nsteps / check_every) doubles.  Returns LBM_DIVERGED
 * if any reported residual is NaN (serial/ComputeResiduals.c:47-51) and, for
 * FP32 and 16-bit storage, also when any node's collision met a NaN or an
 * infinity during these steps, whatever check_every is (the reference's
 * residual cannot see most nodes; FP64 keeps its report).  The state is then
 * lost: lbm_set_state starts again. */
lbm_status lbm_step(lbm_ctx *ctx, int32_t nsteps, int32_t check_every, double *residuals);

/* Fields after the last completed iteration; any pointer may be NULL.
 * f and metaf are cell-major 9 per cell (F and METAF of the reference cells). */
lbm_status lbm_get_fields(lbm_ctx *ctx, double *rho, double *u, double *v, double *f,
                          double *metaf);

/* Full-field FP64 diagnostics of the current state; also advances the
 * du_rel reference fields.  LBM_DIVERGED if any sum is NaN. */
lbm_status lbm_check(lbm_ctx *ctx, lbm_diagnostics *out);

/* lbm_check without any device allocation, for callers that cannot call
 * cudaMalloc when they want the diagnostics (a host that gives all device
 * memory to its own pool, a loop that must not allocate between steps).
 * No counterpart in the reference, whose residual needs no device memory.
 * Same sums as lbm_check except du_rel (returned as NaN: it needs per-cell
 * reference fields).  Uses one fixed 5 MiB device array inside the library
 * (65536 reduction blocks), held on every GPU that loads it until exit.  It
 * reduces on lbm_check's grid (one block column per 128 grid columns, at most
 * 8192 blocks where the width allows), so only domains wider than 65536 x 128
 * (about 8.4 M) grid columns get LBM_INVALID.  Calls share that array:
 * calls whose kernels overlap on the GPU (other streams or host threads)
 * race; serialise them.
 * The first call on a device looks up the array's address; make it before
 * any stream capture. */
lbm_status lbm_check_noalloc(lbm_ctx *ctx, lbm_diagnostics *out);

/* Autotuner (no counterpart in the reference): times every tile variant of
 * the fused step (threads along x, rows per thread) on this context's domain
 * (the median of three runs of steps_per_trial steps each, after two
 * untimed steps) and keeps the fastest.  Must run before lbm_set_state: it steps a scratch
 * state at rest and discards it.  cache_path (NULL = none) is a file of JSON
 * lines keyed by GPU, storage, pattern, model and grid size: a hit skips the
 * timing, a miss appends the result.  report (NULL = none) receives the
 * JSON line. */
lbm_status lbm_autotune(lbm_ctx *ctx, int32_t steps_per_trial, const char *cache_path,
                        char *report, size_t report_cap);

/* Completed iterations, device bytes held, bytes moved per node per step. */
lbm_status lbm_get_info(const lbm_ctx *ctx, int64_t *iteration, int64_t *device_bytes,
                        int32_t *bytes_per_node_step);

/* Host-only view of the preprocessing lbm_create performs (no GPU needed).
 * Per cell (row-major j*n+i, arrays of n*m, any pointer may be NULL):
 *   cls:   0 solid, 1 fluid without boundary work, 3 fluid with boundary work
 *   flags: for class-3 cells, bit k (0..8) = StreamLattice[k], bit 9+k =
 *          (BC_ID[k] == 1), bit 18 lid inlet, bit 19 west inlet, bit 20
 *          BC_ID[1] == 3, bit 21 BoundaryID == drag_lift_id; 0 otherwise
 *   q:     Q[k] of class-3 cells (9 per cell), 0.5 elsewhere
 * These are the decisions of CellIni (serial/CellFunctions.c:99-270). */
lbm_status lbm_inspect_mesh(const lbm_mesh *mesh, const lbm_params *params, int32_t *n,
                            int32_t *m, uint8_t *cls, uint32_t *flags, double *q);

/* ---------------------------------------------------------------------------
 * Batches.  No counterpart in the reference, which runs one case per process:
 * many independent domains (cavities, channels of different sizes and
 * parameters) advanced together: per step one launch over a device-side
 * list of (case, tile), and alongside it one over the (case, node)
 * list of boundary nodes (sorted by boundary kind); the tile list is compacted
 * to the cases still stepping at the start of every run segment.  Per-case convergence flags live on the
 * device; each run segment (check_every steps and one check) is one CUDA graph
 * replay.  All cases share precision (FP64, FP32 or FP16-dev), the A-B pattern,
 * the collision model and the device; everything else is per case.
 * ------------------------------------------------------------------------ */
typedef struct lbm_batch lbm_batch;
lbm_status lbm_batch_create(const lbm_mesh *meshes, const lbm_params *params, int32_t ncases,
                            lbm_batch **out);
void lbm_batch_destroy(lbm_batch *b);
/* Every case at rest: f = f_eq(rho_ini, 0, 0), then its first collision. */
lbm_status lbm_batch_set_rest(lbm_batch *b);
/* Case c restarts from f = f_eq(rho, u, v) (arrays of that case's n*m
 * cells); its counters and convergence state are reset. */
lbm_status lbm_batch_set_state(lbm_batch *b, int32_t case_index, const double *rho,
                               const double *u, const double *v);
/* Fixes the batched step's tile shape (0..3: 128x1, 64x4, 128x2, 128x4 threads x rows). */
lbm_status lbm_batch_set_tile(lbm_batch *b, int32_t tile_variant);
/* Fixes the launch options of FP32 / FP16-dev batches that lbm_batch_autotune
 * otherwise picks: the boundary-node pass's grid (0 = one thread per list
 * entry, k = k blocks per multiprocessor walking the list) and the bulk
 * pass's L2 prefetch of the tile a quarter of a wave of blocks ahead (0 or
 * 1).  The results do not depend on either.  No counterpart in the
 * reference (its loop steps one domain). */
lbm_status lbm_batch_set_launch(lbm_batch *b, int32_t special_blocks_per_sm, int32_t bulk_prefetch);
/* Times the batched step's tile shapes and keeps the fastest (before stepping);
 * for FP32 and FP16-dev batches then also the boundary-node pass's blocks per
 * multiprocessor (one thread per entry, or a grid of 2, 4 or 8 blocks per SM
 * that leaves block slots to the bulk pass running alongside), then the bulk
 * pass's L2 prefetch.  The report is JSON: {"variant", "ms",
 * "special_blocks_per_sm", "special_ms", "bulk_prefetch", "prefetch_ms"}. */
lbm_status lbm_batch_autotune(lbm_batch *b, int32_t steps_per_trial, char *report,
                              size_t report_cap);
/* Steps every unconverged case until all have converged or max_steps have run
 * (max_steps is rounded up to a multiple of check_every: the run advances in
 * whole segments of check_every steps and one check).
 * Every check_every steps each active case gets the relative change per step
 * du_rel = ||(u,v) - (u,v)_prev|| / (check_every ||(u,v)||) against the previous
 * check (FP64 sums), so tol does not depend on check_every; a case with du_rel <= tol
 * stops stepping.  Per case (any pointer may be NULL): fused steps run (the
 * completed iterations are one more), the last du_rel, converged (1 yes, 0 no,
 * -1 NaN seen); seconds = wall time of the loop.  LBM_DIVERGED if a case saw NaN. */
lbm_status lbm_batch_run(lbm_batch *b, int64_t max_steps, int32_t check_every, double tol,
                         int64_t *steps, double *du_rel, int32_t *converged, double *seconds);
lbm_status lbm_batch_get_fields(lbm_batch *b, int32_t case_index, double *rho, double *u,
                                double *v);
lbm_status lbm_batch_dims(const lbm_batch *b, int32_t case_index, int32_t *n, int32_t *m);
lbm_status lbm_batch_info(const lbm_batch *b, int64_t *nodes, int64_t *fluid_nodes,
                          int32_t *tile_variant, int64_t *device_bytes);

/* ---------------------------------------------------------------------------
 * Surrogate network for warm starts (no counterpart in the reference): a
 * 4-level convolutional encoder-decoder with skip connections (channels base,
 * 2 base, 4 base, 4 base; 3x3 convolutions, ReLU, 2x2 average pooling,
 * nearest upsampling, a 1x1 output layer) from in_channels input maps to
 * out_channels output maps on a height x width grid.  BF16 weights and
 * activations, FP32 accumulation on the tensor cores, FP32 master weights
 * trained with Adam; all kernels are this library's own.  Tensors are NHWC
 * FP32 on the host: x[b][y][x][c].  Parameters: for each of the 15 layers in
 * forward order W[cout][Kp] (Kp = taps*cin rounded up to 32, k = tap*cin + ci,
 * zero padding) followed by b[cout].
 * ------------------------------------------------------------------------ */
typedef struct lbm_sg lbm_sg;
typedef struct lbm_sg_config {
  int32_t height, width;   /* multiples of 8, >= 16 */
  int32_t in_channels, out_channels;  /* out_channels <= 8 or a multiple of 8 (<= 64) */
  int32_t base;            /* channels of the first level (multiple of 8) */
  int32_t max_batch;
  float lr, beta1, beta2, eps;  /* Adam */
  uint64_t seed;           /* weight initialisation */
  int32_t device;
  float weight_decay;      /* decoupled (AdamW) decay per unit learning rate; 0 = Adam */
  float coarse_weight;     /* weight of the block-mean loss term (0 = off): the masked means of
                              output and target over coarse_block^2 cells are compared too */
  int32_t coarse_block;    /* divides height and width */
  int32_t products;        /* 0: convolution products on tcgen05 (tensor-memory accumulators)
                              where the shapes allow, 3x3 layers with W a multiple of 128 and C a
                              multiple of 32 in the TMA-fed halo-tile form (several row segments
                              per block where H is a multiple of 4); 1: every product on the
                              mma.sync kernels; 2: tcgen05 with the im2col gather only; 3: as 0
                              with one row segment per halo-tile convolution block */
} lbm_sg_config;
lbm_status lbm_sg_create(const lbm_sg_config *cfg, lbm_sg **out);
void lbm_sg_destroy(lbm_sg *s);
lbm_status lbm_sg_num_params(const lbm_sg *s, int64_t *n);
lbm_status lbm_sg_get_params(lbm_sg *s, float *out);
lbm_status lbm_sg_set_params(lbm_sg *s, const float *in);
/* y[batch][H][W][out] = net(x[batch][H][W][in]) */
lbm_status lbm_sg_forward(lbm_sg *s, int32_t batch, const float *x, float *y);
/* Masked mean-squared-error loss and its gradient (no update): loss = sum over
 * cells and outputs of mask * (y - target)^2 / (sum mask * out_channels), plus
 * coarse_weight * the mean over blocks with mask and outputs of (block mean of y -
 * block mean of target)^2 when coarse_weight > 0;
 * mask NULL = all ones; grads (NULL = not copied) receives num_params floats. */
lbm_status lbm_sg_loss_grads(lbm_sg *s, int32_t batch, const float *x, const float *target,
                             const float *mask, double *loss, float *grads);
/* Learning rate of the following Adam updates (schedules). */
lbm_status lbm_sg_set_lr(lbm_sg *s, float lr);
/* One Adam update from the gradients of the last lbm_sg_loss_grads. */
lbm_status lbm_sg_adam_step(lbm_sg *s);
/* Keeps count samples (x, target, mask) on the device for lbm_sg_train. */
lbm_status lbm_sg_set_dataset(lbm_sg *s, int32_t count, const float *x, const float *y,
                              const float *mask);
/* Adam steps over order[0..n) in batches (a trailing partial batch is
 * dropped); mean_loss = mean batch loss. */
lbm_status lbm_sg_train(lbm_sg *s, int32_t batch, const int32_t *order, int32_t n,
                        double *mean_loss);

/* ---------------------------------------------------------------------------
 * Mesh helpers (the reference's readers, serial/FileIO.c:14-289, and a
 * generator for meshes in the same format).  Buffers returned in lbm_mesh are
 * owned by the library and released with lbm_mesh_free.
 * ------------------------------------------------------------------------ */
lbm_status lbm_mesh_read(const char *node_file, const char *conn_file, lbm_mesh *out);
/* Lid-driven square cavity with the layout of the shipped cases: fluid cells
 * i,j in [1, side], solid ring, an extra solid row on top, unit square,
 * lid (type 2, ID 2) on top, walls left=1, right=3, bottom=4 (type 1). */
lbm_status lbm_mesh_cavity(int32_t side, lbm_mesh *out);
/* Channel nx by ny fluid cells: west inlet (type 2, ID 1), east outlet
 * (type 3, ID 3), walls top=2 / bottom=4, and ncyl circles (type 1, ID 5)
 * with centres (cx, cy) and radius r in lattice units of the fluid-cell grid. */
lbm_status lbm_mesh_channel(int32_t nx, int32_t ny, int32_t ncyl, const double *cx,
                            const double *cy, const double *r, lbm_mesh *out);
lbm_status lbm_mesh_write(const lbm_mesh *mesh, const char *node_file, const char *conn_file);
void lbm_mesh_free(lbm_mesh *mesh);

#ifdef __cplusplus
}
#endif
#endif /* LBM_GB300_H */
