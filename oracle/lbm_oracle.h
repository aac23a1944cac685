/*
 * TEST INFRASTRUCTURE ONLY -- the CPU oracle for the D2Q9 time step.
 *
 * A C restatement of the serial reference solver's per-step update
 * (mate-szoke/ParallelLbmCranfield serial/Iterate.c:263-332 and its callees
 * in serial/CellFunctions.c, serial/BoundaryConditions.c and
 * serial/ComputeResiduals.c), including its quirks, plus the two boundary
 * conditions the reference does not have (constant-pressure outlet,
 * momentum-exchange forces).  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline legs of bench.py may load it; the product never does.
 *
 * Pinning: on this machine the restatement is checked bit-for-bit against
 * the unmodified reference compiled into oracle/_ref/libserialref.so, and
 * both are pinned by the golden fixtures in tests/golden/.
 */
#ifndef LBM_ORACLE_H
#define LBM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_params {
  float uavg, vavg, rho_ini, viscosity; /* ini values are parsed as float (serial/FileIO.c:272-275) */
  int inlet_profile;                    /* 1 parabolic, 2 uniform Uavg */
  int model;                            /* 1 BGKW, 2 TRT, 3 MRT */
  int curved;                           /* 1 curved (Bouzidi), 2 straight bounce-back */
  int outlet;                           /* 1 Zou-He velocity, 2 2nd-order extrapolation,
                                           3 no-op (as serial), 4 constant pressure (new) */
  int drag_id;                          /* CalculateDragLift */
  double rho_out;                       /* pressure outlet density (outlet == 4) */
} or_params;

typedef struct or_sim or_sim;

/* Mesh files in the reference format, parsed with fscanf("%f") like serial/FileIO.c:56-74. */
int or_read_mesh(const char *nodefile, const char *connfile, float **nodes, int *nnodes,
                 float **conns, int *nconn);
void or_free(void *p);

/* nodes: nnodes x 5 floats; conns: nconn x 7 floats (row-major). */
or_sim *or_create(const float *nodes, int nnodes, const float *conns, int nconn,
                  const or_params *p);
void or_destroy(or_sim *s);
void or_dims(const or_sim *s, int *n, int *m);
void or_constants(const or_sim *s, double *out /* omega, omegaA, delta, min_y, max_y */);
void or_get_init(const or_sim *s, int *ints /* 23 per cell */, double *reals /* 14 per cell */);

/* F cell-major (9 per cell) or NULL; macroscopic fields or NULL. */
void or_set_state(or_sim *s, const double *F, const double *rho, const double *u,
                  const double *v);
/* nsteps serial iterations; resid gets 4 doubles per step (L2, L2_weighted, drag, lift). */
int or_run(or_sim *s, int nsteps, double *resid);
void or_get(const or_sim *s, double *F, double *METAF, double *rho, double *u, double *v,
            double *drag, double *lift);

/* Diagnostics the reference does not compute (all FP64, fluid cells only):
 * out[0] full-field ||F - METAF||_2, out[1] mass sum(rho), out[2] sum(rho u), out[3] sum(rho v),
 * out[4], out[5] momentum-exchange force (x, y) on links whose connector carries drag_id. */
void or_diagnostics(const or_sim *s, double *out);

int or_sizeof_cell(void);

#ifdef __cplusplus
}
#endif
#endif
