/*
 * TEST INFRASTRUCTURE ONLY -- never part of the product.
 *
 * Step-level driver around the UNMODIFIED serial reference solver
 * (mate-szoke/ParallelLbmCranfield, serial/).  oracle/Makefile compiles the
 * reference's own .c files from where they lie and links them with this file
 * into oracle/_ref/libserialref.so.  The tests use it to pin the C
 * restatement in lbm_oracle.c and to write the golden fixtures under
 * tests/golden/.
 *
 * Call sequence follows serial/Iterate.c:
 *   mesh read     ReadNodes/ReadBCconn         serial/Iterate.c:98-101
 *   mesh data     CompDataNode/CompDataConn    serial/Iterate.c:107-110
 *   constants     D2Q9Vars, Omega, OmegaA, MRT serial/Iterate.c:176-188
 *   cell init     CellIni (O(N^2))             serial/Iterate.c:204-228
 *   one step      Collision, UpdateF, Streaming, Boundaries, Macroscopic,
 *                 ComputeResiduals             serial/Iterate.c:268-300
 *
 * Deviation from serial/Iterate.c (stated, see Q9 below): CompDataConn is
 * defined with float* arguments (serial/FileIO.c:218-219) but Iteration()
 * passes double* (serial/Iterate.c:109-110), which corrupts the inlet extent.
 * This driver passes real floats, as the definition expects, and widens them.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

#include "ShellFunctions.h"
#include "Iterate.h"
#include "CellFunctions.h"
#include "ComputeResiduals.h"

/* Prototypes exactly as defined in serial/FileIO.c:14, 91, 183, 218. */
float **ReadNodes(char *NodeDataFile, int *NumOfLines);
float **ReadBCconn(char *BCconnectorDataFile, int *NumOfLines);
void CompDataNode(MyReal *Delta, int *m, int *n, float **Nodes, int *NumNodes);
void CompDataConn(int *NumInletNodes, float *MaxInletCoordY, float *MinInletCoordY,
                  float **BCconn, int *NumConn, MyReal *Delta);

typedef struct RefSim {
  int n, m;
  int model, curved, outlet, drag_id;
  MyReal w[9];
  int c[9], cx[9], cy[9], opp[9];
  MyReal omega, omegaA;
  MyReal **tm, **stmiv;
  MyReal delta, min_inlet_y, max_inlet_y;
  struct CellProps *cells;
} RefSim;

static int has_inlet(float **conn, int nconn) {
  for (int i = 0; i < nconn; i++)
    if (conn[i][3] == 2) return 1;
  return 0;
}

RefSim *ref_create(const char *nodefile, const char *connfile, float Uavg, float Vavg,
                   float rho_ini, float viscosity, int inlet_profile, int model,
                   int curved, int outlet, int drag_id) {
  int NumNodes = 0, NumConn = 0;
  float **nodes = ReadNodes((char *)nodefile, &NumNodes);
  float **conn = ReadBCconn((char *)connfile, &NumConn);
  if (!nodes || !conn) return NULL;
  RefSim *s = (RefSim *)calloc(1, sizeof(RefSim));
  s->model = model; s->curved = curved; s->outlet = outlet; s->drag_id = drag_id;
  CompDataNode(&s->delta, &s->m, &s->n, nodes, &NumNodes);
  float fmax = 0.f, fmin = 0.f;
  int ninlet = 0;
  if (has_inlet(conn, NumConn))
    CompDataConn(&ninlet, &fmax, &fmin, conn, &NumConn, &s->delta);
  s->max_inlet_y = fmax;
  s->min_inlet_y = fmin;
  D2Q9Vars(s->w, s->cx, s->cy, s->opp, s->c, &s->n);
  s->omega = 1.0 / (3. * viscosity + 0.5);
  s->omegaA = 8 * (2 - s->omega) / (8 - s->omega);
  s->tm = Create2DArrayMyReal(9, 9);
  s->stmiv = Create2DArrayMyReal(9, 9);
  if (model == 3) MRTInitializer(s->tm, s->stmiv, s->omega);
  s->cells = (struct CellProps *)calloc((size_t)s->n * s->m, sizeof(struct CellProps));
  for (int j = 0; j < s->m; j++)
    for (int i = 0; i < s->n; i++)
      CellIni(nodes, conn, &NumNodes, &NumConn, i, j, &s->min_inlet_y, &s->max_inlet_y,
              &s->delta, Uavg, Vavg, inlet_profile, model, s->opp, s->cells, rho_ini, &s->n);
  for (int i = 0; i < NumNodes; i++) free(nodes[i]);
  for (int i = 0; i < NumConn; i++) free(conn[i]);
  free(nodes);
  free(conn);
  return s;
}

void ref_dims(const RefSim *s, int *n, int *m) { *n = s->n; *m = s->m; }

void ref_constants(const RefSim *s, double *out /* omega, omegaA, delta, min_y, max_y */) {
  out[0] = s->omega; out[1] = s->omegaA; out[2] = s->delta;
  out[3] = s->min_inlet_y; out[4] = s->max_inlet_y;
}

/* Overwrite F (9 per cell, cell-major, may be NULL) and the macroscopic fields. */
void ref_set_state(RefSim *s, const double *F, const double *rho, const double *u,
                   const double *v) {
  size_t N = (size_t)s->n * s->m;
  for (size_t i = 0; i < N; i++) {
    struct CellProps *c = s->cells + i;
    if (F) for (int k = 0; k < 9; k++) c->F[k] = F[i * 9 + k];
    if (rho) c->Rho = rho[i];
    if (u) c->U = u[i];
    if (v) c->V = v[i];
  }
}

/* nsteps iterations of the loop body of serial/Iterate.c:263-307. */
void ref_run(RefSim *s, int nsteps, double *resid /* 4 per step or NULL */) {
  double R[4];
  int N = s->n * s->m;
  for (int it = 0; it < nsteps; it++) {
    CollisionStep(s->cells, &s->m, &s->n, s->w, s->cx, s->cy, s->opp, s->omega, s->omegaA,
                  s->tm, s->stmiv, s->model);
    for (int i = 0; i < N; i++) UpdateF(s->cells, i);
    StreamingStep(s->cells, &s->m, &s->n, s->c);
    HandleBoundariesStep(s->cells, s->cx, s->cy, s->c, s->opp, s->outlet, s->curved, &s->n,
                         &s->m);
    UpdateMacroscopicStep(s->cells, &s->m, &s->n, s->cx, s->cy, s->drag_id);
    ComputeResiduals(s->cells, R, &s->m, &s->n, s->drag_id);
    if (resid) memcpy(resid + 4 * it, R, sizeof R);
  }
}

/* Copy out per-cell state; any pointer may be NULL.  F/METAF are cell-major. */
void ref_get(const RefSim *s, double *F, double *METAF, double *rho, double *u, double *v,
             double *drag, double *lift) {
  size_t N = (size_t)s->n * s->m;
  for (size_t i = 0; i < N; i++) {
    const struct CellProps *c = s->cells + i;
    if (F) for (int k = 0; k < 9; k++) F[i * 9 + k] = c->F[k];
    if (METAF) for (int k = 0; k < 9; k++) METAF[i * 9 + k] = c->METAF[k];
    if (rho) rho[i] = c->Rho;
    if (u) u[i] = c->U;
    if (v) v[i] = c->V;
    if (drag) drag[i] = c->DragF;
    if (lift) lift[i] = c->LiftF;
  }
}

/* Per-cell preprocessing result of CellIni, for checking the O(N) restatement.
 * ints: Fluid, Corner, Boundary, BoundaryID, ID, StreamLattice[9], BC_ID[9] (23 per cell)
 * reals: Q[9], CoordX, CoordY, Uo, Vo, U (14 per cell) */
void ref_get_init(const RefSim *s, int *ints, double *reals) {
  size_t N = (size_t)s->n * s->m;
  for (size_t i = 0; i < N; i++) {
    const struct CellProps *c = s->cells + i;
    int *o = ints + i * 23;
    o[0] = c->Fluid; o[1] = c->Corner; o[2] = c->Boundary; o[3] = c->BoundaryID; o[4] = c->ID;
    for (int k = 0; k < 9; k++) { o[5 + k] = c->StreamLattice[k]; o[14 + k] = c->BC_ID[k]; }
    double *r = reals + i * 14;
    for (int k = 0; k < 9; k++) r[k] = c->Q[k];
    r[9] = c->CoordX; r[10] = c->CoordY; r[11] = c->Uo; r[12] = c->Vo; r[13] = c->U;
  }
}

int ref_sizeof_cell(void) { return (int)sizeof(struct CellProps); }

void ref_destroy(RefSim *s) {
  if (!s) return;
  for (int i = 0; i < 9; i++) { free(s->tm[i]); free(s->stmiv[i]); }
  free(s->tm);
  free(s->stmiv);
  free(s->cells);
  free(s);
}
