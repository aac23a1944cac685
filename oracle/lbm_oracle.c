/*
 * TEST INFRASTRUCTURE ONLY -- CPU oracle for the D2Q9 time step (see lbm_oracle.h).
 *
 * The cell record keeps the reference's array-of-structures layout
 * (serial/include/ShellFunctions.h:14-37, 528 bytes per node) and the step is
 * the same five full-grid sweeps, so that timing this file is a faithful
 * stand-in for the serial reference on hosts where the reference itself is
 * not built.  Arithmetic is written in the reference's order and association;
 * compile with -ffp-contract=off so that no FMA changes a rounding.
 */
#include "lbm_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct or_cell {
  int fluid, corner, stream[9], id, boundary, boundary_id, bc_id[9];
  double q[9], coordx, coordy, u, v, rho, uo, vo, drag, lift;
  double F[9], Feq[9], METAF[9], Fnb[9];
} or_cell;

struct or_sim {
  int n, m;
  or_params p;
  double omega, omegaA, delta, min_y, max_y;
  double stmiv[9][9];
  or_cell *cells;
};

/* D2Q9 lattice of serial/CellFunctions.c:277-342. */
static const int CX[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
static const int CY[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
static const int OPP[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};
static double W[9];

/* MRT transform of serial/CellFunctions.c:37-47 (integer entries). */
static const int TM[9][9] = {
    {1, 1, 1, 1, 1, 1, 1, 1, 1},     {-4, -1, -1, -1, -1, 2, 2, 2, 2},
    {4, -2, -2, -2, -2, 1, 1, 1, 1}, {0, 1, 0, -1, 0, 1, -1, -1, 1},
    {0, -2, 0, 2, 0, 1, -1, -1, 1},  {0, 0, 1, 0, -1, 1, 1, -1, -1},
    {0, 0, -2, 0, 2, 1, 1, -1, -1},  {0, 1, -1, 1, -1, 0, 0, 0, 0},
    {0, 0, 0, 0, 0, 1, -1, 1, -1}};
/* Its inverse in units of 1/36 (serial/CellFunctions.c:24-35). */
static const int TMINV36[9][9] = {
    {4, -4, 4, 0, 0, 0, 0, 0, 0},   {4, -1, -2, 6, -6, 0, 0, 9, 0},
    {4, -1, -2, 0, 0, 6, -6, -9, 0}, {4, -1, -2, -6, 6, 0, 0, 9, 0},
    {4, -1, -2, 0, 0, -6, 6, -9, 0}, {4, 2, 1, 6, 3, 6, 3, 0, 9},
    {4, 2, 1, -6, -3, 6, 3, 0, -9},  {4, 2, 1, -6, -3, -6, -3, 0, 9},
    {4, 2, 1, 6, 3, -6, -3, 0, -9}};

static void lattice_init(void) {
  W[0] = 4. / 9.;
  for (int i = 1; i < 5; i++) W[i] = 1. / 9.;
  for (int i = 5; i < 9; i++) W[i] = 1. / 36.;
}

void or_free(void *p) { free(p); }
int or_sizeof_cell(void) { return (int)sizeof(or_cell); }

/* ---------------------------------------------------------------- mesh input */

/* serial/FileIO.c:14-82 and :91-174: count the records, then read them as floats. */
static float *read_table(const char *path, int ncol, int *nrows, int is_nodes) {
  FILE *f = fopen(path, "r");
  if (!f) return NULL;
  int rows = 0;
  if (is_nodes) {
    int a, b, c;
    float x, y;
    while (fscanf(f, "%d %d %f %f %d", &a, &b, &x, &y, &c) == 5) rows++;
  } else {
    int a, b, c, d, e;
    float x, y;
    while (fscanf(f, "%d %d %d %d %f %f %d", &a, &b, &c, &d, &x, &y, &e) == 7) rows++;
  }
  rewind(f);
  float *t = (float *)calloc((size_t)(rows > 0 ? rows : 1) * ncol, sizeof(float));
  for (int r = 0; r < rows; r++)
    for (int c = 0; c < ncol; c++)
      if (fscanf(f, "%f", &t[(size_t)r * ncol + c]) != 1) t[(size_t)r * ncol + c] = 0.f;
  fclose(f);
  *nrows = rows;
  return t;
}

int or_read_mesh(const char *nodefile, const char *connfile, float **nodes, int *nnodes,
                 float **conns, int *nconn) {
  *nodes = read_table(nodefile, 5, nnodes, 1);
  *conns = read_table(connfile, 7, nconn, 0);
  return (*nodes && *conns) ? 0 : -1;
}

/* ------------------------------------------------------------ preprocessing */

/* CellIni (serial/CellFunctions.c:99-270) restated in O(nodes + connectors):
 * the node record for (A,B) and the connectors of (A,B) are looked up through
 * per-cell tables instead of a full scan per cell.  "Last record wins" is
 * kept for duplicate node lines and for connectors, as in the reference loops. */
static void cell_init(or_sim *s, const float *nodes, int nnodes, const float *conns,
                      int nconn) {
  const int n = s->n, m = s->m;
  const size_t N = (size_t)n * m;
  const double qlat[9] = {0., 1., 1., 1., 1., sqrt(2), sqrt(2), sqrt(2), sqrt(2)};
  int *node_of = (int *)malloc(N * sizeof(int));
  for (size_t i = 0; i < N; i++) node_of[i] = 0; /* calloc'd ID stays 0 when no record matches */
  for (int r = 0; r < nnodes; r++) {
    const float *nd = nodes + (size_t)r * 5;
    /* float == int comparisons of serial/CellFunctions.c:126 */
    double fa = nd[0], fb = nd[1];
    if (fa >= 0 && fb >= 0 && fa < n && fb < m && fa == (int)fa && fb == (int)fb)
      node_of[(size_t)(int)fb * n + (int)fa] = r;
  }
  /* connectors bucketed by cell, file order kept */
  int *head = (int *)malloc(N * sizeof(int)), *next = (int *)malloc((nconn + 1) * sizeof(int));
  int *tail = (int *)malloc(N * sizeof(int));
  for (size_t i = 0; i < N; i++) head[i] = tail[i] = -1;
  for (int r = 0; r < nconn; r++) {
    const float *c = conns + (size_t)r * 7;
    int a = (int)c[0], b = (int)c[1]; /* (int) casts of serial/CellFunctions.c:164 */
    next[r] = -1;
    if (a < 0 || b < 0 || a >= n || b >= m) continue;
    size_t cell = (size_t)b * n + a;
    if (tail[cell] < 0) head[cell] = r; else next[tail[cell]] = r;
    tail[cell] = r;
  }
  for (int B = 0; B < m; B++)
    for (int A = 0; A < n; A++) {
      or_cell *c = s->cells + (size_t)B * n + A;
      c->id = node_of[(size_t)B * n + A];
      const float *nd = nodes + (size_t)c->id * 5;
      c->coordx = nd[2];
      c->coordy = nd[3];
      c->fluid = (int)nd[4];
      c->u = 0; c->v = 0; c->rho = s->p.rho_ini;
      c->boundary = 0; c->boundary_id = 0;
      for (int k = 0; k < 9; k++) { c->bc_id[k] = 0; c->q[k] = 0.5; }
      for (int r = head[(size_t)B * n + A]; r >= 0; r = next[r]) {
        const float *cn = conns + (size_t)r * 7;
        for (int j = 1; j < 9; j++)
          if (cn[2] == j) {
            c->bc_id[j] = (int)cn[3];
            c->boundary_id = (int)cn[6];
            c->q[j] = sqrt(pow(cn[4] - c->coordx, 2) + pow(cn[5] - c->coordy, 2)) /
                      (s->delta * qlat[j]);
          }
      }
      /* node boundary type and corner flag, serial/CellFunctions.c:181-203 */
      c->corner = 0;
      for (int j = 1; j < 9; j++) {
        if (c->bc_id[j] == 0) continue;
        if (c->boundary == 0) c->boundary = c->bc_id[j];
        else if (c->boundary != c->bc_id[j]) { c->boundary = 1; c->corner = 1; }
      }
      /* corner diagonals become walls, serial/CellFunctions.c:213-231 */
      if (c->corner == 1) {
        if (c->bc_id[1] != 0 && c->bc_id[2] != 0) c->bc_id[5] = 1;
        if (c->bc_id[1] != 0 && c->bc_id[4] != 0) c->bc_id[8] = 1;
        if (c->bc_id[2] != 0 && c->bc_id[3] != 0) c->bc_id[6] = 1;
        if (c->bc_id[3] != 0 && c->bc_id[4] != 0) c->bc_id[7] = 1;
      }
      /* no pull across a boundary link, serial/CellFunctions.c:235-249 */
      for (int k = 0; k < 9; k++) c->stream[k] = 1;
      for (int k = 0; k < 9; k++)
        if (c->bc_id[k] != 0) c->stream[OPP[k]] = 0;
      /* inlet velocity, serial/CellFunctions.c:253-267 */
      if (s->p.inlet_profile == 1) {
        double ext = s->max_y - s->min_y, y = c->coordy - s->min_y;
        c->uo = 4 * 1.5 * s->p.uavg * y * (ext - y) / (ext * ext);
        c->vo = s->p.vavg;
      } else {
        c->uo = s->p.uavg;
        c->vo = s->p.vavg;
      }
      c->u = c->uo;
    }
  free(node_of); free(head); free(next); free(tail);
}

or_sim *or_create(const float *nodes, int nnodes, const float *conns, int nconn,
                  const or_params *p) {
  if (nnodes <= 0) return NULL;
  lattice_init();
  or_sim *s = (or_sim *)calloc(1, sizeof(or_sim));
  s->p = *p;
  /* CompDataNode, serial/FileIO.c:183-209 */
  s->n = (int)nodes[(size_t)(nnodes - 1) * 5 + 0] + 1;
  s->m = (int)nodes[(size_t)(nnodes - 1) * 5 + 1] + 1;
  double d1 = 0, d2 = 0;
  for (int i = 0; i < nnodes; i++) {
    const float *nd = nodes + (size_t)i * 5;
    if (nd[0] == 0 && nd[1] == 0) d1 = nd[2];
    if (nd[0] == 1 && nd[1] == 0) d2 = nd[2];
  }
  s->delta = (d1 > d2 ? d1 : d2) - (d1 < d2 ? d1 : d2);
  /* CompDataConn, serial/FileIO.c:218-254, evaluated in float as defined there */
  int has_inlet = 0;
  for (int i = 0; i < nconn; i++) if (conns[(size_t)i * 7 + 3] == 2) has_inlet = 1;
  if (has_inlet) {
    float fmax = 0.f, fmin = 0.f;
    int i = 0;
    while (conns[(size_t)i * 7 + 3] != 2) {
      fmax = conns[(size_t)(i + 1) * 7 + 5];
      fmin = conns[(size_t)(i + 1) * 7 + 5];
      i++;
    }
    for (i = 0; i < nconn; i++) {
      const float *c = conns + (size_t)i * 7;
      if (c[3] == 2 && (c[2] == 1 || c[2] == 2 || c[2] == 3 || c[2] == 4)) {
        if (c[5] > fmax) fmax = c[5];
        if (c[5] < fmin) fmin = c[5];
      }
    }
    fmax = fmax + s->delta / 2;
    fmin = fmin - s->delta / 2;
    s->max_y = fmax;
    s->min_y = fmin;
  }
  /* serial/Iterate.c:179-180 */
  s->omega = 1.0 / (3. * p->viscosity + 0.5);
  s->omegaA = 8 * (2 - s->omega) / (8 - s->omega);
  /* MRTInitializer, serial/CellFunctions.c:60-90: stmiv = Minv * diag(s) */
  const double a1 = 1. / 36.;
  double sm[9] = {1.0, 1.4, 1.4, 1.0, 1.2, 1.0, 1.2, s->omega, s->omega};
  for (int i = 0; i < 9; i++)
    for (int j = 0; j < 9; j++) {
      double tminv = TMINV36[i][j] == 1 ? a1 : (double)TMINV36[i][j] * a1;
      s->stmiv[i][j] = tminv * sm[j];
    }
  s->cells = (or_cell *)calloc((size_t)s->n * s->m, sizeof(or_cell));
  cell_init(s, nodes, nnodes, conns, nconn);
  return s;
}

void or_destroy(or_sim *s) {
  if (!s) return;
  free(s->cells);
  free(s);
}

void or_dims(const or_sim *s, int *n, int *m) { *n = s->n; *m = s->m; }

void or_constants(const or_sim *s, double *out) {
  out[0] = s->omega; out[1] = s->omegaA; out[2] = s->delta;
  out[3] = s->min_y; out[4] = s->max_y;
}

void or_get_init(const or_sim *s, int *ints, double *reals) {
  size_t N = (size_t)s->n * s->m;
  for (size_t i = 0; i < N; i++) {
    const or_cell *c = s->cells + i;
    int *o = ints + i * 23;
    o[0] = c->fluid; o[1] = c->corner; o[2] = c->boundary; o[3] = c->boundary_id; o[4] = c->id;
    for (int k = 0; k < 9; k++) { o[5 + k] = c->stream[k]; o[14 + k] = c->bc_id[k]; }
    double *r = reals + i * 14;
    for (int k = 0; k < 9; k++) r[k] = c->q[k];
    r[9] = c->coordx; r[10] = c->coordy; r[11] = c->uo; r[12] = c->vo; r[13] = c->u;
  }
}

void or_set_state(or_sim *s, const double *F, const double *rho, const double *u,
                  const double *v) {
  size_t N = (size_t)s->n * s->m;
  for (size_t i = 0; i < N; i++) {
    or_cell *c = s->cells + i;
    if (F) for (int k = 0; k < 9; k++) c->F[k] = F[i * 9 + k];
    if (rho) c->rho = rho[i];
    if (u) c->u = u[i];
    if (v) c->v = v[i];
  }
}

/* ---------------------------------------------------------------- collision */

/* f_eq of serial/CellFunctions.c:355-362, same association. */
static void equilibrium(or_cell *c) {
  double T1 = c->u * c->u + c->v * c->v;
  for (int k = 0; k < 9; k++) {
    double T2 = c->u * CX[k] + c->v * CY[k];
    c->Feq[k] = c->rho * W[k] * (1.0 + 3.0 * T2 + 4.5 * T2 * T2 - 1.5 * T1);
  }
}

/* BGKW, serial/CellFunctions.c:352-365 */
static void coll_bgk(or_cell *c, double om) {
  equilibrium(c);
  for (int k = 0; k < 9; k++) c->METAF[k] = om * c->Feq[k] + (1.0 - om) * c->F[k];
}

/* TRT, serial/CellFunctions.c:372-395; the four split terms are float there. */
static void coll_trt(or_cell *c, double om, double omA) {
  equilibrium(c);
  for (int k = 0; k < 9; k++) {
    int o = OPP[k];
    float fp = 0.5 * (c->F[k] + c->F[o]);
    float feqp = 0.5 * (c->Feq[k] + c->Feq[o]);
    float fm = 0.5 * (c->F[k] - c->F[o]);
    float feqm = 0.5 * (c->Feq[k] - c->Feq[o]);
    c->METAF[k] = c->F[k] - (fp - feqp) * om - (fm - feqm) * omA;
  }
}

/* MRT, serial/CellFunctions.c:401-438: moments m = TM f, then f - Minv S (m - meq). */
static void coll_mrt(or_cell *c, const double stmiv[9][9]) {
  double U = c->u, V = c->v, R = c->rho, mom[9], meq[9];
  meq[0] = R;
  meq[1] = R * (-2.0 + 3.0 * R * (U * U + V * V));
  meq[2] = R * (1.0 - 3.0 * R * (U * U + V * V));
  meq[3] = R * U;
  meq[4] = -R * U;
  meq[5] = R * V;
  meq[6] = -R * V;
  meq[7] = R * (U * U - V * V);
  meq[8] = R * U * V;
  for (int k = 0; k < 9; k++) {
    double a = 0.0;
    for (int l = 0; l < 9; l++) a = a + (double)TM[k][l] * c->F[l];
    mom[k] = a;
  }
  for (int k = 0; k < 9; k++) {
    double b = 0.0;
    for (int l = 0; l < 9; l++) b = b + stmiv[k][l] * (mom[l] - meq[l]);
    c->METAF[k] = c->F[k] - b;
  }
}

/* ------------------------------------------------------- boundary conditions */

/* InletBC, serial/BoundaryConditions.c:14-58 */
static void bc_inlet(or_cell *c) {
  if (c->boundary != 2) return;
  double *F = c->F;
  if (c->bc_id[2] == 2 && c->corner != 1) { /* lid: moving-wall form without (f1-f3)/2 */
    double rhoN = F[0] + F[1] + F[3] + 2 * (F[2] + F[6] + F[5]);
    F[4] = F[2];
    F[8] = F[6] + rhoN * c->uo / 6.0;
    F[7] = F[5] - rhoN * c->uo / 6.0;
  }
  if (c->bc_id[3] == 2 && c->corner != 1) { /* west Zou-He velocity inlet */
    double rhoW = (F[0] + F[2] + F[4] + 2.0 * (F[3] + F[6] + F[7])) / (1.0 - c->uo);
    F[1] = F[3] + 2 * rhoW * c->uo / 3;
    F[5] = F[7] + rhoW * c->uo / 6;
    F[8] = F[6] + rhoW * c->uo / 6;
  }
}

/* OutletBoundaries, serial/BoundaryConditions.c:67-95 (east velocity outlet with Uo) */
static void bc_outlet_velocity(or_cell *c) {
  if (c->bc_id[1] != 3) return;
  double *F = c->F;
  double rhoE = (F[0] + F[2] + F[4] + 2.0 * (F[1] + F[5] + F[8])) / (1 - c->uo);
  F[3] = F[1] - 2 * rhoE * c->uo / 3.0;
  F[7] = F[5] - rhoE * c->uo / 6.0;
  F[6] = F[8] - rhoE * c->uo / 6.0;
}

/* Constant-pressure east outlet (Zou-He density condition).  Not in the
 * reference: its outlets are velocity or extrapolation only. */
static void bc_outlet_pressure(or_cell *c, double rho_out) {
  if (c->bc_id[1] != 3) return;
  double *F = c->F;
  double ux = -1.0 + (F[0] + F[2] + F[4] + 2.0 * (F[1] + F[5] + F[8])) / rho_out;
  double ru = rho_out * ux;
  double d24 = 0.5 * (F[2] - F[4]);
  F[3] = F[1] - (2.0 / 3.0) * ru;
  F[7] = F[5] + d24 - ru / 6.0;
  F[6] = F[8] - d24 - ru / 6.0;
}

/* WallBC, serial/BoundaryConditions.c:104-118: sequential, in place, using the
 * streamed-in population. */
static void bc_wall(or_cell *c) {
  for (int k = 0; k < 9; k++)
    if (c->bc_id[k] == 1) c->F[OPP[k]] = c->F[k];
}

/* CurvedWallBoundaries, serial/BoundaryConditions.c:127-146 (Bouzidi) */
static void bc_curved(or_cell *c) {
  for (int k = 0; k < 9; k++) {
    if (c->bc_id[k] != 1) continue;
    double q = c->q[k];
    if (q < 0.5)
      c->F[OPP[k]] = 2 * q * c->METAF[k] + (1 - 2 * q) * c->Fnb[k];
    else
      c->F[OPP[k]] = c->METAF[k] / 2 / q + (2 * q - 1) / (2 * q) * c->METAF[OPP[k]];
  }
}

/* ----------------------------------------------------------------- one step */

int or_run(or_sim *s, int nsteps, double *resid) {
  const int n = s->n, m = s->m;
  const int N = n * m;
  /* pull offsets of serial/CellFunctions.c:332-340 */
  const int c[9] = {0, -1, -n, 1, n, -n - 1, -n + 1, n + 1, n - 1};
  for (int it = 0; it < nsteps; it++) {
    or_cell *C = s->cells;
    /* CollisionStep, serial/Iterate.c:420-467 */
    for (int i = 0; i < N; i++) {
      if (C[i].fluid != 1) continue;
      if (s->p.model == 1) coll_bgk(C + i, s->omega);
      else if (s->p.model == 2) coll_trt(C + i, s->omega, s->omegaA);
      else if (s->p.model == 3) coll_mrt(C + i, s->stmiv);
    }
    /* UpdateF for every cell, serial/Iterate.c:275-276 */
    for (int i = 0; i < N; i++) memcpy(C[i].F, C[i].METAF, sizeof C[i].F);
    /* StreamingStep, serial/Iterate.c:470-488 */
    for (int i = 0; i < N; i++) {
      if (C[i].fluid != 1) continue;
      for (int k = 0; k < 9; k++)
        if (C[i].stream[k] == 1) C[i].F[k] = C[i + c[k]].METAF[k];
    }
    /* HandleBoundariesStep, serial/Iterate.c:491-550, j-major sweep */
    for (int j = 0; j < m; j++)
      for (int i = 0; i < n; i++) {
        or_cell *x = C + j * n + i;
        if (x->fluid != 1) continue;
        bc_inlet(x);
        if (s->p.curved == 1) {
          for (int k = 0; k < 9; k++) x->Fnb[k] = C[j * n + i + c[k]].METAF[k];
          bc_curved(x);
        } else if (s->p.curved == 2) {
          bc_wall(x);
        }
        if (s->p.outlet == 1) {
          bc_outlet_velocity(x);
        } else if (s->p.outlet == 2) {
          if (x->bc_id[1] == 3) {
            const or_cell *a = C + j * n + i - 1, *b = C + j * n + i - 2;
            x->F[1] = 2 * (a->F[1]) - b->F[1];
            x->F[5] = 2 * (a->F[5]) - b->F[5];
            x->F[8] = 2 * (a->F[8]) - b->F[8];
          }
        } else if (s->p.outlet == 4) {
          bc_outlet_pressure(x, s->p.rho_out);
        }
      }
    /* UpdateMacroscopicStep, serial/Iterate.c:554-567 and CellFunctions.c:457-495 */
    for (int i = 0; i < N; i++) {
      or_cell *x = C + i;
      if (x->fluid != 1) continue;
      double S = 0.0, Us = 0.0, Vs = 0.0;
      for (int k = 0; k < 9; k++) S = S + x->F[k];
      x->rho = S;
      for (int k = 0; k < 9; k++) {
        Us = Us + x->F[k] * CX[k];
        Vs = Vs + x->F[k] * CY[k];
      }
      x->u = Us / x->rho;
      x->v = Vs / x->rho;
      if (x->bc_id[1] == 3) x->v = 0.0;
      if (s->p.drag_id != 0 && x->boundary_id == s->p.drag_id) {
        x->drag = x->rho / 3 * (20 - x->coordx) / 5;
        x->lift = x->rho / 3 * (20 - x->coordy) / 5;
      }
    }
    /* ComputeResiduals, serial/ComputeResiduals.c:6-51, including its index
     * quirk: the double loop over (i<m, j<n) reads cell i only. */
    double L2 = 0.0, drag = 0.0, lift = 0.0;
    for (int i = 0; i < m; i++)
      for (int j = 0; j < n; j++) {
        for (int k = 0; k < 9; k++) L2 = L2 + pow(C[i].F[k] - C[i].METAF[k], 2);
        if (C[i].boundary_id == s->p.drag_id) {
          drag += C[i].drag;
          lift += C[i].lift;
        }
      }
    double L2w = sqrt(L2 / (m * n));
    L2 = sqrt(L2);
    if (resid) {
      resid[4 * it + 0] = L2;
      resid[4 * it + 1] = L2w;
      resid[4 * it + 2] = drag;
      resid[4 * it + 3] = lift;
    }
    if (L2 != L2) return 1; /* the reference prints DIVERGENCE! and exits(1) */
  }
  return 0;
}

void or_get(const or_sim *s, double *F, double *METAF, double *rho, double *u, double *v,
            double *drag, double *lift) {
  size_t N = (size_t)s->n * s->m;
  for (size_t i = 0; i < N; i++) {
    const or_cell *c = s->cells + i;
    if (F) for (int k = 0; k < 9; k++) F[i * 9 + k] = c->F[k];
    if (METAF) for (int k = 0; k < 9; k++) METAF[i * 9 + k] = c->METAF[k];
    if (rho) rho[i] = c->rho;
    if (u) u[i] = c->u;
    if (v) v[i] = c->v;
    if (drag) drag[i] = c->drag;
    if (lift) lift[i] = c->lift;
  }
}

void or_diagnostics(const or_sim *s, double *out) {
  size_t N = (size_t)s->n * s->m;
  double full = 0, mass = 0, mx = 0, my = 0, fx = 0, fy = 0;
  for (size_t i = 0; i < N; i++) {
    const or_cell *c = s->cells + i;
    if (c->fluid != 1) continue;
    for (int k = 0; k < 9; k++) {
      double d = c->F[k] - c->METAF[k];
      full += d * d;
    }
    mass += c->rho;
    mx += c->rho * c->u;
    my += c->rho * c->v;
    if (s->p.drag_id != 0 && c->boundary_id == s->p.drag_id)
      for (int k = 1; k < 9; k++)
        if (c->bc_id[k] == 1) {
          double g = c->METAF[k] + c->F[OPP[k]];
          fx += g * CX[k];
          fy += g * CY[k];
        }
  }
  out[0] = sqrt(full); out[1] = mass; out[2] = mx; out[3] = my; out[4] = fx; out[5] = fy;
}
