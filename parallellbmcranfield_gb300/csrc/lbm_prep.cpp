// Host preprocessing: from the reference's mesh arrays to the per-node class
// bytes and boundary records the fused kernel reads.
//
// The per-cell decisions are those of CellIni (serial/CellFunctions.c:99-270),
// evaluated in O(nodes + connectors) instead of the reference's scan of all
// nodes and connectors for every cell.  Mesh-derived constants follow
// CompDataNode / CompDataConn (serial/FileIO.c:183-254) in float where the
// reference computes in float, and Omega / OmegaA / MRT follow
// serial/Iterate.c:179-188 and serial/CellFunctions.c:11-92.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "lbm_internal.h"

namespace lbm {

namespace {
const int PCX[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
const int PCY[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
const int POPP[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};
// MRT inverse transform in units of 1/36 (serial/CellFunctions.c:24-35)
const int MINV36[9][9] = {
    {4, -4, 4, 0, 0, 0, 0, 0, 0},   {4, -1, -2, 6, -6, 0, 0, 9, 0},
    {4, -1, -2, 0, 0, 6, -6, -9, 0}, {4, -1, -2, -6, 6, 0, 0, 9, 0},
    {4, -1, -2, 0, 0, -6, 6, -9, 0}, {4, 2, 1, 6, 3, 6, 3, 0, 9},
    {4, 2, 1, -6, -3, 6, 3, 0, -9},  {4, 2, 1, -6, -3, -6, -3, 0, 9},
    {4, 2, 1, 6, 3, -6, -3, 0, -9}};
}  // namespace

lbm_status preprocess(const lbm_mesh *mesh, const lbm_params *p, Prep *P) {
  if (!mesh || !p || !P) return fail(LBM_INVALID, "null argument");
  if (mesh->num_nodes <= 0 || !mesh->nodes) return fail(LBM_INVALID, "mesh has no nodes");
  if (mesh->num_conns < 0 || (mesh->num_conns > 0 && !mesh->conns))
    return fail(LBM_INVALID, "bad connector array");
  if (p->collision_model < 1 || p->collision_model > 3)
    return fail(LBM_INVALID, "collision_model must be 1 (BGKW), 2 (TRT) or 3 (MRT)");
  if (p->outlet_profile < 1 || p->outlet_profile > 4)
    return fail(LBM_INVALID, "outlet_profile must be 1..4");
  if (p->outlet_profile == 4 && !(p->rho_out > 0))
    return fail(LBM_INVALID, "outlet_profile 4 needs rho_out > 0");
  const float *nodes = mesh->nodes, *conns = mesh->conns;
  const int nn = mesh->num_nodes, nc = mesh->num_conns;

  // CompDataNode, serial/FileIO.c:193-208
  const int n = (int)nodes[(size_t)(nn - 1) * 5 + 0] + 1;
  const int m = (int)nodes[(size_t)(nn - 1) * 5 + 1] + 1;
  if (n < 3 || m < 3) return fail(LBM_INVALID, "grid must be at least 3x3");
  if ((long long)n * m > (1LL << 31))
    return fail(LBM_INVALID, "grid larger than 2^31 cells");
  double d1 = 0, d2 = 0;
  for (int i = 0; i < nn; i++) {
    const float *nd = nodes + (size_t)i * 5;
    if (nd[0] == 0 && nd[1] == 0) d1 = nd[2];
    if (nd[0] == 1 && nd[1] == 0) d2 = nd[2];
  }
  P->n = n;
  P->m = m;
  P->delta = (d1 > d2 ? d1 : d2) - (d1 < d2 ? d1 : d2);
  // CompDataConn, serial/FileIO.c:218-254, in float as defined there
  bool has_inlet = false;
  for (int i = 0; i < nc; i++)
    if (conns[(size_t)i * 7 + 3] == 2) has_inlet = true;
  if (has_inlet) {
    float fmax = 0.f, fmin = 0.f;
    int i = 0;
    while (conns[(size_t)i * 7 + 3] != 2) {
      fmax = conns[(size_t)(i + 1) * 7 + 5];
      fmin = conns[(size_t)(i + 1) * 7 + 5];
      i++;
    }
    for (i = 0; i < nc; i++) {
      const float *c = conns + (size_t)i * 7;
      if (c[3] == 2 && (c[2] == 1 || c[2] == 2 || c[2] == 3 || c[2] == 4)) {
        if (c[5] > fmax) fmax = c[5];
        if (c[5] < fmin) fmin = c[5];
      }
    }
    fmax = fmax + P->delta / 2;
    fmin = fmin - P->delta / 2;
    P->max_y = fmax;
    P->min_y = fmin;
  }
  // collision constants, serial/Iterate.c:179-180 and MRTInitializer
  P->omega = 1.0 / (3. * p->viscosity + 0.5);
  P->omegaA = 8 * (2 - P->omega) / (8 - P->omega);
  {
    const double a1 = 1. / 36.;
    const double sm[9] = {1.0, 1.4, 1.4, 1.0, 1.2, 1.0, 1.2, P->omega, P->omega};
    for (int i = 0; i < 9; i++)
      for (int j = 0; j < 9; j++) P->stmiv[i * 9 + j] = ((double)MINV36[i][j] * a1) * sm[j];
  }

  const int pitch = (n + 255) / 256 * 256;  // whole warps of the widest vector tile
  P->pitch = pitch;
  P->plane = (long long)m * pitch;
  const size_t N = (size_t)n * m;
  P->cls.assign((size_t)P->plane, CLS_SOLID);
  P->aux.assign((size_t)P->plane, 0u);
  P->rec.clear();
  P->nfluid = 0;

  // node record of every cell: last matching line wins, ID 0 if none
  // (serial/CellFunctions.c:123-131)
  std::vector<int32_t> node_of(N, 0);
  for (int r = 0; r < nn; r++) {
    const float *nd = nodes + (size_t)r * 5;
    double fa = nd[0], fb = nd[1];
    if (fa >= 0 && fb >= 0 && fa < n && fb < m && fa == (double)(int)fa && fb == (double)(int)fb)
      node_of[(size_t)(int)fb * n + (int)fa] = r;
  }
  // connectors per cell, file order kept (serial/CellFunctions.c:162-178)
  std::vector<int32_t> head(N, -1), tail(N, -1), next(nc > 0 ? nc : 1, -1);
  for (int r = 0; r < nc; r++) {
    const float *c = conns + (size_t)r * 7;
    int a = (int)c[0], b = (int)c[1];
    if (a < 0 || b < 0 || a >= n || b >= m) continue;
    size_t cell = (size_t)b * n + a;
    if (tail[cell] < 0) head[cell] = r;
    else next[tail[cell]] = r;
    tail[cell] = r;
  }
  const bool profile = p->inlet_profile == 1;
  if (profile) P->uo_cell.assign(N, 0.0);
  else P->uo_cell.clear();

  auto fluid_of = [&](int a, int b) -> bool {
    if (a < 0 || b < 0 || a >= n || b >= m) return false;
    return (int)nodes[(size_t)node_of[(size_t)b * n + a] * 5 + 4] == 1;
  };
  const double qlat[9] = {0., 1., 1., 1., 1., std::sqrt(2), std::sqrt(2), std::sqrt(2),
                          std::sqrt(2)};
  std::vector<uint32_t> east_cells;
  for (int B = 0; B < m; B++)
    for (int A = 0; A < n; A++) {
      const size_t cell = (size_t)B * n + A;
      const float *nd = nodes + (size_t)node_of[cell] * 5;
      const double cx = nd[2], cy = nd[3];
      const int fluid = (int)nd[4];
      int bc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, boundary = 0, boundary_id = 0, corner = 0;
      double q[9];
      for (int k = 0; k < 9; k++) q[k] = 0.5;
      for (int r = head[cell]; r >= 0; r = next[r]) {
        const float *cn = conns + (size_t)r * 7;
        for (int j = 1; j < 9; j++)
          if (cn[2] == j) {
            bc[j] = (int)cn[3];
            boundary_id = (int)cn[6];
            q[j] = std::sqrt(std::pow(cn[4] - cx, 2) + std::pow(cn[5] - cy, 2)) /
                   (P->delta * qlat[j]);
          }
      }
      for (int j = 1; j < 9; j++) {
        if (bc[j] == 0) continue;
        if (boundary == 0) boundary = bc[j];
        else if (boundary != bc[j]) {
          boundary = 1;
          corner = 1;
        }
      }
      if (corner == 1) {
        if (bc[1] != 0 && bc[2] != 0) bc[5] = 1;
        if (bc[1] != 0 && bc[4] != 0) bc[8] = 1;
        if (bc[2] != 0 && bc[3] != 0) bc[6] = 1;
        if (bc[3] != 0 && bc[4] != 0) bc[7] = 1;
      }
      int stream[9];
      for (int k = 0; k < 9; k++) stream[k] = 1;
      for (int k = 0; k < 9; k++)
        if (bc[k] != 0) stream[POPP[k]] = 0;
      double uo;
      if (profile) {
        double ext = P->max_y - P->min_y, y = cy - P->min_y;
        uo = 4 * 1.5 * p->uavg * y * (ext - y) / (ext * ext);
        P->uo_cell[cell] = uo;
      } else {
        uo = p->uavg;
      }
      if (fluid != 1) continue;
      P->nfluid++;
      if (A == 0 || B == 0 || A == n - 1 || B == m - 1)
        return fail(LBM_INVALID, "fluid cell (" + std::to_string(A) + "," + std::to_string(B) +
                                     ") on the grid border; a solid ring is required");
      bool any_bc = false, all_nb_fluid = true;
      for (int k = 1; k < 9; k++) {
        if (bc[k] != 0) any_bc = true;
        if (!fluid_of(A + PCX[k], B + PCY[k])) all_nb_fluid = false;
      }
      const size_t node = (size_t)B * pitch + A;
      if (!any_bc && all_nb_fluid) {
        P->cls[node] = CLS_BULK;
        continue;
      }
      BRec r;
      std::memset(&r, 0, sizeof r);
      r.node = (uint32_t)node;
      uint32_t fl = 0;
      for (int k = 0; k < 9; k++) {
        if (stream[k] == 1) fl |= 1u << (FL_STREAM_SHIFT + k);
        if (bc[k] == 1) fl |= 1u << (FL_WALL_SHIFT + k);
      }
      if (boundary == 2 && bc[2] == 2 && corner != 1) fl |= FL_LID;
      if (boundary == 2 && bc[3] == 2 && corner != 1) fl |= FL_WEST;
      if (bc[1] == 3) fl |= FL_EAST;
      if (p->drag_lift_id != 0 && boundary_id == p->drag_lift_id) fl |= FL_DRAG;
      r.flags = fl;
      r.uo = uo;
      for (int k = 0; k < 9; k++) r.q[k] = q[k];
      r.x = cx;
      r.y = cy;
      P->cls[node] = CLS_SPECIAL;
      P->aux[node] = (uint32_t)P->rec.size();
      P->rec.push_back(r);
      if (fl & FL_EAST) east_cells.push_back((uint32_t)node);
    }

  // 2nd-order outlet extrapolation reads the treated cells i-1 and i-2 of the
  // same row (serial/Iterate.c:538-540); those must not be outlet cells.
  if (p->outlet_profile == 2)
    for (uint32_t node : east_cells) {
      const int x = (int)(node % pitch);
      if (x < 2) return fail(LBM_INVALID, "outlet cell closer than 2 cells to the west border");
      for (int d = 1; d <= 2; d++) {
        uint32_t z = node - d;
        if (P->cls[z] == CLS_SPECIAL && (P->rec[P->aux[z]].flags & FL_EAST))
          return fail(LBM_INVALID, "outlet extrapolation source is itself an outlet cell");
      }
    }

  // AA pattern: every cell whose METAF a special cell reads gets a side-buffer slot.
  P->nsb = 0;
  if (p->pattern == LBM_AA) {
    uint32_t nrec = (uint32_t)P->rec.size();
    for (uint32_t i = 0; i < nrec; i++) P->rec[i].sb = i;
    uint32_t next_sb = nrec;
    auto mark = [&](long long center) {
      for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++) {
          long long z = center + dx + (long long)dy * pitch;
          if (z < 0 || z >= P->plane) continue;
          if (P->cls[z] == CLS_BULK) {
            P->cls[z] = CLS_BULK_REC;
            P->aux[z] = next_sb++;
          }
        }
    };
    for (uint32_t i = 0; i < nrec; i++) {
      long long node = P->rec[i].node;
      mark(node);
      if (p->outlet_profile == 2 && (P->rec[i].flags & FL_EAST)) {
        mark(node - 1);
        mark(node - 2);
      }
    }
    P->nsb = next_sb;
  }
  return LBM_OK;
}

}  // namespace lbm

extern "C" lbm_status lbm_inspect_mesh(const lbm_mesh *mesh, const lbm_params *params,
                                       int32_t *n, int32_t *m, uint8_t *cls, uint32_t *flags,
                                       double *q) {
  lbm_params p = *params;
  p.pattern = LBM_AB;
  lbm::Prep P;
  lbm_status s = lbm::preprocess(mesh, &p, &P);
  if (s != LBM_OK) return s;
  if (n) *n = P.n;
  if (m) *m = P.m;
  for (int y = 0; y < P.m; y++)
    for (int x = 0; x < P.n; x++) {
      const size_t cell = (size_t)y * P.n + x, node = (size_t)y * P.pitch + x;
      const uint8_t c = P.cls[node];
      if (cls) cls[cell] = c;
      if (flags) flags[cell] = c == lbm::CLS_SPECIAL ? P.rec[P.aux[node]].flags : 0u;
      if (q)
        for (int k = 0; k < 9; k++)
          q[cell * 9 + k] = c == lbm::CLS_SPECIAL ? P.rec[P.aux[node]].q[k] : 0.5;
    }
  return LBM_OK;
}
