// Mesh input in the reference's file format: reader, writer and generators.
//
// File formats (serial/FileIO.c:39-44 and :116-133):
//   D2node.dat        i j x y fluid                 one line per lattice node
//   BCconnectors.dat  i j dir type x y boundary_id  one line per boundary link
// The reader parses with fscanf("%f"), as serial/FileIO.c:56-74 and :147-166
// do, so every value is the float the reference sees.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/lbm_gb300.h"
#include "lbm_internal.h"

namespace {

const int MCX[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
const int MCY[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};

float *read_table(const char *path, int ncol, int *nrows, bool nodes) {
  FILE *f = std::fopen(path, "r");
  if (!f) return nullptr;
  int rows = 0;
  if (nodes) {
    int a, b, c;
    float x, y;
    while (std::fscanf(f, "%d %d %f %f %d", &a, &b, &x, &y, &c) == 5) rows++;
  } else {
    int a, b, c, d, e;
    float x, y;
    while (std::fscanf(f, "%d %d %d %d %f %f %d", &a, &b, &c, &d, &x, &y, &e) == 7) rows++;
  }
  std::rewind(f);
  float *t = (float *)std::calloc((size_t)(rows > 0 ? rows : 1) * ncol, sizeof(float));
  if (!t) {
    std::fclose(f);
    return nullptr;
  }
  for (int r = 0; r < rows; r++)
    for (int c = 0; c < ncol; c++)
      if (std::fscanf(f, "%f", &t[(size_t)r * ncol + c]) != 1) t[(size_t)r * ncol + c] = 0.f;
  std::fclose(f);
  *nrows = rows;
  return t;
}

// A mesh whose fluid cells are given by a predicate on cell indices, solid
// elsewhere.  Boundary links are found by walking each fluid cell's 8 links
// and intersecting them with the wall geometry supplied by `hit`.
struct Link {
  float x, y;
  int type, id;
};

template <class Fluid, class Hit>
lbm_status build_mesh(int n, int m, double delta, Fluid fluid, Hit hit, lbm_mesh *out) {
  const size_t N = (size_t)n * m;
  float *nodes = (float *)std::malloc(N * 5 * sizeof(float));
  if (!nodes) return LBM_NOMEM;
  std::vector<float> conns;
  for (int j = 0; j < m; j++)
    for (int i = 0; i < n; i++) {
      float *nd = nodes + ((size_t)j * n + i) * 5;
      nd[0] = (float)i;
      nd[1] = (float)j;
      nd[2] = (float)((i - 0.5) * delta);
      nd[3] = (float)((j - 0.5) * delta);
      nd[4] = fluid(i, j) ? 1.f : 0.f;
    }
  for (int j = 0; j < m; j++)
    for (int i = 0; i < n; i++) {
      if (!fluid(i, j)) continue;
      for (int k = 1; k < 9; k++) {
        int a = i + MCX[k], b = j + MCY[k];
        bool solid = a < 0 || b < 0 || a >= n || b >= m || !fluid(a, b);
        if (!solid) continue;
        Link l = hit(i, j, k);
        conns.insert(conns.end(), {(float)i, (float)j, (float)k, (float)l.type, l.x, l.y,
                                   (float)l.id});
      }
    }
  float *c = (float *)std::malloc((conns.size() > 0 ? conns.size() : 1) * sizeof(float));
  if (!c) {
    std::free(nodes);
    return LBM_NOMEM;
  }
  if (!conns.empty()) std::memcpy(c, conns.data(), conns.size() * sizeof(float));
  out->nodes = nodes;
  out->num_nodes = (int32_t)N;
  out->conns = c;
  out->num_conns = (int32_t)(conns.size() / 7);
  return LBM_OK;
}

// First crossing of the link from cell (i,j) along e_k with the axis-aligned
// box [x0,x1] x [y0,y1] (physical units); ties between a vertical and a
// horizontal wall go to the horizontal one.
struct BoxHit {
  double t;
  double x, y;
  int side;  // 0 west, 1 east, 2 south, 3 north
};

BoxHit box_exit(double px, double py, double dx, double dy, double x0, double x1, double y0,
                double y1) {
  double tx = 1e300, ty = 1e300;
  int sx = -1, sy = -1;
  if (dx < 0) { tx = (x0 - px) / dx; sx = 0; }
  if (dx > 0) { tx = (x1 - px) / dx; sx = 1; }
  if (dy < 0) { ty = (y0 - py) / dy; sy = 2; }
  if (dy > 0) { ty = (y1 - py) / dy; sy = 3; }
  BoxHit h;
  if (ty <= tx + 1e-9) { h.t = ty; h.side = sy; }
  else { h.t = tx; h.side = sx; }
  h.x = px + h.t * dx;
  h.y = py + h.t * dy;
  // snap the coordinate that lies on the wall
  if (h.side == 0) h.x = x0;
  if (h.side == 1) h.x = x1;
  if (h.side == 2) h.y = y0;
  if (h.side == 3) h.y = y1;
  return h;
}

}  // namespace

extern "C" {

lbm_status lbm_mesh_read(const char *node_file, const char *conn_file, lbm_mesh *out) {
  if (!node_file || !conn_file || !out) return lbm::fail(LBM_INVALID, "null argument");
  int nn = 0, nc = 0;
  float *nodes = read_table(node_file, 5, &nn, true);
  if (!nodes) return lbm::fail(LBM_IO, std::string("cannot read ") + node_file);
  float *conns = read_table(conn_file, 7, &nc, false);
  if (!conns) {
    std::free(nodes);
    return lbm::fail(LBM_IO, std::string("cannot read ") + conn_file);
  }
  out->nodes = nodes;
  out->num_nodes = nn;
  out->conns = conns;
  out->num_conns = nc;
  return LBM_OK;
}

void lbm_mesh_free(lbm_mesh *mesh) {
  if (!mesh) return;
  std::free((void *)mesh->nodes);
  std::free((void *)mesh->conns);
  mesh->nodes = nullptr;
  mesh->conns = nullptr;
  mesh->num_nodes = mesh->num_conns = 0;
}

lbm_status lbm_mesh_cavity(int32_t side, lbm_mesh *out) {
  if (side < 2 || !out) return lbm::fail(LBM_INVALID, "cavity side must be >= 2");
  // layout of the shipped cases: n = side + 2 columns, m = side + 3 rows,
  // walls half-way between the fluid ring and the solid ring, unit square
  const int n = side + 2, m = side + 3;
  const double d = 1.0 / side;
  auto fluid = [side](int i, int j) { return i >= 1 && i <= side && j >= 1 && j <= side; };
  auto hit = [d](int i, int j, int k) {
    BoxHit h = box_exit((i - 0.5) * d, (j - 0.5) * d, MCX[k] * d, MCY[k] * d, 0.0, 1.0, 0.0, 1.0);
    Link l;
    l.x = (float)h.x;
    l.y = (float)h.y;
    const int ids[4] = {1, 3, 4, 2};  // west, east, south, north (lid)
    l.id = ids[h.side];
    l.type = h.side == 3 ? 2 : 1;
    return l;
  };
  return build_mesh(n, m, d, fluid, hit, out);
}

lbm_status lbm_mesh_channel(int32_t nx, int32_t ny, int32_t ncyl, const double *cx,
                            const double *cy, const double *r, lbm_mesh *out) {
  if (nx < 4 || ny < 2 || !out || ncyl < 0 || (ncyl > 0 && (!cx || !cy || !r)))
    return lbm::fail(LBM_INVALID, "bad channel arguments");
  const int n = nx + 2, m = ny + 2;
  const double d = 1.0 / ny;
  std::vector<double> X(cx, cx + ncyl), Y(cy, cy + ncyl), RR(r, r + ncyl);
  auto in_cyl = [&](double i, double j) {
    for (int c = 0; c < ncyl; c++)
      if ((i - X[c]) * (i - X[c]) + (j - Y[c]) * (j - Y[c]) <= RR[c] * RR[c]) return c;
    return -1;
  };
  auto fluid = [&](int i, int j) {
    return i >= 1 && i <= nx && j >= 1 && j <= ny && in_cyl(i, j) < 0;
  };
  auto hit = [&](int i, int j, int k) {
    Link l;
    int a = i + MCX[k], b = j + MCY[k];
    int c = (a >= 1 && a <= nx && b >= 1 && b <= ny) ? in_cyl(a, b) : -1;
    if (c >= 0) {
      // segment-circle intersection in cell-index units, nearest root in (0,1]
      double px = i - X[c], py = j - Y[c], dx = MCX[k], dy = MCY[k];
      double A = dx * dx + dy * dy, B = 2 * (px * dx + py * dy), C = px * px + py * py - RR[c] * RR[c];
      double disc = B * B - 4 * A * C;
      double t = disc > 0 ? (-B - std::sqrt(disc)) / (2 * A) : 0.5;
      if (t < 0) t = 0;
      if (t > 1) t = 1;
      double ix = i + t * dx, iy = j + t * dy;
      l.x = (float)((ix - 0.5) * d);
      l.y = (float)((iy - 0.5) * d);
      l.type = 1;
      l.id = 5;
      return l;
    }
    BoxHit h = box_exit((i - 0.5) * d, (j - 0.5) * d, MCX[k] * d, MCY[k] * d, 0.0, nx * d, 0.0,
                        ny * d);
    l.x = (float)h.x;
    l.y = (float)h.y;
    const int ids[4] = {1, 3, 4, 2};    // west inlet, east outlet, bottom, top
    const int types[4] = {2, 3, 1, 1};
    l.id = ids[h.side];
    l.type = types[h.side];
    return l;
  };
  return build_mesh(n, m, d, fluid, hit, out);
}

lbm_status lbm_mesh_write(const lbm_mesh *mesh, const char *node_file, const char *conn_file) {
  if (!mesh || !node_file || !conn_file) return lbm::fail(LBM_INVALID, "null argument");
  FILE *f = std::fopen(node_file, "w");
  if (!f) return lbm::fail(LBM_IO, std::string("cannot write ") + node_file);
  for (int r = 0; r < mesh->num_nodes; r++) {
    const float *a = mesh->nodes + (size_t)r * 5;
    std::fprintf(f, "%d    %d    %.9g    %.9g    %d\n", (int)a[0], (int)a[1], a[2], a[3],
                 (int)a[4]);
  }
  std::fclose(f);
  f = std::fopen(conn_file, "w");
  if (!f) return lbm::fail(LBM_IO, std::string("cannot write ") + conn_file);
  for (int r = 0; r < mesh->num_conns; r++) {
    const float *a = mesh->conns + (size_t)r * 7;
    std::fprintf(f, "%d    %d    %d  %d   %.9g   %.9g   %d\n", (int)a[0], (int)a[1], (int)a[2],
                 (int)a[3], a[4], a[5], (int)a[6]);
  }
  std::fclose(f);
  return LBM_OK;
}

}  // extern "C"
