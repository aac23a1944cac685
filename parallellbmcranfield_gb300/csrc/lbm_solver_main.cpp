// lbm_solver: drop-in replacement of the serial solver's program
// (serial/main.c + Iteration in serial/Iterate.c) on the C ABI.
//
// Reads SetUpData.ini and Mesh/D2node.dat, Mesh/BCconnectors.dat from the case
// directory, runs the time loop on the GPU and writes the reference's files
// into Results/: logFile.log, InitialData.csv|dat, residuals.dat (one line per
// iteration, or one per --check-every), autosave_iterNNNNN.csv|dat,
// SerialTimeMeasuerment.dat and FinalData.csv|dat.
//
//   lbm_solver [--dir CASE] [--precision fp64|fp32|fp16dev|bf16dev|fp16neq] [--pattern ab|aa]
//              [--tile N] [--check-every K] [--final-data compat|fields|both]
//
// FinalData keeps the reference's index quirk by default (serial/FileIO.c:368
// writes cell i for i < n, m times: the first row repeated); --final-data
// fields writes every cell, --final-data both writes FinalData and
// FinalDataFields.
#include <sys/stat.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/lbm_gb300.h"

namespace {

struct Ini {
  float uavg = 0, vavg = 0, rho_ini = 1, viscosity = 0.01f;
  int inlet_profile = 2, model = 1, curved = 2, outlet = 2, iterations = 0;
  int autosave_every = 1 << 30, autosave_after = 1 << 30, postproc = 1, drag_lift = 0;
  float crit_u = -1, crit_rho = -1;
  int read_former = 0;
};

// ReadIniData, serial/FileIO.c:263-289: sixteen values in a fixed order.
bool read_ini(const std::string &path, Ini *o) {
  FILE *f = std::fopen(path.c_str(), "r");
  if (!f) return false;
  int ok = 0;
  ok += std::fscanf(f, "%f", &o->uavg);
  ok += std::fscanf(f, "%f", &o->vavg);
  ok += std::fscanf(f, "%f", &o->rho_ini);
  ok += std::fscanf(f, "%f", &o->viscosity);
  ok += std::fscanf(f, "%d", &o->inlet_profile);
  ok += std::fscanf(f, "%d", &o->model);
  ok += std::fscanf(f, "%d", &o->curved);
  ok += std::fscanf(f, "%d", &o->outlet);
  ok += std::fscanf(f, "%d", &o->iterations);
  ok += std::fscanf(f, "%d", &o->autosave_every);
  ok += std::fscanf(f, "%d", &o->autosave_after);
  ok += std::fscanf(f, "%d", &o->postproc);
  ok += std::fscanf(f, "%d", &o->drag_lift);
  ok += std::fscanf(f, "%f", &o->crit_u);
  ok += std::fscanf(f, "%f", &o->crit_rho);
  ok += std::fscanf(f, "%d", &o->read_former);
  std::fclose(f);
  return ok == 16;
}

struct CellGeom {
  std::vector<double> x, y;
  std::vector<int> fluid;
};

// CoordX/CoordY/Fluid of every cell from its node record (last matching line,
// ID 0 when none), serial/CellFunctions.c:123-138.
CellGeom cell_geometry(const lbm_mesh &mesh, int n, int m) {
  CellGeom g;
  const size_t N = (size_t)n * m;
  std::vector<int> id(N, 0);
  for (int r = 0; r < mesh.num_nodes; r++) {
    const float *nd = mesh.nodes + (size_t)r * 5;
    double a = nd[0], b = nd[1];
    if (a >= 0 && b >= 0 && a < n && b < m && a == (int)a && b == (int)b)
      id[(size_t)(int)b * n + (int)a] = r;
  }
  g.x.resize(N);
  g.y.resize(N);
  g.fluid.resize(N);
  for (size_t c = 0; c < N; c++) {
    const float *nd = mesh.nodes + (size_t)id[c] * 5;
    g.x[c] = nd[2];
    g.y[c] = nd[3];
    g.fluid[c] = (int)nd[4];
  }
  return g;
}

// WriteResults, serial/FileIO.c:298-348.
void write_results(const std::string &path, int postproc, int n, int m, const CellGeom &g,
                   const double *rho, const double *u, const double *v) {
  FILE *f = std::fopen(path.c_str(), "w");
  if (!f) return;
  const size_t N = (size_t)n * m;
  if (postproc == 1) {
    std::fprintf(f, "x,y,u,v,vel_mag,rho,press,fluid\n");
    for (size_t i = 0; i < N; i++)
      std::fprintf(f, "%f, %f, %f, %f, %f, %f, %f, %d\n", g.x[i], g.y[i], u[i], v[i],
                   std::sqrt(std::pow(u[i], 2) + std::pow(v[i], 2)), rho[i], rho[i] / 3.0,
                   g.fluid[i]);
  } else if (postproc == 2) {
    std::fprintf(f, "Title = \"LBM results\"\n");
    std::fprintf(f, "Variables = \"x\",\"y\",\"u\",\"v\",\"u mag\",\"rho\",\"press\",\"fluid\"\n");
    std::fprintf(f, "Zone i=%d, j=%d, f=point\n", n, m);
    for (size_t i = 0; i < N; i++)
      std::fprintf(f, "%f %f %f %f %f %f %f %d\n", g.x[i], g.y[i], u[i], v[i],
                   std::sqrt(std::pow(u[i], 2) + std::pow(v[i], 2)), rho[i], rho[i] / 3.0,
                   g.fluid[i]);
  }
  std::fclose(f);
}

// WriteFinalResults, serial/FileIO.c:354-427.  compat = the reference's
// (Cells+i) indexing inside the j, i loops; otherwise cell j*n+i.
void write_final(const std::string &path, int postproc, int n, int m, const CellGeom &g,
                 const double *rho, const double *u, const double *v, const double *F,
                 bool compat) {
  FILE *f = std::fopen(path.c_str(), "w");
  if (!f) return;
  const char *sep = postproc == 1 ? ", " : " ";
  if (postproc == 1) {
    std::fprintf(f, "x,y,u,v,vel_mag,rho,press,fluid,f0,f1,f2,f3,f4,f5,f6,f7,f8\n");
  } else {
    std::fprintf(f, "Title = \"LBM results\"\n");
    std::fprintf(f, "Variables = \"x\",\"y\",\"u\",\"v\",\"u mag\",\"rho\",\"press\",\"fluid\","
                    "\"f0\",\"f1\",\"f2\",\"f3\",\"f4\",\"f5\",\"f6\",\"f7\",\"f8\"\n");
    std::fprintf(f, "Zone i=%d, j=%d, f=point\n", n, m);
  }
  for (int j = 0; j < m; j++)
    for (int i = 0; i < n; i++) {
      const size_t c = compat ? (size_t)i : (size_t)j * n + i;
      std::fprintf(f, "%f%s%f%s%f%s%f%s%f%s%f%s%f%s%d", g.x[c], sep, g.y[c], sep, u[c], sep, v[c],
                   sep, std::sqrt(std::pow(u[c], 2) + std::pow(v[c], 2)), sep, rho[c], sep,
                   rho[c] / 3, sep, g.fluid[c]);
      for (int k = 0; k < 9; k++) std::fprintf(f, "%s%f", sep, F[c * 9 + k]);
      std::fprintf(f, "\n");
    }
  std::fclose(f);
}

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int usage() {
  std::fprintf(stderr,
               "usage: lbm_solver [--dir CASE] [--precision fp64|fp32|fp16dev|bf16dev|fp16neq] "
               "[--pattern ab|aa] [--tile N] [--check-every K] [--final-data compat|fields|both]\n");
  return 2;
}

}  // namespace

int main(int argc, char **argv) {
  std::string dir = ".", final_mode = "compat";
  int precision = LBM_FP64, pattern = LBM_AB, tile = 0, check_every = 1;
  for (int i = 1; i < argc; i++) {
    std::string a = argv[i];
    auto val = [&](void) -> std::string { return i + 1 < argc ? argv[++i] : ""; };
    if (a == "--dir") dir = val();
    else if (a == "--precision") {
      std::string p = val();
      precision = p == "fp64" ? LBM_FP64 : p == "fp32" ? LBM_FP32 : p == "fp16dev" ? LBM_FP16DEV
                : p == "bf16dev" ? LBM_BF16DEV : p == "fp16neq" ? LBM_FP16NEQ : -1;
      if (precision < 0) return usage();
    } else if (a == "--pattern") {
      std::string p = val();
      pattern = p == "aa" ? LBM_AA : LBM_AB;
    } else if (a == "--tile") tile = std::atoi(val().c_str());
    else if (a == "--check-every") check_every = std::atoi(val().c_str());
    else if (a == "--final-data") final_mode = val();
    else return usage();
  }
  if (check_every < 1) check_every = 1;
  std::printf("\n###############################################\n");
  std::printf("#### This is a 2D lattice-Boltzmann solver ####\n");
  std::printf("#### GB300 GPU time step (C ABI)           ####\n");
  std::printf("###############################################\n");
  const double t_start = now_s();
  const std::string res_dir = dir + "/Results";
  mkdir(res_dir.c_str(), 0755);  // continue if it already exists, like CreateDirectory
  Ini ini;
  if (!read_ini(dir + "/SetUpData.ini", &ini)) {
    std::fprintf(stderr, "Can't read %s/SetUpData.ini\n", dir.c_str());
    return LBM_IO;
  }
  lbm_mesh mesh;
  if (lbm_mesh_read((dir + "/Mesh/D2node.dat").c_str(), (dir + "/Mesh/BCconnectors.dat").c_str(),
                    &mesh) != LBM_OK) {
    std::fprintf(stderr, "%s\n", lbm_last_error());
    return LBM_IO;
  }
  lbm_params p;
  std::memset(&p, 0, sizeof p);
  p.uavg = ini.uavg;
  p.vavg = ini.vavg;
  p.rho_ini = ini.rho_ini;
  p.viscosity = ini.viscosity;
  p.inlet_profile = ini.inlet_profile;
  p.collision_model = ini.model;
  p.curved_boundaries = ini.curved;
  p.outlet_profile = ini.outlet;
  p.drag_lift_id = ini.drag_lift;
  p.precision = precision;
  p.pattern = pattern;
  p.tile_variant = tile;
  p.rho_out = ini.rho_ini;
  const double t_init0 = now_s();
  lbm_ctx *ctx = nullptr;
  lbm_status st = lbm_create(&mesh, &p, &ctx);
  if (st != LBM_OK) {
    std::fprintf(stderr, "lbm_create: %s: %s\n", lbm_status_string(st), lbm_last_error());
    lbm_mesh_free(&mesh);
    return st;
  }
  int n = 0, m = 0;
  lbm_get_dims(ctx, &n, &m);
  const CellGeom geom = cell_geometry(mesh, n, m);
  // inlet extent as CompDataConn computes it (in float, serial/FileIO.c:218-254)
  double min_y = 0, max_y = 0, delta = 0;
  int n_inlet = 0;
  {
    double d1 = 0, d2 = 0;
    for (int i = 0; i < mesh.num_nodes; i++) {
      const float *nd = mesh.nodes + (size_t)i * 5;
      if (nd[0] == 0 && nd[1] == 0) d1 = nd[2];
      if (nd[0] == 1 && nd[1] == 0) d2 = nd[2];
    }
    delta = std::fabs(d1 - d2);
    // CompDataConn (serial/FileIO.c:218-254), evaluated in float as defined there
    float fmax = 0, fmin = 0;
    bool any = false;
    for (int i = 0; i < mesh.num_conns; i++)
      if (mesh.conns[(size_t)i * 7 + 3] == 2) any = true;
    if (any) {
      int i = 0;
      while (mesh.conns[(size_t)i * 7 + 3] != 2) {
        fmax = fmin = mesh.conns[(size_t)(i + 1) * 7 + 5];
        i++;
      }
      for (i = 0; i < mesh.num_conns; i++) {
        const float *c = mesh.conns + (size_t)i * 7;
        if (c[3] == 2 && (c[2] == 1 || c[2] == 2 || c[2] == 3 || c[2] == 4)) {
          if (c[5] > fmax) fmax = c[5];
          if (c[5] < fmin) fmin = c[5];
          n_inlet++;
        }
      }
      fmax = fmax + delta / 2;
      fmin = fmin - delta / 2;
    }
    max_y = fmax;
    min_y = fmin;
  }
  lbm_mesh_free(&mesh);

  // logFile.log, serial/Iterate.c:113-166
  FILE *log = std::fopen((res_dir + "/logFile.log").c_str(), "w");
  if (log) {
    std::fprintf(log, "This is the 2D lattice Boltzmann *.log file\n\n");
    std::fprintf(log, "\n:::: Imported variables from the *.ini file :::: \n");
    std::fprintf(log, ">>> Uavg              : %3.6f\n", ini.uavg);
    std::fprintf(log, ">>> Vavg              : %3.6f\n", ini.vavg);
    std::fprintf(log, ">>> Initial density   : %2.1f\n", ini.rho_ini);
    std::fprintf(log, ">>> Viscosity         : %3.8f\n", ini.viscosity);
    std::fprintf(log, ">>> # of iterations   : %1.1d\n", ini.iterations);
    std::fprintf(log, ">>> Autosave after    : %1.1d\n", ini.autosave_after);
    std::fprintf(log, ">>> Autosave every    : %1.1d\n", ini.autosave_every);
    std::fprintf(log, ">>> Convergence Veloc : %3.8f\n", ini.crit_u);
    std::fprintf(log, ">>> Convergence Rho   : %3.8f\n", ini.crit_rho);
    std::fprintf(log, ">>> Former data iter# : %1.1d\n", ini.read_former);
    const char *models[] = {"", "BGKW", "TRT", "MRT"};
    if (ini.model >= 1 && ini.model <= 3)
      std::fprintf(log, ">>> CollisionModel   : %s\n", models[ini.model]);
    if (ini.inlet_profile == 1) std::fprintf(log, ">>> InletProfile     : ON\n");
    if (ini.inlet_profile == 2) std::fprintf(log, ">>> InletProfile     : OFF\n");
    if (ini.outlet == 1) std::fprintf(log, ">>> OutletProfile    : ON\n");
    if (ini.outlet == 2) std::fprintf(log, ">>> OutletProfile    : OFF\n");
    if (ini.curved == 1) std::fprintf(log, ">>> CurvedBoundaries : ON\n");
    if (ini.curved == 2) std::fprintf(log, ">>> CurvedBoundaries : OFF\n");
    if (ini.postproc == 1) std::fprintf(log, ">>> Results format   : Paraview (*.csv)\n");
    if (ini.postproc == 2) std::fprintf(log, ">>> Results format   : Tecplot (*.dat)\n");
    if (ini.drag_lift != 0) std::fprintf(log, ">>> Drag, lift @ BC  : %d\n", ini.drag_lift);
    else std::fprintf(log, ">>> Drag, lift was not calculated\n");
    std::fprintf(log, "\n:::: Calculated variables from mesh :::: \n");
    std::fprintf(log, ">>> Grid spacing        = %f\n", delta);
    std::fprintf(log, ">>> # of nodes in x (n) = %d\n", n);
    std::fprintf(log, ">>> # of nodes in y (m) = %d\n", m);
    std::fprintf(log, ">>> NumInletNodes       = %d\n", n_inlet);
    std::fprintf(log, ">>> MaxInletCoordY      = %f\n", max_y);
    std::fprintf(log, ">>> MinInletCoordY      = %f\n", min_y);
    std::fprintf(log, "\n:::: Initializing ::::\n");
  }
  const double t_init = now_s() - t_init0;
  if (log) std::fprintf(log, "\n:::: Initialization done! ::::\n");
  const std::string ext = ini.postproc == 2 ? ".dat" : ".csv";
  const size_t N = (size_t)n * m;
  std::vector<double> rho(N), u(N), v(N);
  lbm_get_fields(ctx, rho.data(), u.data(), v.data(), nullptr, nullptr);
  write_results(res_dir + "/InitialData" + ext, ini.postproc, n, m, geom, rho.data(), u.data(),
                v.data());
  std::printf("\nInitialized data was written to %s\n", (res_dir + "/InitialData" + ext).c_str());
  FILE *resid = std::fopen((res_dir + "/residuals.dat").c_str(), "w");
  if (resid) std::fprintf(resid, "Iter L2_norm L2_norm_weighted Drag Lift\n");
  if (log) std::fprintf(log, "\n:::: Start Iterations ::::\n");
  std::printf("\n:::: Start Iterations ::::\n");

  // the loop of serial/Iterate.c:263-332
  double R[4] = {100.0, 100.0, 0.0, 0.0};
  int iter = 0, status = 0;
  double t_write = 0.0;
  std::string last_autosave = "NOWHERE!";
  const double t_loop0 = now_s();
  while (R[0] > ini.crit_u && R[1] > ini.crit_rho && iter < ini.iterations) {
    int k = check_every;
    if (iter + k > ini.iterations) k = ini.iterations - iter;
    // stop at the next autosave / progress boundary so those happen on time
    const int to_save = ini.autosave_every > 0 ? ini.autosave_every - iter % ini.autosave_every : k;
    const int to_prog = 100 - iter % 100;
    if (k > to_save) k = to_save;
    if (k > to_prog) k = to_prog;
    st = lbm_step(ctx, k, k, R);
    if (st == LBM_DIVERGED) {
      std::printf("\nDIVERGENCE!\n");
      status = 1;
      break;
    }
    if (st != LBM_OK) {
      std::fprintf(stderr, "lbm_step: %s: %s\n", lbm_status_string(st), lbm_last_error());
      status = st;
      break;
    }
    iter += k;
    if (resid) std::fprintf(resid, "%d %5.4e %5.4e %f %f\n", iter - 1, R[0], R[1], R[2], R[3]);
    if (iter % 100 == 0) {
      std::printf("Iterations: %05d/%05d || ", iter, ini.iterations);
      std::printf("Residuals: l2norm  %e; L2_norm_weighted  %e\n", R[0], R[1]);
    }
    if (ini.autosave_every > 0 && iter % ini.autosave_every == 0 && iter > ini.autosave_after) {
      char name[64];
      std::snprintf(name, sizeof name, "/autosave_iter%05d", iter);
      last_autosave = res_dir + name + ext;
      const double t0 = now_s();
      lbm_get_fields(ctx, rho.data(), u.data(), v.data(), nullptr, nullptr);
      write_results(last_autosave, ini.postproc, n, m, geom, rho.data(), u.data(), v.data());
      t_write += now_s() - t0;
    }
  }
  const double t_iter = now_s() - t_loop0;
  if (resid) std::fclose(resid);
  const double t_all = now_s() - t_start;
  if (log) {
    std::fprintf(log, "\nOverall calculations took %f seconds\n", t_all);
    std::fprintf(log, "Main while loop took %f seconds\n", t_iter);
    std::fprintf(log, "Initialization took %f seconds\n", t_init);
    std::fprintf(log, "Fused GPU step (collision, streaming, boundaries, macroscopic, "
                      "residuals) took %f seconds\n", t_iter - t_write);
    std::fprintf(log, "Writing results took %f seconds\n", t_write);
    std::fprintf(log, "\n:::: Iterations done! ::::\n");
    std::fclose(log);
  }
  // the phases of serial/Iterate.c:360-371 run as one fused launch per step here
  FILE *tf = std::fopen((res_dir + "/SerialTimeMeasuerment.dat").c_str(), "w");
  if (tf) {
    std::fprintf(tf, "tOverall %f\n", t_all);
    std::fprintf(tf, "tIteration %f\n", t_iter);
    std::fprintf(tf, "tInitialization %f\n", t_init);
    std::fprintf(tf, "tFusedStep %f\n", t_iter - t_write);
    std::fprintf(tf, "tWriting %f\n", t_write);
    std::fclose(tf);
  }
  if (iter > 0) {
    std::vector<double> F(N * 9);
    lbm_get_fields(ctx, rho.data(), u.data(), v.data(), F.data(), nullptr);
    if (final_mode == "compat" || final_mode == "both")
      write_final(res_dir + "/FinalData" + ext, ini.postproc, n, m, geom, rho.data(), u.data(),
                  v.data(), F.data(), true);
    if (final_mode == "fields" || final_mode == "both")
      write_final(res_dir + (final_mode == "both" ? "/FinalDataFields" : "/FinalData") + ext,
                  ini.postproc, n, m, geom, rho.data(), u.data(), v.data(), F.data(), false);
  }
  std::printf("\n\nLog was written to %s/logFile.log\n", res_dir.c_str());
  std::printf("Last autosave result can be found at %s\n", last_autosave.c_str());
  std::printf("Residuals were written to %s/residuals.dat\n", res_dir.c_str());
  lbm_destroy(ctx);
  return status;
}
