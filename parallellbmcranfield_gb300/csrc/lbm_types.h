// Host/device shared types of the D2Q9 step library.
#pragma once
#include <cstdint>

namespace lbm {

// Per-node class byte (the only per-node metadata every launch reads).
enum NodeClass : uint8_t {
  CLS_SOLID = 0,    // solid or padding: never updated, reads as F = METAF = 0
  CLS_BULK = 1,     // fluid, no boundary link, all 8 neighbours fluid
  CLS_BULK_REC = 2, // bulk node whose METAF is also kept in the side buffer (AA only)
  CLS_SPECIAL = 3   // fluid node with boundary work: described by a BRec
};

// Flag bits of BRec::flags.
enum : uint32_t {
  FL_STREAM_SHIFT = 0,  // bits 0..8: StreamLattice[k] == 1
  FL_WALL_SHIFT = 9,    // bits 9..17: BC_ID[k] == 1
  FL_LID = 1u << 18,    // InletBC top branch active (serial/BoundaryConditions.c:25)
  FL_WEST = 1u << 19,   // InletBC left branch active (serial/BoundaryConditions.c:39)
  FL_EAST = 1u << 20,   // BC_ID[1] == 3: east outlet cell
  FL_DRAG = 1u << 21,   // BoundaryID == CalculateDragLift != 0
};

// One record per special node (cold data, read only by that node's thread
// and by the outlet extrapolation of its east neighbours).
struct BRec {
  uint32_t node;  // linear node index y * pitch + x
  uint32_t flags;
  uint32_t sb;    // side-buffer slot (AA pattern)
  uint32_t pad;
  double uo;      // Uo of CellIni (inlet / velocity-outlet speed)
  double q[9];    // Q[k] of CellIni
  double x, y;    // CoordX, CoordY (drag/lift placeholder)
};
static_assert(sizeof(BRec) == 112, "BRec layout");

// Layout / phase of the population array for one launch.
enum Phase : int {
  PH_AB = 0,    // pull from src (A-B pattern)
  PH_AA_A = 1,  // AA: state in A layout (slot opp(k) at x), output B layout
  PH_AA_B = 2   // AA: state in B layout (slot k at x + e_k), output A layout
};

// Tile variants of the fused step.  kind 0: one thread per node column
// with NPT rows (bx threads per block); kind 1: V nodes per thread moved as
// one vector word per plane; kind 3: two nodes per thread as one 32-bit word
// per plane, NPT rows (16-bit storage; other storage runs kind 0 with bx 128);
// kind 2: TMA pipeline -- tiles of tx x ty nodes
// whose 9 source planes are staged in shared memory by cp.async.bulk row
// copies (a ring of stages, mbarrier completion), rpt rows per thread.  The
// autotuner picks one per domain and storage.
struct TileVariant {
  int kind, bx, v, npt, tx, ty, rpt;
};
constexpr int NVAR = 6;
constexpr TileVariant VARS[NVAR] = {
    {0, 128, 1, 1, 0, 0, 0},   {0, 64, 1, 4, 0, 0, 0},   {1, 128, 4, 1, 0, 0, 0},
    {2, 0, 0, 0, 128, 4, 2},   {3, 128, 2, 2, 0, 0, 0},  {3, 128, 2, 4, 0, 0, 0}};
// Bulk-step tiles of the moment storage: blocks of 4 warps x 60 columns, these
// rows per thread.
constexpr int MOM_NVAR = 4;
constexpr int MOM_NPT[MOM_NVAR] = {34, 34, 64, 64};  // (NPT + 2) % 3 == 0
constexpr int MOM_MINB[MOM_NVAR] = {4, 5, 4, 5};     // resident blocks per SM (register cap)
constexpr bool MOM_PFL[MOM_NVAR] = {true, true, true, true};  // L2 prefetch of the rows ahead
constexpr int MOM_LD[MOM_NVAR] = {2, 1, 2, 1};       // source rows loaded this many rows ahead
constexpr int TMA_MAX_SMEM = 200 * 1024;  // dynamic shared memory budget of one TMA block
constexpr int TMA_MAX_STAGES = 4;

// Scale of the stored FP16 non-equilibrium moments of the moment storage
// (a power of two: stored = neq_s x value).
constexpr float MOM_NEQ_S = 4096.f;

constexpr int NSUM = 10;  // finish-kernel reduction lanes
enum SumLane : int {
  S_L2 = 0, S_MASS, S_MX, S_MY, S_FX, S_FY, S_DU, S_UU, S_VMAX, S_NAN
};

// Everything a launch needs, passed by value (kernel parameter space).
struct StepArgs {
  int n, m, pitch;
  int model, curved, outlet;
  long long plane;          // elements per population plane
  const uint8_t *cls;
  const uint32_t *aux;      // record index (CLS_SPECIAL) / side-buffer slot (CLS_BULK_REC)
  const BRec *rec;
  void *src;                // population state read
  void *dst;                // population state written (== src for AA)
  double *sb_src, *sb_dst;  // AA side buffers (9 doubles per recorded node)
  double omega, omegaA, rho_out;
  double rho0;              // deviation reference density (16-bit storage)
  float scale[9], inv_scale[9];
  double stmiv[81];         // Minv * diag(s) of MRTInitializer, row-major
  int *err;                 // device error word: set when a bounded wait gives up
  int *nanflag;             // set to 1 by a reduced-precision step that produced a NaN or
                            // infinity (null: no check, the FP64 parity mode and batches)
  int tma_stages;           // ring depth of the TMA step (from the shared-memory budget)
  int tma_tiles_x, tma_tiles_y;
  int pf_blocks;            // paired 16-bit step: L2 prefetch for the block this many launch
                            // positions ahead (a fraction of a wave of resident blocks); 0 = off
  // moment storage (LBM_FP16NEQ)
  float *ss_src, *ss_dst;   // FP32 post-collision deviations of class-3 nodes (9 per record)
  const uint32_t *mlist;    // class-3 and class-2 nodes, updated by the special-node kernel
  int mlist_n;
  float fx_rho, fx_irho;    // fixed-point step of rho - rho0 and its inverse
  float fx_j, fx_ij;        // fixed-point step of j and its inverse
  float fx_irho0;           // 1 / rho0
  float neq_s, neq_is;      // scale of the stored non-equilibrium moments and its inverse
  unsigned gen;             // generation written by this launch (seed of the rounding dither)
  float f_rho0, f_om, f_omA;  // rho0, omega, omegaA in FP32 (moment storage)
  float f_i4rho0;           // 1 / (4 rho0) in FP32 (moment storage)
  float fx_enc[2];          // 64 / fx_rho and 32 / fx_j: the scaled codes of the dithered rounding
  float fx_rlim, fx_jlim;   // largest |rho - rho0| and |j| whose codes stay within the range
  float enc_c[6];           // storage references from codes: 2 S h_r, -3 S h_j^2, -S h_r,
                            // 3 S h_j^2, S h_j, -S h_j^2 / rho0 (S = neq_s, h = fixed-point steps)
  float enc_s[9];           // collision folded into the encoding: 3 S s12, -2 S s12, S s12,
                            // -3 S s12, S (1 - s12), -S s46, S (1 - s46), S om, S (1 - om)
};

// Outputs of the read-only finish kernel (any pointer may be null).
struct FinishOut {
  double *rho, *u, *v;      // n*m, cell-major
  double *f, *metaf;        // 9*n*m, cell-major
  const double *rho_solid;  // values reported for solid cells (set_state)
  const double *u_solid, *v_solid;
  float *uprev, *vprev;     // du_rel reference fields (read, then replaced), n*m
  double *partial;          // NSUM per block
};

}  // namespace lbm
