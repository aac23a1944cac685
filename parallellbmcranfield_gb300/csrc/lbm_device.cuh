// Device code of the fused D2Q9 step: storage policies, collision models,
// boundary handling, and the kernel templates instantiated per precision in
// lbm_kernels_<precision>.cu.
//
// State convention.  The population state between launches is the
// post-collision field METAF_t of the reference cells (serial/CellFunctions.c
// :352-438).  One fused launch performs the tail of serial iteration t
// (UpdateF + StreamingStep + HandleBoundariesStep + UpdateMacroscopicStep,
// serial/Iterate.c:275-294) and the head of iteration t+1 (CollisionStep),
// producing METAF_{t+1}.  The streamed and boundary-treated F_{t+1} and the
// macroscopic fields live only in registers; the read-only finish kernel
// recomputes them when they are asked for.
//
// Arithmetic.  With FP64 storage (R = double) every expression keeps the
// reference's operand order and association; the translation unit is
// compiled with --fmad=false so that no multiply-add is contracted, which
// makes the FP64 mode bit-identical to the serial C code compiled without
// contraction.  With FP32 and 16-bit storage (R = float) the algebraically
// equivalent short forms are used and contraction is allowed.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <type_traits>

#include "lbm_types.h"

namespace lbm {

__device__ __constant__ constexpr int CX[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
__device__ __constant__ constexpr int CY[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
__device__ __constant__ constexpr int OPP[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};

template <class R>
__device__ __forceinline__ R wgt(int k) {
  // D2Q9Vars weights, serial/CellFunctions.c:294-300
  return k == 0 ? R(4. / 9.) : (k < 5 ? R(1. / 9.) : R(1. / 36.));
}

// ------------------------------------------------------------ storage policies

struct StF64 {
  using T = double;
  using R = double;
  static __device__ __forceinline__ R ld(const T *p, int, const StepArgs &) { return __ldg(p); }
  static __device__ __forceinline__ void st(T *p, int, R v, const StepArgs &) { *p = v; }
};

struct StF32 {
  using T = float;
  using R = float;
  static __device__ __forceinline__ R ld(const T *p, int, const StepArgs &) { return __ldg(p); }
  static __device__ __forceinline__ void st(T *p, int, R v, const StepArgs &) { __stcs(p, v); }
};

// 16-bit storage of s_k = (f_k - w_k rho0) * scale_k; arithmetic in FP32.
struct StF16 {
  using T = __half;
  using R = float;
  static __device__ __forceinline__ R ld(const T *p, int k, const StepArgs &a) {
    return fmaf(__half2float(__ldg(p)), a.inv_scale[k], wgt<float>(k) * (float)a.rho0);
  }
  static __device__ __forceinline__ void st(T *p, int k, R v, const StepArgs &a) {
    *p = __float2half_rn((v - wgt<float>(k) * (float)a.rho0) * a.scale[k]);
  }
};

struct StB16 {
  using T = __nv_bfloat16;
  using R = float;
  static __device__ __forceinline__ R ld(const T *p, int k, const StepArgs &a) {
    return fmaf(__bfloat162float(__ldg(p)), a.inv_scale[k], wgt<float>(k) * (float)a.rho0);
  }
  static __device__ __forceinline__ void st(T *p, int k, R v, const StepArgs &a) {
    *p = __float2bfloat16_rn((v - wgt<float>(k) * (float)a.rho0) * a.scale[k]);
  }
};

// Offset of the neighbour x + e_k in linear node index.
__device__ __forceinline__ long long nb(int k, int pitch) {
  return (long long)CX[k] + (long long)CY[k] * pitch;
}

// Slot holding METAF[k](z) in a state of the given layout.
//   PH_AB   : slot k at z
//   PH_AA_A : slot opp(k) at z
//   PH_AA_B : slot k at z + e_k
template <int L>
__device__ __forceinline__ long long slot_of(int k, long long z, const StepArgs &a) {
  if (L == PH_AB) return (long long)k * a.plane + z;
  if (L == PH_AA_A) return (long long)OPP[k] * a.plane + z;
  return (long long)k * a.plane + z + nb(k, a.pitch);
}

// Read METAF[k](z) of the state (solid and padding cells read as 0, as the
// reference's never-collided solid cells do).
template <class ST, int L>
struct AccMain {
  using R = typename ST::R;
  const StepArgs &a;
  const typename ST::T *s;
  __device__ AccMain(const StepArgs &a_, const void *src)
      : a(a_), s((const typename ST::T *)src) {}
  __device__ __forceinline__ R meta(long long z, int k) const {
    if (a.cls[z] == CLS_SOLID) return R(0);
    return ST::ld(s + slot_of<L>(k, z, a), k, a);
  }
};

// AA pattern: METAF of recorded nodes comes from the side buffer of the
// current parity, never from the in-place array another thread rewrites.
template <class ST>
struct AccSide {
  using R = typename ST::R;
  const StepArgs &a;
  __device__ AccSide(const StepArgs &a_, const void *) : a(a_) {}
  __device__ __forceinline__ R meta(long long z, int k) const {
    uint8_t c = a.cls[z];
    if (c == CLS_SOLID) return R(0);
    uint32_t s = a.aux[z];
    if (c == CLS_SPECIAL) s = a.rec[s].sb;
    return (R)a.sb_src[(size_t)s * 9 + k];
  }
};

// ------------------------------------------------------- macroscopic moments

// UpdateMacroscopic, serial/CellFunctions.c:462-481.
template <class R>
__device__ __forceinline__ void moments(const R F[9], R &rho, R &u, R &v) {
  if constexpr (std::is_same<R, double>::value) {
    R S = 0.0;
#pragma unroll
    for (int k = 0; k < 9; k++) S = S + F[k];
    rho = S;
    R Us = 0.0, Vs = 0.0;
#pragma unroll
    for (int k = 0; k < 9; k++) {
      Us = Us + F[k] * CX[k];
      Vs = Vs + F[k] * CY[k];
    }
    u = Us / rho;
    v = Vs / rho;
  } else {
    rho = ((F[0] + F[1]) + (F[2] + F[3])) + ((F[4] + F[5]) + (F[6] + F[7])) + F[8];
    R jx = (F[1] - F[3]) + (F[5] - F[6]) + (F[8] - F[7]);
    R jy = (F[2] - F[4]) + (F[5] - F[7]) + (F[6] - F[8]);
    R inv = R(1) / rho;
    u = jx * inv;
    v = jy * inv;
  }
}

// ----------------------------------------------------------------- collision

// BGKW / TRT equilibrium, serial/CellFunctions.c:355-362 and :374-381.
template <class R>
__device__ __forceinline__ void equilibrium(R rho, R u, R v, R feq[9]) {
  R T1 = u * u + v * v;
#pragma unroll
  for (int k = 0; k < 9; k++) {
    R T2 = u * CX[k] + v * CY[k];
    feq[k] = rho * wgt<R>(k) * (R(1.0) + R(3.0) * T2 + R(4.5) * T2 * T2 - R(1.5) * T1);
  }
}

template <class R>
__device__ __forceinline__ void collide_bgk(const R F[9], R rho, R u, R v, R om, R M[9]) {
  R feq[9];
  equilibrium(rho, u, v, feq);
#pragma unroll
  for (int k = 0; k < 9; k++) {
    if constexpr (std::is_same<R, double>::value)
      M[k] = om * feq[k] + (1.0 - om) * F[k];  // serial/CellFunctions.c:363
    else
      M[k] = fmaf(om, feq[k] - F[k], F[k]);
  }
}

template <class R>
__device__ __forceinline__ void collide_trt(const R F[9], R rho, R u, R v, R om, R omA,
                                            R M[9]) {
  R feq[9];
  equilibrium(rho, u, v, feq);
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const int o = OPP[k];
    if constexpr (std::is_same<R, double>::value) {
      // serial/CellFunctions.c:383-393: the four split terms are float there
      float fp = __double2float_rn(0.5 * (F[k] + F[o]));
      float feqp = __double2float_rn(0.5 * (feq[k] + feq[o]));
      float fm = __double2float_rn(0.5 * (F[k] - F[o]));
      float feqm = __double2float_rn(0.5 * (feq[k] - feq[o]));
      M[k] = F[k] - (double)__fsub_rn(fp, feqp) * om - (double)__fsub_rn(fm, feqm) * omA;
    } else {
      R sp = R(0.5) * ((F[k] + F[o]) - (feq[k] + feq[o]));
      R sm = R(0.5) * ((F[k] - F[o]) - (feq[k] - feq[o]));
      M[k] = F[k] - om * sp - omA * sm;
    }
  }
}

// MRT transform rows (serial/CellFunctions.c:37-47).
__device__ __constant__ constexpr int TMAT[9][9] = {
    {1, 1, 1, 1, 1, 1, 1, 1, 1},     {-4, -1, -1, -1, -1, 2, 2, 2, 2},
    {4, -2, -2, -2, -2, 1, 1, 1, 1}, {0, 1, 0, -1, 0, 1, -1, -1, 1},
    {0, -2, 0, 2, 0, 1, -1, -1, 1},  {0, 0, 1, 0, -1, 1, 1, -1, -1},
    {0, 0, -2, 0, 2, 1, 1, -1, -1},  {0, 1, -1, 1, -1, 0, 0, 0, 0},
    {0, 0, 0, 0, 0, 1, -1, 1, -1}};

template <class R>
__device__ __forceinline__ void collide_mrt(const R F[9], R rho, R u, R v, const StepArgs &a,
                                            R M[9]) {
  if constexpr (std::is_same<R, double>::value) {
    // serial/CellFunctions.c:401-438, same sums in the same order
    double meq[9], mom[9];
    meq[0] = rho;
    meq[1] = rho * (-2.0 + 3.0 * rho * (u * u + v * v));
    meq[2] = rho * (1.0 - 3.0 * rho * (u * u + v * v));
    meq[3] = rho * u;
    meq[4] = -rho * u;
    meq[5] = rho * v;
    meq[6] = -rho * v;
    meq[7] = rho * (u * u - v * v);
    meq[8] = rho * u * v;
#pragma unroll
    for (int k = 0; k < 9; k++) {
      double s = 0.0;
#pragma unroll
      for (int l = 0; l < 9; l++) s = s + (double)TMAT[k][l] * F[l];
      mom[k] = s;
    }
#pragma unroll
    for (int k = 0; k < 9; k++) {
      double s = 0.0;
#pragma unroll
      for (int l = 0; l < 9; l++) s = s + a.stmiv[k * 9 + l] * (mom[l] - meq[l]);
      M[k] = F[k] - s;
    }
  } else {
    // Same operator in moment space with the integer structure of M and Minv
    // exploited: d = S (M f - meq), then f - Minv d with Minv = (1/36) * ints.
    const R om = (R)a.omega;
    const R s12 = R(1.4), s46 = R(1.2);
    R a14 = (F[1] + F[3]) + (F[2] + F[4]);
    R a58 = (F[5] + F[7]) + (F[6] + F[8]);
    R m0 = (F[0] + a14) + a58;
    R m1 = -R(4) * F[0] - a14 + R(2) * a58;
    R m2 = R(4) * F[0] - R(2) * a14 + a58;
    R d13 = F[1] - F[3], d24 = F[2] - F[4];
    R x58 = (F[5] - F[7]) + (F[8] - F[6]);  // f5 - f6 - f7 + f8
    R y58 = (F[5] - F[7]) + (F[6] - F[8]);  // f5 + f6 - f7 - f8
    R m3 = d13 + x58, m4 = -R(2) * d13 + x58;
    R m5 = d24 + y58, m6 = -R(2) * d24 + y58;
    R m7 = (F[1] + F[3]) - (F[2] + F[4]);
    R m8 = (F[5] + F[7]) - (F[6] + F[8]);
    R q = u * u + v * v;
    R d0 = m0 - rho;
    R d1 = s12 * (m1 - rho * (R(-2) + R(3) * rho * q));
    R d2 = s12 * (m2 - rho * (R(1) - R(3) * rho * q));
    R ru = rho * u, rv = rho * v;
    R d3 = m3 - ru;
    R d4 = s46 * (m4 + ru);
    R d5 = m5 - rv;
    R d6 = s46 * (m6 + rv);
    R d7 = om * (m7 - rho * (u * u - v * v));
    R d8 = om * (m8 - ru * v);
    const R c = R(1.0 / 36.0);
    R ax = R(4) * d0 - d1 - R(2) * d2;
    R dg = R(4) * d0 + R(2) * d1 + d2;
    R X = R(6) * (d3 - d4), Y = R(6) * (d5 - d6), P = R(9) * d7;
    R Xd = R(6) * d3 + R(3) * d4, Yd = R(6) * d5 + R(3) * d6, Q = R(9) * d8;
    M[0] = F[0] - c * (R(4) * ((d0 - d1) + d2));
    M[1] = F[1] - c * (ax + X + P);
    M[2] = F[2] - c * (ax + Y - P);
    M[3] = F[3] - c * (ax - X + P);
    M[4] = F[4] - c * (ax - Y - P);
    M[5] = F[5] - c * (dg + Xd + Yd + Q);
    M[6] = F[6] - c * (dg - Xd + Yd - Q);
    M[7] = F[7] - c * (dg - Xd - Yd + Q);
    M[8] = F[8] - c * (dg + Xd - Yd - Q);
  }
}

template <int MODEL, class R>
__device__ __forceinline__ void collide(const R F[9], R rho, R u, R v, const StepArgs &a,
                                        R M[9]) {
  if (MODEL == 1) collide_bgk<R>(F, rho, u, v, (R)a.omega, M);
  else if (MODEL == 2) collide_trt<R>(F, rho, u, v, (R)a.omega, (R)a.omegaA, M);
  else collide_mrt<R>(F, rho, u, v, a, M);
}

// ------------------------------------------------------ boundary conditions

// F of a special node after streaming and the inlet / wall treatments of
// HandleBoundariesStep (serial/Iterate.c:495-523), plus its outlet treatment
// when OUTLET is set (serial/Iterate.c:525-546).  Any node class is accepted:
// solid returns 0 (UpdateF copied the never-written METAF), bulk returns the
// plain pull.  `acc` reads METAF of the current state.
template <bool OUTLET, class R, class ACC>
__device__ void boundary_F(const StepArgs &a, const ACC &acc, long long node, R F[9]);

template <class R, class ACC>
__device__ __noinline__ void boundary_F_noout(const StepArgs &a, const ACC &acc, long long node,
                                              R F[9]) {
  boundary_F<false, R, ACC>(a, acc, node, F);
}

template <bool OUTLET, class R, class ACC>
__device__ void boundary_F(const StepArgs &a, const ACC &acc, long long node, R F[9]) {
  const uint8_t c = a.cls[node];
  if (c == CLS_SOLID) {
#pragma unroll
    for (int k = 0; k < 9; k++) F[k] = R(0);
    return;
  }
  if (c != CLS_SPECIAL) {
#pragma unroll
    for (int k = 0; k < 9; k++) F[k] = acc.meta(node - nb(k, a.pitch), k);
    return;
  }
  const BRec &r = a.rec[a.aux[node]];
  const uint32_t fl = r.flags;
  // StreamingStep, serial/Iterate.c:478-484 (F = own METAF where not streamed)
#pragma unroll
  for (int k = 0; k < 9; k++)
    F[k] = ((fl >> (FL_STREAM_SHIFT + k)) & 1u) ? acc.meta(node - nb(k, a.pitch), k)
                                                 : acc.meta(node, k);
  const R uo = (R)r.uo;
  // InletBC, serial/BoundaryConditions.c:25-50
  if (fl & FL_LID) {
    R rhoN = F[0] + F[1] + F[3] + R(2) * (F[2] + F[6] + F[5]);
    F[4] = F[2];
    F[8] = F[6] + rhoN * uo / R(6.0);
    F[7] = F[5] - rhoN * uo / R(6.0);
  }
  if (fl & FL_WEST) {
    R rhoW = (F[0] + F[2] + F[4] + R(2.0) * (F[3] + F[6] + F[7])) / (R(1.0) - uo);
    F[1] = F[3] + R(2) * rhoW * uo / R(3);
    F[5] = F[7] + rhoW * uo / R(6);
    F[8] = F[6] + rhoW * uo / R(6);
  }
  const uint32_t wall = (fl >> FL_WALL_SHIFT) & 0x1FFu;
  if (a.curved == 1) {
    // CurvedWallBoundaries, serial/BoundaryConditions.c:127-146
#pragma unroll
    for (int k = 1; k < 9; k++) {
      if (!((wall >> k) & 1u)) continue;
      const R q = (R)r.q[k];
      const int o = OPP[k];
      if (q < R(0.5)) {
        R fnb = acc.meta(node - nb(k, a.pitch), k);
        F[o] = R(2) * q * acc.meta(node, k) + (R(1) - R(2) * q) * fnb;
      } else {
        F[o] = acc.meta(node, k) / R(2) / q + (R(2) * q - R(1)) / (R(2) * q) * acc.meta(node, o);
      }
    }
  } else if (a.curved == 2) {
    // WallBC, serial/BoundaryConditions.c:109-115 (sequential, in place)
#pragma unroll
    for (int k = 1; k < 9; k++)
      if ((wall >> k) & 1u) F[OPP[k]] = F[k];
  }
  if (OUTLET && (fl & FL_EAST)) {
    if (a.outlet == 1) {
      // OutletBoundaries, serial/BoundaryConditions.c:70-81
      R rhoE = (F[0] + F[2] + F[4] + R(2.0) * (F[1] + F[5] + F[8])) / (R(1) - uo);
      F[3] = F[1] - R(2) * rhoE * uo / R(3.0);
      F[7] = F[5] - rhoE * uo / R(6.0);
      F[6] = F[8] - rhoE * uo / R(6.0);
    } else if (a.outlet == 2) {
      // 2nd-order extrapolation from the already treated i-1, i-2 cells,
      // serial/Iterate.c:535-541
      R A[9], B[9];
      boundary_F_noout<R, ACC>(a, acc, node - 1, A);
      boundary_F_noout<R, ACC>(a, acc, node - 2, B);
      F[1] = R(2) * (A[1]) - B[1];
      F[5] = R(2) * (A[5]) - B[5];
      F[8] = R(2) * (A[8]) - B[8];
    } else if (a.outlet == 4) {
      // constant-pressure east outlet (Zou-He density condition; not in the reference)
      const R ro = (R)a.rho_out;
      R ux = R(-1.0) + (F[0] + F[2] + F[4] + R(2.0) * (F[1] + F[5] + F[8])) / ro;
      R ru = ro * ux;
      R d24 = R(0.5) * (F[2] - F[4]);
      F[3] = F[1] - (R(2.0) / R(3.0)) * ru;
      F[7] = F[5] + d24 - ru / R(6.0);
      F[6] = F[8] - d24 - ru / R(6.0);
    }
  }
}

// Full treatment of a special node as one out-of-line call (keeps the bulk
// path's register budget small).  Returns F and the macroscopic fields
// (V = 0 on east-outlet cells, serial/CellFunctions.c:483-486).
template <class R, class ACC>
__device__ __noinline__ void special_node(const StepArgs &a, const ACC &acc, long long node,
                                          R F[9], R *mac) {
  boundary_F<true, R, ACC>(a, acc, node, F);
  R rho, u, v;
  moments<R>(F, rho, u, v);
  if (a.rec[a.aux[node]].flags & FL_EAST) v = R(0.0);
  mac[0] = rho;
  mac[1] = u;
  mac[2] = v;
}

// ------------------------------------------------------------------- kernels

__device__ __forceinline__ bool node_xy(const StepArgs &a, int &x, int &y) {
  x = blockIdx.x * blockDim.x + threadIdx.x;
  y = blockIdx.y;
  return x < a.n;
}

// Fused step: METAF_t (layout PH) -> METAF_{t+1}.
template <class ST, int MODEL, int PH>
__global__ void __launch_bounds__(128) k_step(const __grid_constant__ StepArgs a) {
  using R = typename ST::R;
  using T = typename ST::T;
  int x, y;
  if (!node_xy(a, x, y)) return;
  const long long node = (long long)y * a.pitch + x;
  const uint8_t c = a.cls[node];
  if (c == CLS_SOLID) return;
  const T *s = (const T *)a.src;
  T *d = (T *)a.dst;
  R F[9], rho, u, v;
  if (c != CLS_SPECIAL) {
#pragma unroll
    for (int k = 0; k < 9; k++) {
      long long i;
      if (PH == PH_AB) i = (long long)k * a.plane + node - nb(k, a.pitch);
      else if (PH == PH_AA_A) i = (long long)OPP[k] * a.plane + node - nb(k, a.pitch);
      else i = (long long)k * a.plane + node;
      F[k] = ST::ld(s + i, k, a);
    }
    moments<R>(F, rho, u, v);
  } else {
    R mac[3];
    if (PH == PH_AB) special_node<R>(a, AccMain<ST, PH_AB>(a, a.src), node, F, mac);
    else special_node<R>(a, AccSide<ST>(a, nullptr), node, F, mac);
    rho = mac[0];
    u = mac[1];
    v = mac[2];
  }
  R M[9];
  collide<MODEL, R>(F, rho, u, v, a, M);
#pragma unroll
  for (int k = 0; k < 9; k++) {
    long long i;
    if (PH == PH_AB) i = (long long)k * a.plane + node;
    else if (PH == PH_AA_A) i = (long long)k * a.plane + node + nb(k, a.pitch);
    else i = (long long)OPP[k] * a.plane + node;
    ST::st(d + i, k, M[k], a);
  }
  if (PH != PH_AB && c != CLS_BULK) {
    uint32_t sbi = a.aux[node];
    if (c == CLS_SPECIAL) sbi = a.rec[sbi].sb;
#pragma unroll
    for (int k = 0; k < 9; k++) a.sb_dst[(size_t)sbi * 9 + k] = (double)M[k];
  }
}

// First collision after lbm_set_state: METAF = Coll(F0, rho0, u0, v0) on
// fluid cells, written in layout AB (dst) or AA-A; side buffer for AA.
template <class ST, int MODEL, int PH>
__global__ void __launch_bounds__(128) k_init(const __grid_constant__ StepArgs a, const double *f0,
                                              const double *rho0, const double *u0,
                                              const double *v0) {
  using R = typename ST::R;
  using T = typename ST::T;
  int x, y;
  if (!node_xy(a, x, y)) return;
  const long long node = (long long)y * a.pitch + x;
  const long long cell = (long long)y * a.n + x;
  const uint8_t c = a.cls[node];
  T *d = (T *)a.dst;
  R F[9], M[9];
  R rho = (R)rho0[cell], u = (R)u0[cell], v = (R)v0[cell];
  if (f0) {
#pragma unroll
    for (int k = 0; k < 9; k++) F[k] = (R)f0[cell * 9 + k];
  } else {
    R feq[9];
    equilibrium<R>(rho, u, v, feq);
#pragma unroll
    for (int k = 0; k < 9; k++) F[k] = feq[k];
  }
  if (c == CLS_SOLID) {
#pragma unroll
    for (int k = 0; k < 9; k++) M[k] = R(0);
  } else {
    collide<MODEL, R>(F, rho, u, v, a, M);
  }
  if (c == CLS_SOLID && PH != PH_AB) return;  // AA: solid slots belong to the neighbours
#pragma unroll
  for (int k = 0; k < 9; k++) {
    long long i = (PH == PH_AB) ? (long long)k * a.plane + node : (long long)OPP[k] * a.plane + node;
    ST::st(d + i, k, M[k], a);
  }
  if (PH != PH_AB && c != CLS_BULK && c != CLS_SOLID) {
    uint32_t sbi = a.aux[node];
    if (c == CLS_SPECIAL) sbi = a.rec[sbi].sb;
#pragma unroll
    for (int k = 0; k < 9; k++) a.sb_dst[(size_t)sbi * 9 + k] = (double)M[k];
  }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Block reduction of NSUM lanes into partial[block * NSUM + lane]
// (fixed order: deterministic for a fixed launch shape).
__device__ __forceinline__ void block_reduce_store(double acc[NSUM], double *partial) {
  __shared__ double sh[NSUM][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int i = 0; i < NSUM; i++) {
    double v = (i == S_VMAX) ? warp_max(acc[i]) : warp_sum(acc[i]);
    if (lane == 0) sh[i][wid] = v;
  }
  __syncthreads();
  if (threadIdx.x < NSUM) {
    const int i = threadIdx.x;
    double v = (i == S_VMAX) ? 0.0 : 0.0;
    for (int w = 0; w < nw; w++) v = (i == S_VMAX) ? fmax(v, sh[i][w]) : v + sh[i][w];
    partial[((size_t)blockIdx.y * gridDim.x + blockIdx.x) * NSUM + i] = v;
  }
}

// Read-only: F_{t+1}, macroscopic fields and FP64 diagnostics from METAF_t.
template <class ST, int L>
__global__ void __launch_bounds__(128) k_finish(const __grid_constant__ StepArgs a, const FinishOut o) {
  using R = typename ST::R;
  int x = blockIdx.x * blockDim.x + threadIdx.x;
  int y = blockIdx.y;
  double acc[NSUM];
#pragma unroll
  for (int i = 0; i < NSUM; i++) acc[i] = 0.0;
  if (x < a.n) {
    const long long node = (long long)y * a.pitch + x;
    const long long cell = (long long)y * a.n + x;
    const uint8_t c = a.cls[node];
    AccMain<ST, L> acc_m(a, a.src);
    if (c == CLS_SOLID) {
      if (o.f)
        for (int k = 0; k < 9; k++) o.f[cell * 9 + k] = 0.0;
      if (o.metaf)
        for (int k = 0; k < 9; k++) o.metaf[cell * 9 + k] = 0.0;
      if (o.rho) o.rho[cell] = o.rho_solid[cell];
      if (o.u) o.u[cell] = o.u_solid[cell];
      if (o.v) o.v[cell] = o.v_solid[cell];
    } else {
      R F[9], rho, u, v;
      if (c != CLS_SPECIAL) {
        boundary_F<false, R>(a, acc_m, node, F);
        moments<R>(F, rho, u, v);
      } else {
        R mac[3];
        special_node<R>(a, acc_m, node, F, mac);
        rho = mac[0];
        u = mac[1];
        v = mac[2];
      }
      double l2 = 0.0;
#pragma unroll
      for (int k = 0; k < 9; k++) {
        double mk = (double)acc_m.meta(node, k);
        double dk = (double)F[k] - mk;
        l2 += dk * dk;
        if (o.f) o.f[cell * 9 + k] = (double)F[k];
        if (o.metaf) o.metaf[cell * 9 + k] = mk;
      }
      if (o.rho) o.rho[cell] = (double)rho;
      if (o.u) o.u[cell] = (double)u;
      if (o.v) o.v[cell] = (double)v;
      const double dr = rho, du = u, dv = v;
      acc[S_L2] = l2;
      acc[S_MASS] = dr;
      acc[S_MX] = dr * du;
      acc[S_MY] = dr * dv;
      acc[S_UU] = du * du + dv * dv;
      acc[S_VMAX] = sqrt(du * du + dv * dv);
      acc[S_NAN] = (dr != dr || du != du || dv != dv) ? 1.0 : 0.0;
      if (o.uprev) {
        double pu = o.uprev[cell], pv = o.vprev[cell];
        acc[S_DU] = (du - pu) * (du - pu) + (dv - pv) * (dv - pv);
        o.uprev[cell] = (float)du;
        o.vprev[cell] = (float)dv;
      }
      if (c == CLS_SPECIAL) {
        const BRec &r = a.rec[a.aux[node]];
        if (r.flags & FL_DRAG) {
          // momentum exchange over the wall links of this cell
          const uint32_t wall = (r.flags >> FL_WALL_SHIFT) & 0x1FFu;
          for (int k = 1; k < 9; k++)
            if ((wall >> k) & 1u) {
              double g = (double)acc_m.meta(node, k) + (double)F[OPP[k]];
              acc[S_FX] += g * CX[k];
              acc[S_FY] += g * CY[k];
            }
        }
      }
    }
  }
  block_reduce_store(acc, o.partial);
}

// Sum the per-block partials in a fixed order (one block of 32*NSUM threads).
static __global__ void k_reduce_partials(const double *partial, int nblocks, double *out) {
  const int lane = threadIdx.x & 31, i = threadIdx.x >> 5;
  if (i >= NSUM) return;
  double v = 0.0;
  for (int b = lane; b < nblocks; b += 32) {
    double p = partial[(size_t)b * NSUM + i];
    v = (i == S_VMAX) ? fmax(v, p) : v + p;
  }
  v = (i == S_VMAX) ? warp_max(v) : warp_sum(v);
  if (lane == 0) out[i] = v;
}

// The serial residual (serial/ComputeResiduals.c:6-51) with its index quirk:
// only cells 0..m-1 (reference numbering j*n+i) are visited, each n times.
// One block; writes L2, L2_weighted, Drag, Lift to out[0..3].
template <class ST, int L>
__global__ void __launch_bounds__(256) k_resid_ref(const __grid_constant__ StepArgs a, double *out) {
  using R = typename ST::R;
  __shared__ double sh[3][256];
  AccMain<ST, L> acc_m(a, a.src);
  double s2 = 0.0, sd = 0.0, sl = 0.0;
  for (int c = threadIdx.x; c < a.m; c += blockDim.x) {
    const int x = c % a.n, y = c / a.n;
    const long long node = (long long)y * a.pitch + x;
    const uint8_t cl = a.cls[node];
    if (cl == CLS_SOLID) continue;  // F = METAF = 0, DragF = 0
    R F[9], rho, u, v;
    if (cl != CLS_SPECIAL) {
      boundary_F<false, R>(a, acc_m, node, F);
      moments<R>(F, rho, u, v);
    } else {
      R mac[3];
      special_node<R>(a, acc_m, node, F, mac);
      rho = mac[0];
      const BRec &r = a.rec[a.aux[node]];
      if (r.flags & FL_DRAG) {
        sd += (double)rho / 3 * (20 - r.x) / 5;
        sl += (double)rho / 3 * (20 - r.y) / 5;
      }
    }
    for (int k = 0; k < 9; k++) {
      double dk = (double)F[k] - (double)acc_m.meta(node, k);
      s2 += dk * dk;
    }
  }
  sh[0][threadIdx.x] = s2;
  sh[1][threadIdx.x] = sd;
  sh[2][threadIdx.x] = sl;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t2 = 0.0, td = 0.0, tl = 0.0;
    for (int i = 0; i < (int)blockDim.x; i++) {
      t2 += sh[0][i];
      td += sh[1][i];
      tl += sh[2][i];
    }
    const double nn = (double)a.n;
    const double L2sq = t2 * nn;
    out[0] = sqrt(L2sq);
    out[1] = sqrt(L2sq / (double)(a.m * a.n));
    out[2] = td * nn;
    out[3] = tl * nn;
  }
}

}  // namespace lbm
