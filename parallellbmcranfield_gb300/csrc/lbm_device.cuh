// Device code of the fused D2Q9 step: storage policies, collision models,
// boundary handling, and the kernel templates instantiated per precision and
// collision model by lbm_kernels_inst.cu (compiled once per combination).
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

#include <cstring>
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

// Each policy gives absolute populations (cvt / pack / ld / st, used by the
// boundary paths and the read-back) and, for the bulk path, populations in
// the form its arithmetic uses (cvt_dev / pack_dev / ld_dev / st_dev): with
// SHIFT the deviations f_k - w_k rho0 ("DDF shifting"), which keeps the
// rounding of FP32 arithmetic and of 16-bit storage relative to the small
// deviations instead of to f ~ w_k rho0.  FP64 (the parity mode) stays absolute.
struct StF64 {
  using T = double;
  using R = double;
  static constexpr bool SHIFT = false;
  static __device__ __forceinline__ R cvt(T v, int, const StepArgs &) { return v; }
  static __device__ __forceinline__ T pack(R v, int, const StepArgs &) { return v; }
  static __device__ __forceinline__ R ld(const T *p, int, const StepArgs &) { return __ldg(p); }
  static __device__ __forceinline__ void st(T *p, int, R v, const StepArgs &) { *p = v; }
  static __device__ __forceinline__ R cvt_dev(T v, int k, const StepArgs &a) { return cvt(v, k, a); }
  static __device__ __forceinline__ T pack_dev(R v, int k, const StepArgs &a) { return pack(v, k, a); }
};

// FP32 storage of d_k = f_k - w_k rho0.
struct StF32 {
  using T = float;
  using R = float;
  static constexpr bool SHIFT = true;
  static __device__ __forceinline__ R cvt(T v, int k, const StepArgs &a) {
    return v + wgt<float>(k) * (float)a.rho0;
  }
  static __device__ __forceinline__ T pack(R v, int k, const StepArgs &a) {
    return v - wgt<float>(k) * (float)a.rho0;
  }
  static __device__ __forceinline__ R ld(const T *p, int k, const StepArgs &a) {
    return cvt(__ldg(p), k, a);
  }
  static __device__ __forceinline__ void st(T *p, int k, R v, const StepArgs &a) {
    __stcs(p, pack(v, k, a));
  }
  static __device__ __forceinline__ R cvt_dev(T v, int, const StepArgs &) { return v; }
  static __device__ __forceinline__ T pack_dev(R v, int, const StepArgs &) { return v; }
};

// 16-bit storage of s_k = (f_k - w_k rho0) * scale_k; arithmetic in FP32.
struct StF16 {
  using T = __half;
  using R = float;
  static constexpr bool SHIFT = true;
  static __device__ __forceinline__ R cvt(T v, int k, const StepArgs &a) {
    return fmaf(__half2float(v), a.inv_scale[k], wgt<float>(k) * (float)a.rho0);
  }
  static __device__ __forceinline__ T pack(R v, int k, const StepArgs &a) {
    return __float2half_rn((v - wgt<float>(k) * (float)a.rho0) * a.scale[k]);
  }
  static __device__ __forceinline__ R ld(const T *p, int k, const StepArgs &a) {
    return cvt(__ldg(p), k, a);
  }
  static __device__ __forceinline__ void st(T *p, int k, R v, const StepArgs &a) { *p = pack(v, k, a); }
  static __device__ __forceinline__ R cvt_dev(T v, int k, const StepArgs &a) {
    return __half2float(v) * a.inv_scale[k];
  }
  static __device__ __forceinline__ T pack_dev(R v, int k, const StepArgs &a) {
    return __float2half_rn(v * a.scale[k]);
  }
};

struct StB16 {
  using T = __nv_bfloat16;
  using R = float;
  static constexpr bool SHIFT = true;
  static __device__ __forceinline__ R cvt(T v, int k, const StepArgs &a) {
    return fmaf(__bfloat162float(v), a.inv_scale[k], wgt<float>(k) * (float)a.rho0);
  }
  static __device__ __forceinline__ T pack(R v, int k, const StepArgs &a) {
    return __float2bfloat16_rn((v - wgt<float>(k) * (float)a.rho0) * a.scale[k]);
  }
  static __device__ __forceinline__ R ld(const T *p, int k, const StepArgs &a) {
    return cvt(__ldg(p), k, a);
  }
  static __device__ __forceinline__ void st(T *p, int k, R v, const StepArgs &a) { *p = pack(v, k, a); }
  static __device__ __forceinline__ R cvt_dev(T v, int k, const StepArgs &a) {
    return __bfloat162float(v) * a.inv_scale[k];
  }
  static __device__ __forceinline__ T pack_dev(R v, int k, const StepArgs &a) {
    return __float2bfloat16_rn(v * a.scale[k]);
  }
};

// Aligned loads / streaming stores of V consecutive elements as 4..16-byte words.
template <class T, int V>
struct VecIO {
  static constexpr int B = (int)sizeof(T) * V;
  static_assert(B == 2 || B == 4 || B == 8 || B % 16 == 0, "vector width");
  static __device__ __forceinline__ void load(const T *p, T out[V]) {
    if constexpr (B == 2) {
      unsigned short r = __ldg((const unsigned short *)p);
      memcpy(out, &r, 2);
    } else if constexpr (B == 4) {
      unsigned r = __ldg((const unsigned *)p);
      memcpy(out, &r, 4);
    } else if constexpr (B == 8) {
      uint2 r = __ldg((const uint2 *)p);
      memcpy(out, &r, 8);
    } else {
#pragma unroll
      for (int i = 0; i < B / 16; i++) {
        uint4 r = __ldg((const uint4 *)p + i);
        memcpy((char *)out + 16 * i, &r, 16);
      }
    }
  }
  static __device__ __forceinline__ void store(T *p, const T in[V]) {
    if constexpr (B == 2) {
      unsigned short r;
      memcpy(&r, in, 2);
      __stcs((unsigned short *)p, r);
    } else if constexpr (B == 4) {
      unsigned r;
      memcpy(&r, in, 4);
      __stcs((unsigned *)p, r);
    } else if constexpr (B == 8) {
      uint2 r;
      memcpy(&r, in, 8);
      __stcs((uint2 *)p, r);
    } else {
#pragma unroll
      for (int i = 0; i < B / 16; i++) {
        uint4 r;
        memcpy(&r, (const char *)in + 16 * i, 16);
        __stcs((uint4 *)p + i, r);
      }
    }
  }
};

// Bulk-form load / streaming store of one population.
template <class ST>
__device__ __forceinline__ typename ST::R ld_dev(const typename ST::T *p, int k,
                                                 const StepArgs &a) {
  return ST::cvt_dev(__ldg(p), k, a);
}
template <class ST>
__device__ __forceinline__ void st_dev(typename ST::T *p, int k, typename ST::R v,
                                       const StepArgs &a) {
  if constexpr (sizeof(typename ST::T) == 2) {
    *p = ST::pack_dev(v, k, a);
  } else {
    __stcs(p, ST::pack_dev(v, k, a));
  }
}

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
// reference's never-collided solid cells do).  With DEV the value comes back
// as the deviation METAF - w_k rho0 (a solid cell's 0 becomes -w_k rho0).
template <class ST, int L, bool DEV = false>
struct AccMain {
  using R = typename ST::R;
  static constexpr bool dev = DEV;
  const StepArgs &a;
  const typename ST::T *s;
  __device__ AccMain(const StepArgs &a_, const void *src)
      : a(a_), s((const typename ST::T *)src) {}
  __device__ __forceinline__ R meta(long long z, int k) const {
    if (a.cls[z] == CLS_SOLID) return DEV ? -wgt<R>(k) * (R)a.rho0 : R(0);
    const typename ST::T *p = s + slot_of<L>(k, z, a);
    return DEV ? ST::cvt_dev(__ldg(p), k, a) : ST::ld(p, k, a);
  }
};

// AA pattern: METAF of recorded nodes comes from the side buffer of the
// current parity, never from the in-place array another thread rewrites.
template <class ST, bool DEV = false>
struct AccSide {
  using R = typename ST::R;
  static constexpr bool dev = DEV;
  const StepArgs &a;
  __device__ AccSide(const StepArgs &a_, const void *) : a(a_) {}
  __device__ __forceinline__ R meta(long long z, int k) const {
    uint8_t c = a.cls[z];
    if (c == CLS_SOLID) return DEV ? -wgt<R>(k) * (R)a.rho0 : R(0);
    uint32_t s = a.aux[z];
    if (c == CLS_SPECIAL) s = a.rec[s].sb;
    const double v = a.sb_src[(size_t)s * 9 + k];
    return DEV ? (R)(v - wgt<double>(k) * a.rho0) : (R)v;
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

// Moments of populations in the storage's bulk form (deviations for the
// shifted storages: rho = rho0 + sum d, j = sum c d; absolute otherwise).
template <class ST>
__device__ __forceinline__ void moments_form(const typename ST::R F[9], const StepArgs &a,
                                             typename ST::R &rho, typename ST::R &u,
                                             typename ST::R &v) {
  using R = typename ST::R;
  if constexpr (ST::SHIFT) {
    R rt = ((F[0] + F[1]) + (F[2] + F[3])) + ((F[4] + F[5]) + (F[6] + F[7])) + F[8];
    R jx = (F[1] - F[3]) + (F[5] - F[6]) + (F[8] - F[7]);
    R jy = (F[2] - F[4]) + (F[5] - F[7]) + (F[6] - F[8]);
    rho = (R)a.rho0 + rt;
    R inv = R(1) / rho;
    u = jx * inv;
    v = jy * inv;
  } else {
    moments<R>(F, rho, u, v);
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

// Divergence flag of the reduced-precision steps.  A NaN or infinity in any
// population a node pulls reaches its M[0] (every collision operator forms
// M[0] from rho and j, which sum all nine), so one compare per node finds it
// and one plain store records it; nothing else is read or written.
__device__ __forceinline__ void flag_nonfinite(const StepArgs &a, float m0) {
  if (!(fabsf(m0) <= 3.0e38f) && a.nanflag) *a.nanflag = 1;
}

// Moments plus collision of a node without boundary work.  In FP32 the MRT
// operator takes rho, j from its own moment transform (rho = m0, j = m3, m5)
// so the conserved moments relax by exactly zero and need no work; rho^2 q is
// formed as |j|^2.  FP64 keeps the reference's two-pass arithmetic.
template <int MODEL, class R>
__device__ __forceinline__ void collide_bulk(const R F[9], const StepArgs &a, R M[9]) {
  if constexpr (MODEL == 3 && !std::is_same<R, double>::value) {
    const R om = (R)a.omega;
    R a13 = F[1] + F[3], a24 = F[2] + F[4];
    R a14 = a13 + a24;
    R p57 = F[5] + F[7], p68 = F[6] + F[8];
    R a58 = p57 + p68;
    R rho = (F[0] + a14) + a58;
    R m1 = R(2) * a58 - a14 - R(4) * F[0];
    R m2 = (R(4) * F[0] + a58) - R(2) * a14;
    R d13 = F[1] - F[3], d24 = F[2] - F[4];
    R e57 = F[5] - F[7], e86 = F[8] - F[6];
    R x58 = e57 + e86, y58 = e57 - e86;
    R jx = d13 + x58, jy = d24 + y58;
    R m4 = x58 - R(2) * d13, m6 = y58 - R(2) * d24;
    R m7 = a13 - a24, m8 = p57 - p68;
    R inv = R(1) / rho;
    R jj = jx * jx + jy * jy;
    R d1 = R(1.4) * (m1 + R(2) * rho - R(3) * jj);
    R d2 = R(1.4) * (m2 - rho + R(3) * jj);
    R d4 = R(1.2) * (m4 + jx);
    R d6 = R(1.2) * (m6 + jy);
    R d7 = om * (m7 - (jx * jx - jy * jy) * inv);
    R d8 = om * (m8 - jx * jy * inv);
    const R c = R(1.0 / 36.0);
    R ax = -d1 - R(2) * d2;
    R dg = R(2) * d1 + d2;
    R X = R(-6) * d4, Y = R(-6) * d6, P = R(9) * d7;
    R Xd = R(3) * d4, Yd = R(3) * d6, Q = R(9) * d8;
    M[0] = F[0] - c * (R(4) * (d2 - d1));
    M[1] = F[1] - c * (ax + X + P);
    M[2] = F[2] - c * (ax + Y - P);
    M[3] = F[3] - c * (ax - X + P);
    M[4] = F[4] - c * (ax - Y - P);
    M[5] = F[5] - c * (dg + Xd + Yd + Q);
    M[6] = F[6] - c * (dg - Xd + Yd - Q);
    M[7] = F[7] - c * (dg - Xd - Yd + Q);
    M[8] = F[8] - c * (dg + Xd - Yd - Q);
  } else {
    R rho, u, v;
    moments<R>(F, rho, u, v);
    collide<MODEL, R>(F, rho, u, v, a, M);
  }
}

// Bulk collision in the storage's bulk form: FP64 absolute (collide_bulk
// above, the reference's arithmetic); the shifted storages take and return
// deviations d_k = f_k - w_k rho0.  With rho~ = sum d (= rho - rho0) and
// j = sum c d, the operators are the same as on f: the MRT rows 1, 2 see
// M w = (1, -2, 1, 0, ...) so m1 + 2 rho becomes m1(d) + 2 rho~ and
// m2 - rho becomes m2(d) - rho~; BGK/TRT use f_eq - w rho0 =
// w (rho~ + rho (3 c.u + 4.5 (c.u)^2 - 1.5 u^2)).
template <int MODEL, class ST>
__device__ __forceinline__ void collide_bulk_dev(const typename ST::R F[9], const StepArgs &a,
                                                 typename ST::R M[9]) {
  using R = typename ST::R;
  if constexpr (!ST::SHIFT) {
    collide_bulk<MODEL, R>(F, a, M);
  } else if constexpr (MODEL == 3) {
    const R om = (R)a.omega;
    R a13 = F[1] + F[3], a24 = F[2] + F[4];
    R a14 = a13 + a24;
    R p57 = F[5] + F[7], p68 = F[6] + F[8];
    R a58 = p57 + p68;
    R rt = (F[0] + a14) + a58;
    R rho = (R)a.rho0 + rt;
    R m1 = R(2) * a58 - a14 - R(4) * F[0];
    R m2 = (R(4) * F[0] + a58) - R(2) * a14;
    R d13 = F[1] - F[3], d24 = F[2] - F[4];
    R e57 = F[5] - F[7], e86 = F[8] - F[6];
    R x58 = e57 + e86, y58 = e57 - e86;
    R jx = d13 + x58, jy = d24 + y58;
    R m4 = x58 - R(2) * d13, m6 = y58 - R(2) * d24;
    R m7 = a13 - a24, m8 = p57 - p68;
    R inv = R(1) / rho;
    R jj = jx * jx + jy * jy;
    R d1 = R(1.4) * (m1 + R(2) * rt - R(3) * jj);
    R d2 = R(1.4) * (m2 - rt + R(3) * jj);
    R d4 = R(1.2) * (m4 + jx);
    R d6 = R(1.2) * (m6 + jy);
    R d7 = om * (m7 - (jx * jx - jy * jy) * inv);
    R d8 = om * (m8 - jx * jy * inv);
    const R c = R(1.0 / 36.0);
    R ax = -d1 - R(2) * d2;
    R dg = R(2) * d1 + d2;
    R X = R(-6) * d4, Y = R(-6) * d6, P = R(9) * d7;
    R Xd = R(3) * d4, Yd = R(3) * d6, Q = R(9) * d8;
    M[0] = F[0] - c * (R(4) * (d2 - d1));
    M[1] = F[1] - c * (ax + X + P);
    M[2] = F[2] - c * (ax + Y - P);
    M[3] = F[3] - c * (ax - X + P);
    M[4] = F[4] - c * (ax - Y - P);
    M[5] = F[5] - c * (dg + Xd + Yd + Q);
    M[6] = F[6] - c * (dg - Xd + Yd - Q);
    M[7] = F[7] - c * (dg - Xd - Yd + Q);
    M[8] = F[8] - c * (dg + Xd - Yd - Q);
    flag_nonfinite(a, M[0]);
  } else {
    R rt = ((F[0] + F[1]) + (F[2] + F[3])) + ((F[4] + F[5]) + (F[6] + F[7])) + F[8];
    R jx = (F[1] - F[3]) + (F[5] - F[6]) + (F[8] - F[7]);
    R jy = (F[2] - F[4]) + (F[5] - F[7]) + (F[6] - F[8]);
    R rho = (R)a.rho0 + rt;
    R inv = R(1) / rho;
    R u = jx * inv, v = jy * inv;
    R T1 = u * u + v * v;
    R feq[9];
#pragma unroll
    for (int k = 0; k < 9; k++) {
      R T2 = u * CX[k] + v * CY[k];
      feq[k] = wgt<R>(k) * (rt + rho * (R(3) * T2 + R(4.5) * T2 * T2 - R(1.5) * T1));
    }
    if (MODEL == 1) {
      const R om = (R)a.omega;
#pragma unroll
      for (int k = 0; k < 9; k++) M[k] = fmaf(om, feq[k] - F[k], F[k]);
    } else {
      const R om = (R)a.omega, omA = (R)a.omegaA;
#pragma unroll
      for (int k = 0; k < 9; k++) {
        const int o = OPP[k];
        R sp = R(0.5) * ((F[k] + F[o]) - (feq[k] + feq[o]));
        R sm = R(0.5) * ((F[k] - F[o]) - (feq[k] - feq[o]));
        M[k] = F[k] - om * sp - omA * sm;
      }
    }
    flag_nonfinite(a, M[0]);
  }
}

// ------------------------------------------------------ boundary conditions

// F of a special node after streaming and the inlet / wall treatments of
// HandleBoundariesStep (serial/Iterate.c:495-523), plus its outlet treatment
// when OUTLET is set (serial/Iterate.c:525-546).  Any node class is accepted:
// solid returns 0 (UpdateF copied the never-written METAF), bulk returns the
// plain pull.  `acc` reads METAF of the current state.
//
// With an accessor in deviation form (ACC::dev) F is returned as deviations
// d_k = F_k - w_k rho0.  Every treatment keeps its form because it only
// copies or combines populations of equal weight with coefficients summing to
// one; the density sums gain rho0 (the weights in each sum add up to 1).
template <bool OUTLET, class R, class ACC>
__device__ void boundary_F(const StepArgs &a, const ACC &acc, long long node, R F[9]);

template <class R, class ACC>
__device__ __noinline__ void boundary_F_noout(const StepArgs &a, const ACC &acc, long long node,
                                              R F[9]) {
  boundary_F<false, R, ACC>(a, acc, node, F);
}

// The treatment of a special node whose boundary record is `r`.  Without
// EXTRAP the extrapolating outlet (outlet 2, which treats the two nodes
// upstream through an out-of-line call) is left out, so that `a` need not
// live in memory; the caller routes those nodes elsewhere.
template <bool OUTLET, class R, class ACC, bool EXTRAP = true, class REC = BRec>
__device__ __forceinline__ void boundary_F_rec(const StepArgs &a, const ACC &acc, long long node,
                                               const REC &r, R F[9]);

template <bool OUTLET, class R, class ACC>
__device__ void boundary_F(const StepArgs &a, const ACC &acc, long long node, R F[9]) {
  constexpr bool DEV = ACC::dev;
  const R rho0 = DEV ? (R)a.rho0 : R(0);
  const uint8_t c = a.cls[node];
  if (c == CLS_SOLID) {
#pragma unroll
    for (int k = 0; k < 9; k++) F[k] = DEV ? -wgt<R>(k) * rho0 : R(0);
    return;
  }
  if (c != CLS_SPECIAL) {
#pragma unroll
    for (int k = 0; k < 9; k++) F[k] = acc.meta(node - nb(k, a.pitch), k);
    return;
  }
  boundary_F_rec<OUTLET, R, ACC>(a, acc, node, a.rec[a.aux[node]], F);
}

// REC: BRec, or a record with the same members (flags, uo, q) in FP32.
template <bool OUTLET, class R, class ACC, bool EXTRAP, class REC>
__device__ __forceinline__ void boundary_F_rec(const StepArgs &a, const ACC &acc, long long node,
                                               const REC &r, R F[9]) {
  constexpr bool DEV = ACC::dev;
  const R rho0 = DEV ? (R)a.rho0 : R(0);
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
    if (DEV) rhoN = rho0 + rhoN;
    F[4] = F[2];
    F[8] = F[6] + rhoN * uo / R(6.0);
    F[7] = F[5] - rhoN * uo / R(6.0);
  }
  if (fl & FL_WEST) {
    R sW = F[0] + F[2] + F[4] + R(2.0) * (F[3] + F[6] + F[7]);
    if (DEV) sW = rho0 + sW;
    R rhoW = sW / (R(1.0) - uo);
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
      R sE = F[0] + F[2] + F[4] + R(2.0) * (F[1] + F[5] + F[8]);
      if (DEV) sE = rho0 + sE;
      R rhoE = sE / (R(1) - uo);
      F[3] = F[1] - R(2) * rhoE * uo / R(3.0);
      F[7] = F[5] - rhoE * uo / R(6.0);
      F[6] = F[8] - rhoE * uo / R(6.0);
    } else if (a.outlet == 2) {
      // 2nd-order extrapolation from the already treated i-1, i-2 cells,
      // serial/Iterate.c:535-541
      if constexpr (EXTRAP) {
        R A[9], B[9];
        boundary_F_noout<R, ACC>(a, acc, node - 1, A);
        boundary_F_noout<R, ACC>(a, acc, node - 2, B);
        F[1] = R(2) * (A[1]) - B[1];
        F[5] = R(2) * (A[5]) - B[5];
        F[8] = R(2) * (A[8]) - B[8];
      }
    } else if (a.outlet == 4) {
      // constant-pressure east outlet (Zou-He density condition; not in the reference)
      const R ro = (R)a.rho_out;
      R sP = F[0] + F[2] + F[4] + R(2.0) * (F[1] + F[5] + F[8]);
      if (DEV) sP = rho0 + sP;
      R ux = R(-1.0) + sP / ro;
      R ru = ro * ux;
      R d24 = R(0.5) * (F[2] - F[4]);
      F[3] = F[1] - (R(2.0) / R(3.0)) * ru;
      F[7] = F[5] + d24 - ru / R(6.0);
      F[6] = F[8] - d24 - ru / R(6.0);
    }
  }
}

// Full treatment of a special node as one out-of-line call (keeps the bulk
// path's register budget small).  Returns F (in the accessor's form) and the
// macroscopic fields (V = 0 on east-outlet cells,
// serial/CellFunctions.c:483-486).
template <class R, class ACC, bool EXTRAP = true, class REC = BRec>
__device__ __forceinline__ void special_node_rec(const StepArgs &a, const ACC &acc, long long node,
                                                 const REC &r, R F[9], R *mac) {
  boundary_F_rec<true, R, ACC, EXTRAP, REC>(a, acc, node, r, F);
  R rho, u, v;
  if constexpr (ACC::dev) {
    R rt = ((F[0] + F[1]) + (F[2] + F[3])) + ((F[4] + F[5]) + (F[6] + F[7])) + F[8];
    R jx = (F[1] - F[3]) + (F[5] - F[6]) + (F[8] - F[7]);
    R jy = (F[2] - F[4]) + (F[5] - F[7]) + (F[6] - F[8]);
    rho = (R)a.rho0 + rt;
    R inv = R(1) / rho;
    u = jx * inv;
    v = jy * inv;
  } else {
    moments<R>(F, rho, u, v);
  }
  if (r.flags & FL_EAST) v = R(0.0);
  mac[0] = rho;
  mac[1] = u;
  mac[2] = v;
}

template <class R, class ACC>
__device__ __noinline__ void special_node(const StepArgs &a, const ACC &acc, long long node,
                                          R F[9], R *mac) {
  special_node_rec<R, ACC>(a, acc, node, a.rec[a.aux[node]], F, mac);
}

// Collision of deviations d = F - w rho0 with given rho, u, v (the special
// nodes of the shifted storages, where v may be forced to 0).  Same operators
// as collide<>, written for d: f_eq - w rho0 = w ((rho - rho0) + rho (3 c.u +
// 4.5 (c.u)^2 - 1.5 u^2)); MRT rows 0..2 gain the rho0 M w terms.
template <int MODEL>
__device__ __forceinline__ void collide_dev(const float F[9], float rho, float u, float v,
                                            const StepArgs &a, float M[9]) {
  const float rho0 = (float)a.rho0, rt = rho - rho0;
  if (MODEL == 3) {
    const float om = (float)a.omega;
    float a13 = F[1] + F[3], a24 = F[2] + F[4];
    float a14 = a13 + a24;
    float p57 = F[5] + F[7], p68 = F[6] + F[8];
    float a58 = p57 + p68;
    float m0 = (F[0] + a14) + a58;
    float m1 = 2.f * a58 - a14 - 4.f * F[0];
    float m2 = (4.f * F[0] + a58) - 2.f * a14;
    float d13 = F[1] - F[3], d24 = F[2] - F[4];
    float e57 = F[5] - F[7], e86 = F[8] - F[6];
    float x58 = e57 + e86, y58 = e57 - e86;
    float m3 = d13 + x58, m5 = d24 + y58;
    float m4 = x58 - 2.f * d13, m6 = y58 - 2.f * d24;
    float m7 = a13 - a24, m8 = p57 - p68;
    const float ru = rho * u, rv = rho * v, rrq = rho * rho * (u * u + v * v);
    // m(F) - meq with m(F) = m(d) + rho0 (1, -2, 1, 0, ...)
    float d0 = m0 - rt;
    float d1 = 1.4f * (m1 + 2.f * rt - 3.f * rrq);
    float d2 = 1.4f * (m2 - rt + 3.f * rrq);
    float d3 = m3 - ru;
    float d4 = 1.2f * (m4 + ru);
    float d5 = m5 - rv;
    float d6 = 1.2f * (m6 + rv);
    float d7 = om * (m7 - rho * (u * u - v * v));
    float d8 = om * (m8 - ru * v);
    const float c = 1.f / 36.f;
    float ax = 4.f * d0 - d1 - 2.f * d2;
    float dg = 4.f * d0 + 2.f * d1 + d2;
    float X = 6.f * (d3 - d4), Y = 6.f * (d5 - d6), P = 9.f * d7;
    float Xd = 6.f * d3 + 3.f * d4, Yd = 6.f * d5 + 3.f * d6, Q = 9.f * d8;
    M[0] = F[0] - c * (4.f * ((d0 - d1) + d2));
    M[1] = F[1] - c * (ax + X + P);
    M[2] = F[2] - c * (ax + Y - P);
    M[3] = F[3] - c * (ax - X + P);
    M[4] = F[4] - c * (ax - Y - P);
    M[5] = F[5] - c * (dg + Xd + Yd + Q);
    M[6] = F[6] - c * (dg - Xd + Yd - Q);
    M[7] = F[7] - c * (dg - Xd - Yd + Q);
    M[8] = F[8] - c * (dg + Xd - Yd - Q);
  } else {
    const float T1 = u * u + v * v;
    float feq[9];
#pragma unroll
    for (int k = 0; k < 9; k++) {
      const float T2 = u * CX[k] + v * CY[k];
      feq[k] = wgt<float>(k) * (rt + rho * (3.f * T2 + 4.5f * T2 * T2 - 1.5f * T1));
    }
    const float om = (float)a.omega, omA = (float)a.omegaA;
#pragma unroll
    for (int k = 0; k < 9; k++) {
      if (MODEL == 1) {
        M[k] = fmaf(om, feq[k] - F[k], F[k]);
      } else {
        const int o = OPP[k];
        float sp = 0.5f * ((F[k] + F[o]) - (feq[k] + feq[o]));
        float sm = 0.5f * ((F[k] - F[o]) - (feq[k] - feq[o]));
        M[k] = F[k] - om * sp - omA * sm;
      }
    }
  }
  flag_nonfinite(a, M[0]);
}

// ------------------------------------------------------------------- kernels

__device__ __forceinline__ bool node_xy(const StepArgs &a, int &x, int &y) {
  x = blockIdx.x * blockDim.x + threadIdx.x;
  y = blockIdx.y;
  return x < a.n;
}

// Store of one fluid node's post-collision populations in the output layout
// (plus its side-buffer copy in the AA pattern when it is recorded).
template <class ST, int PH>
__device__ __forceinline__ void store_node(const StepArgs &a, long long node, uint8_t c,
                                           const typename ST::R M[9]) {
  using T = typename ST::T;
  T *d = (T *)a.dst;
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

// Collision and store of one fluid node whose F and moments are known.
template <class ST, int MODEL, int PH>
__device__ __forceinline__ void collide_store(const StepArgs &a, long long node, uint8_t c,
                                              const typename ST::R F[9], typename ST::R rho,
                                              typename ST::R u, typename ST::R v) {
  using R = typename ST::R;
  R M[9];
  collide<MODEL, R>(F, rho, u, v, a, M);
  store_node<ST, PH>(a, node, c, M);
}

// Store of a bulk node's post-collision populations given in the storage's
// bulk form (deviations for shifted storage); the AA side buffer keeps
// absolute values.
template <class ST, int PH>
__device__ __forceinline__ void store_node_dev(const StepArgs &a, long long node, uint8_t c,
                                               const typename ST::R M[9]) {
  using T = typename ST::T;
  T *d = (T *)a.dst;
#pragma unroll
  for (int k = 0; k < 9; k++) {
    long long i;
    if (PH == PH_AB) i = (long long)k * a.plane + node;
    else if (PH == PH_AA_A) i = (long long)k * a.plane + node + nb(k, a.pitch);
    else i = (long long)OPP[k] * a.plane + node;
    st_dev<ST>(d + i, k, M[k], a);
  }
  if (PH != PH_AB && c != CLS_BULK) {
    uint32_t sbi = a.aux[node];
    if (c == CLS_SPECIAL) sbi = a.rec[sbi].sb;
#pragma unroll
    for (int k = 0; k < 9; k++)
      a.sb_dst[(size_t)sbi * 9 + k] = (double)M[k] + (ST::SHIFT ? wgt<double>(k) * a.rho0 : 0.0);
  }
}

// Collision and store of a node without boundary work (F in bulk form).
template <class ST, int MODEL, int PH>
__device__ __forceinline__ void bulk_store(const StepArgs &a, long long node, uint8_t c,
                                           const typename ST::R F[9]) {
  using R = typename ST::R;
  R M[9];
  collide_bulk_dev<MODEL, ST>(F, a, M);
  store_node_dev<ST, PH>(a, node, c, M);
}

// Index of the pulled F[k](node) in the state of layout PH.
template <int PH>
__device__ __forceinline__ long long pull_index(int k, long long node, const StepArgs &a) {
  if (PH == PH_AB) return (long long)k * a.plane + node - nb(k, a.pitch);
  if (PH == PH_AA_A) return (long long)OPP[k] * a.plane + node - nb(k, a.pitch);
  return (long long)k * a.plane + node;
}

// The whole fused update of one node of any class.
template <class ST, int MODEL, int PH>
__device__ __forceinline__ void step_one(const StepArgs &a, long long node, uint8_t c) {
  using R = typename ST::R;
  using T = typename ST::T;
  if (c == CLS_SOLID) return;
  const T *s = (const T *)a.src;
  R F[9], rho, u, v;
  if (c != CLS_SPECIAL) {
#pragma unroll
    for (int k = 0; k < 9; k++) F[k] = ld_dev<ST>(s + pull_index<PH>(k, node, a), k, a);
    bulk_store<ST, MODEL, PH>(a, node, c, F);
    return;
  } else {
    constexpr bool SH = ST::SHIFT;
    R mac[3];
    if constexpr (PH == PH_AB) special_node<R>(a, AccMain<ST, PH_AB, SH>(a, a.src), node, F, mac);
    else special_node<R>(a, AccSide<ST, SH>(a, nullptr), node, F, mac);
    rho = mac[0];
    u = mac[1];
    v = mac[2];
    if constexpr (SH) {
      R M[9];
      collide_dev<MODEL>(F, rho, u, v, a, M);
      store_node_dev<ST, PH>(a, node, c, M);
      return;
    }
  }
  collide_store<ST, MODEL, PH>(a, node, c, F, rho, u, v);
}

// The per-node path as a called function, for the paired kernels whose warps
// take it only where a boundary runs through them: keeping it out of line
// keeps its registers out of the bulk path's allocation.
template <class ST, int MODEL, int PH>
__device__ __noinline__ void step_one_cold(const StepArgs &a, long long node, uint8_t c) {
  step_one<ST, MODEL, PH>(a, node, c);
}

// Fused step: METAF_t (layout PH) -> METAF_{t+1}.  A block is BX threads
// along x; each thread updates NPT consecutive rows of its column.  When all
// NPT nodes are free of boundary work their 9*NPT loads are issued before any
// arithmetic (more bytes in flight per thread).
// One column of NPT nodes.  With SKIP_SPECIAL the nodes with boundary work
// are left out (another pass updates them from a compact list), so that a
// warp never waits on one lane's boundary treatment.
template <class ST, int MODEL, int PH, int NPT, bool SKIP_SPECIAL = false>
__device__ __forceinline__ void step_column(const StepArgs &a, int x, int y0) {
  using R = typename ST::R;
  using T = typename ST::T;
  if (x >= a.n) return;
  uint8_t c[NPT];
  bool bulk = true;
#pragma unroll
  for (int j = 0; j < NPT; j++) {
    const int y = y0 + j;
    c[j] = (y < a.m) ? a.cls[(long long)y * a.pitch + x] : (uint8_t)CLS_SOLID;
    if (SKIP_SPECIAL && c[j] == CLS_SPECIAL) c[j] = CLS_SOLID;
    bulk = bulk && c[j] != CLS_SPECIAL;
  }
  if (NPT == 1 || !bulk) {
#pragma unroll
    for (int j = 0; j < NPT; j++)
      step_one<ST, MODEL, PH>(a, (long long)(y0 + j) * a.pitch + x, c[j]);
    return;
  }
  const T *s = (const T *)a.src;
  R F[NPT][9];
#pragma unroll
  for (int j = 0; j < NPT; j++) {
    const long long node = (long long)(y0 + j) * a.pitch + x;
#pragma unroll
    for (int k = 0; k < 9; k++)
      F[j][k] = (c[j] != CLS_SOLID) ? ld_dev<ST>(s + pull_index<PH>(k, node, a), k, a) : R(0);
  }
#pragma unroll
  for (int j = 0; j < NPT; j++) {
    if (c[j] == CLS_SOLID) continue;
    bulk_store<ST, MODEL, PH>(a, (long long)(y0 + j) * a.pitch + x, c[j], F[j]);
  }
}

template <class ST, int MODEL, int PH, int BX, int NPT>
__global__ void __launch_bounds__(BX) k_step(const __grid_constant__ StepArgs a) {
  step_column<ST, MODEL, PH, NPT>(a, blockIdx.x * BX + threadIdx.x, blockIdx.y * NPT);
}

// Fused step over x-chunks: each thread owns V consecutive nodes of NPT rows
// and moves every population plane with one aligned 4..16-byte word per
// chunk.  The +-1 x-shift of the pull is served by a warp shuffle from the
// neighbouring lane (lanes 0 and 31 read the chunk edge themselves).  Warps
// that touch any node with boundary work fall back to the per-node path, so
// the shuffles always run with the whole warp.
template <class ST, int MODEL, int PH, int BX, int V, int NPT>
__global__ void __launch_bounds__(BX) k_step_vec(const __grid_constant__ StepArgs a) {
  using R = typename ST::R;
  using T = typename ST::T;
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int x0 = (blockIdx.x * BX + threadIdx.x) * V;
  const int y0 = blockIdx.y * NPT;
  if (x0 - lane * V >= a.pitch) return;  // the whole warp lies past the row
  uint8_t cl[NPT][V];
  bool special = false, fluid = false;
#pragma unroll
  for (int j = 0; j < NPT; j++)
#pragma unroll
    for (int i = 0; i < V; i++) {
      const int y = y0 + j, x = x0 + i;
      cl[j][i] = (y < a.m && x < a.n) ? a.cls[(long long)y * a.pitch + x] : (uint8_t)CLS_SOLID;
      special = special || cl[j][i] == CLS_SPECIAL;
      fluid = fluid || cl[j][i] != CLS_SOLID;
    }
  if (__any_sync(FULL, special)) {
#pragma unroll
    for (int j = 0; j < NPT; j++)
#pragma unroll
      for (int i = 0; i < V; i++)
        if (x0 + i < a.n && y0 + j < a.m)
          step_one<ST, MODEL, PH>(a, (long long)(y0 + j) * a.pitch + x0 + i, cl[j][i]);
    return;
  }
  if (!__any_sync(FULL, fluid)) return;
  const T *s = (const T *)a.src;
  T *d = (T *)a.dst;
  R F[NPT][V][9];
#pragma unroll
  for (int j = 0; j < NPT; j++) {
    const int y = y0 + j;
    const bool inner = y >= 1 && y < a.m - 1;  // warp-uniform: border rows are solid
#pragma unroll
    for (int k = 0; k < 9; k++) {
      if (!inner) {
#pragma unroll
        for (int i = 0; i < V; i++) F[j][i][k] = R(0);
        continue;
      }
      const int plane = (PH == PH_AA_A) ? OPP[k] : k;
      const int sx = (PH == PH_AA_B) ? 0 : CX[k];
      const int row = (PH == PH_AA_B) ? y : y - CY[k];
      const long long base = (long long)plane * a.plane + (long long)row * a.pitch + x0;
      T raw[V];
      VecIO<T, V>::load(s + base, raw);
      R val[V];
#pragma unroll
      for (int i = 0; i < V; i++) val[i] = ST::cvt_dev(raw[i], k, a);
      if (sx == 0) {
#pragma unroll
        for (int i = 0; i < V; i++) F[j][i][k] = val[i];
      } else if (sx == 1) {
        R edge = __shfl_up_sync(FULL, val[V - 1], 1);
        if (lane == 0) edge = x0 > 0 ? ld_dev<ST>(s + base - 1, k, a) : R(0);
        F[j][0][k] = edge;
#pragma unroll
        for (int i = 1; i < V; i++) F[j][i][k] = val[i - 1];
      } else {
        R edge = __shfl_down_sync(FULL, val[0], 1);
        if (lane == 31) edge = ld_dev<ST>(s + base + V, k, a);
        F[j][V - 1][k] = edge;
#pragma unroll
        for (int i = 0; i < V - 1; i++) F[j][i][k] = val[i + 1];
      }
    }
  }
#pragma unroll
  for (int j = 0; j < NPT; j++) {
    const int y = y0 + j;
    if (!(y >= 1 && y < a.m - 1)) continue;
    bool rowfluid = false;
#pragma unroll
    for (int i = 0; i < V; i++) {
      rowfluid = rowfluid || cl[j][i] != CLS_SOLID;
      R M[9];
      if (cl[j][i] != CLS_SOLID) {
        collide_bulk_dev<MODEL, ST>(F[j][i], a, M);
      } else {
#pragma unroll
        for (int k = 0; k < 9; k++) M[k] = R(0);
      }
#pragma unroll
      for (int k = 0; k < 9; k++) F[j][i][k] = M[k];
      if (PH != PH_AB && cl[j][i] == CLS_BULK_REC) {
        const uint32_t sbi = a.aux[(long long)y * a.pitch + x0 + i];
#pragma unroll
        for (int k = 0; k < 9; k++)
          a.sb_dst[(size_t)sbi * 9 + k] = (double)M[k] + (ST::SHIFT ? wgt<double>(k) * a.rho0 : 0.0);
      }
    }
    if (!rowfluid) continue;
    const long long node0 = (long long)y * a.pitch + x0;
#pragma unroll
    for (int k = 0; k < 9; k++) {
      if (PH == PH_AA_A) {
        // neighbour write x + e_k: element-wise (only fluid nodes own a slot there)
#pragma unroll
        for (int i = 0; i < V; i++)
          if (cl[j][i] != CLS_SOLID)
            st_dev<ST>(d + (long long)k * a.plane + node0 + i + nb(k, a.pitch), k, F[j][i][k], a);
      } else {
        T raw[V];
#pragma unroll
        for (int i = 0; i < V; i++) raw[i] = ST::pack_dev(F[j][i][k], k, a);
        const int plane = (PH == PH_AB) ? k : OPP[k];
        VecIO<T, V>::store(d + (long long)plane * a.plane + node0, raw);
      }
    }
  }
}

// ------------------------------------------------ 16-bit storage, paired nodes

// Two adjacent nodes per thread, moved as one 32-bit word (two 16-bit
// values) per population plane.  All 9 x NPT words of a thread are loaded
// before any arithmetic; the +-1 x-shift of the pull is a warp shuffle of the
// neighbouring lane's word and a byte permute (lanes 0 and 31 load the
// half-word beyond the warp themselves, also up front).  Warps that touch a
// node with boundary work run the per-node path instead, so the shuffles
// always involve the whole warp.  Only for 2-byte storage.
// Packed FP32 pairs: the two nodes of a 32-bit word go through the bulk
// collision together with the paired FP32 instructions of sm_100-class GPUs
// (one FFMA2/FADD2/FMUL2 does the work of two scalar ones).
__device__ __forceinline__ float2 bc2(float s) { return make_float2(s, s); }
__device__ __forceinline__ float2 add2(float2 x, float2 y) { return __fadd2_rn(x, y); }
__device__ __forceinline__ float2 sub2(float2 x, float2 y) { return __ffma2_rn(y, bc2(-1.f), x); }
__device__ __forceinline__ float2 mul2(float2 x, float2 y) { return __fmul2_rn(x, y); }
__device__ __forceinline__ float2 fma2(float2 x, float2 y, float2 z) { return __ffma2_rn(x, y, z); }

// Deviations of a word's two nodes (bulk form of a shifted 16-bit storage).
template <class ST>
__device__ __forceinline__ float2 unpack2v(uint32_t w, int k, const StepArgs &a) {
  float2 f;
  if constexpr (std::is_same<typename ST::T, __half>::value) {
    __half2 h;
    memcpy(&h, &w, 4);
    f = __half22float2(h);
  } else {
    __nv_bfloat162 h;
    memcpy(&h, &w, 4);
    f = __bfloat1622float2(h);
  }
  return mul2(f, bc2(a.inv_scale[k]));
}
template <class ST>
__device__ __forceinline__ uint32_t pack2v(float2 d, int k, const StepArgs &a) {
  const float2 sc = mul2(d, bc2(a.scale[k]));
  uint32_t w;
  if constexpr (std::is_same<typename ST::T, __half>::value) {
    const __half2 h = __float22half2_rn(sc);
    memcpy(&w, &h, 4);
  } else {
    const __nv_bfloat162 h = __float22bfloat162_rn(sc);
    memcpy(&w, &h, 4);
  }
  return w;
}

// The two stored 16-bit values of a word as floats, without the deviation
// scale (raw storage units), and back.
template <class ST>
__device__ __forceinline__ float2 raw2(uint32_t w) {
  if constexpr (std::is_same<typename ST::T, __half>::value) {
    __half2 h;
    memcpy(&h, &w, 4);
    return __half22float2(h);
  } else {
    __nv_bfloat162 h;
    memcpy(&h, &w, 4);
    return __bfloat1622float2(h);
  }
}
template <class ST>
__device__ __forceinline__ uint32_t pack_raw2(float2 v) {
  uint32_t w;
  if constexpr (std::is_same<typename ST::T, __half>::value) {
    const __half2 h = __float22half2_rn(v);
    memcpy(&w, &h, 4);
  } else {
    const __nv_bfloat162 h = __float22bfloat162_rn(v);
    memcpy(&w, &h, 4);
  }
  return w;
}
template <class ST>
__device__ __forceinline__ typename ST::T to_raw(float v) {
  if constexpr (std::is_same<typename ST::T, __half>::value) return __float2half_rn(v);
  else return __float2bfloat16_rn(v);
}

// MRT bulk collision of two nodes (the operator of collide_bulk_dev, model 3,
// constants folded) on packed FP32 pairs and raw storage values.  16-bit storage keeps
// s_k = d_k * scale_k with scale_k = S / (w_k rho0), so in the unit
// u0 = rho0 / (36 S) (= inv_scale[8]) the deviation is d_k / u0 = c_k s_k with
// c_k = 36 w_k = 16, 4, 1: exact powers of two.  The operator is written in
// that unit (its quadratic terms gain a factor u0, rho = rho0 + u0 * sum) and
// the input factors c_k and output factors 1 / c_k are folded into its
// constants, so neither the load nor the store scales anything:
//   g1 = 4 (a58 + t14) - 32 s0 - 3 u0 jj,  g2 = 48 s0 - 12 t14 + 3 u0 jj,
//   E4 = (m4 + jx) / 2,  E6 = (m6 + jy) / 2.
__device__ __forceinline__ void collide_mrt_pair_raw(const float2 S[9], const StepArgs &a, float2 O[9]) {
  const float u0 = a.inv_scale[8];
  const float2 t13 = add2(S[1], S[3]), t24 = add2(S[2], S[4]);
  const float2 t14 = add2(t13, t24);
  const float2 p57 = add2(S[5], S[7]), p68 = add2(S[6], S[8]);
  const float2 a58 = add2(p57, p68);
  const float2 rt = fma2(bc2(16.f), S[0], fma2(bc2(4.f), t14, a58));
  const float2 rho = fma2(bc2(u0), rt, bc2((float)a.rho0));
  const float2 u13 = sub2(S[1], S[3]), u24 = sub2(S[2], S[4]);
  const float2 e57 = sub2(S[5], S[7]), e86 = sub2(S[8], S[6]);
  const float2 x58 = add2(e57, e86), y58 = sub2(e57, e86);
  const float2 jx = fma2(bc2(4.f), u13, x58), jy = fma2(bc2(4.f), u24, y58);
  const float2 E4 = fma2(bc2(-2.f), u13, x58), E6 = fma2(bc2(-2.f), u24, y58);
  const float2 w7 = sub2(t13, t24), m8 = sub2(p57, p68);
  const float2 jj = fma2(jx, jx, mul2(jy, jy));
  const float2 ninv = make_float2(__fdividef(-u0, rho.x), __fdividef(-u0, rho.y));
  const float2 g1 = fma2(bc2(-3.f * u0), jj, fma2(bc2(-32.f), S[0], mul2(bc2(4.f), add2(a58, t14))));
  const float2 g2 = fma2(bc2(3.f * u0), jj, fma2(bc2(48.f), S[0], mul2(bc2(-12.f), t14)));
  const float2 h7 = fma2(mul2(sub2(jx, jy), add2(jx, jy)), ninv, mul2(bc2(4.f), w7));
  const float2 h8 = fma2(mul2(jx, jy), ninv, m8);
  const float om = (float)a.omega;
  const float2 P4 = mul2(bc2(om * (1.f / 16.f)), h7), Q = mul2(bc2(0.25f * om), h8);
  const float2 A4 = mul2(bc2(-1.4f / 144.f), fma2(bc2(2.f), g2, g1));
  const float2 D = mul2(bc2(1.4f / 36.f), fma2(bc2(2.f), g1, g2));
  const float2 ApP = add2(A4, P4), AmP = sub2(A4, P4), DpQ = add2(D, Q), DmQ = sub2(D, Q);
  const float2 S46 = add2(E4, E6), T46 = sub2(E4, E6);
  O[0] = fma2(bc2(-5.6f / 576.f), sub2(g2, g1), S[0]);
  O[1] = fma2(bc2(0.1f), E4, sub2(S[1], ApP));
  O[3] = fma2(bc2(-0.1f), E4, sub2(S[3], ApP));
  O[2] = fma2(bc2(0.1f), E6, sub2(S[2], AmP));
  O[4] = fma2(bc2(-0.1f), E6, sub2(S[4], AmP));
  O[5] = fma2(bc2(-0.2f), S46, sub2(S[5], DpQ));
  O[7] = fma2(bc2(0.2f), S46, sub2(S[7], DpQ));
  O[6] = fma2(bc2(0.2f), T46, sub2(S[6], DmQ));
  O[8] = fma2(bc2(-0.2f), T46, sub2(S[8], DmQ));
}

// Edge half-word slot of a shifted plane: cx = +1 planes 1, 5, 8 (lane 0) and
// cx = -1 planes 3, 6, 7 (lane 31) each use slots 0..2.
__device__ __forceinline__ constexpr int edge_slot(int k) {
  return (k == 1 || k == 3) ? 0 : ((k == 5 || k == 6) ? 1 : 2);
}

template <class ST, int MODEL, int PH, int NPT>
__global__ void __launch_bounds__(128, NPT == 2 ? 8 : 1) k_step_h2(const __grid_constant__ StepArgs a) {
  using T = typename ST::T;
  static_assert(sizeof(T) == 2, "paired-node kernel is for 16-bit storage");
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int x0 = (blockIdx.x * 128 + threadIdx.x) * 2;
  const int y0 = blockIdx.y * NPT;
  // L2 prefetch for the block a.pf_blocks launch positions ahead (a fraction
  // of a wave later): 9 planes x NPT rows of its 256-node tile, one 512-byte bulk
  // prefetch each, and its NPT rows of class bytes (256 bytes each: the
  // first loads of a block, on which all others wait), so that its loads find
  // their sectors in L2.  A hint only: no completion to wait for; every
  // address lies inside the state or the class array (16-byte aligned: the
  // pitch is a multiple of 256).
  if (a.pf_blocks > 0 && threadIdx.x < 10 * NPT) {
    const long long L = (long long)blockIdx.y * gridDim.x + blockIdx.x + a.pf_blocks;
    if (L < (long long)gridDim.x * gridDim.y) {
      const int px = (int)(L % gridDim.x), py = (int)(L / gridDim.x);
      const int k = threadIdx.x / NPT, y = py * NPT + threadIdx.x % NPT;
      if (y < a.m && px * 256 + 256 <= a.pitch) {
        if (k < 9) {
          const int plane = (PH == PH_AA_A) ? OPP[k] : k;
          const T *p = (const T *)a.src + (long long)plane * a.plane + (long long)y * a.pitch + px * 256;
          asm volatile("cp.async.bulk.prefetch.L2.global [%0], 512;" ::"l"(p) : "memory");
        } else {
          const uint8_t *p = a.cls + (long long)y * a.pitch + px * 256;
          asm volatile("cp.async.bulk.prefetch.L2.global [%0], 256;" ::"l"(p) : "memory");
        }
      }
    }
  }
  if (x0 - lane * 2 >= a.pitch) return;  // the whole warp lies past the row
  uint8_t cl[NPT][2];
  bool special = false, fluid = false;
#pragma unroll
  for (int j = 0; j < NPT; j++)
#pragma unroll
    for (int i = 0; i < 2; i++) {
      const int y = y0 + j, x = x0 + i;
      cl[j][i] = (y < a.m && x < a.n) ? a.cls[(long long)y * a.pitch + x] : (uint8_t)CLS_SOLID;
      special = special || cl[j][i] == CLS_SPECIAL;
      fluid = fluid || cl[j][i] != CLS_SOLID;
    }
  if (__any_sync(FULL, special)) {
#pragma unroll
    for (int j = 0; j < NPT; j++)
#pragma unroll
      for (int i = 0; i < 2; i++)
        if (x0 + i < a.n && y0 + j < a.m)
          step_one_cold<ST, MODEL, PH>(a, (long long)(y0 + j) * a.pitch + x0 + i, cl[j][i]);
    return;
  }
  if (!__any_sync(FULL, fluid)) return;
  const T *s = (const T *)a.src;
  T *d = (T *)a.dst;
  constexpr bool SHIFT = PH != PH_AA_B;
  // ---- loads: every word first, the two warp-edge half-words alongside
  uint32_t w[NPT][9];
  T edge[NPT][3];  // lane 0: x0-1 for the cx=+1 planes; lane 31: x0+2 for cx=-1
#pragma unroll
  for (int j = 0; j < NPT; j++) {
    const int y = y0 + j;
    const bool inner = y >= 1 && y < a.m - 1;  // warp-uniform: border rows are solid
#pragma unroll
    for (int k = 0; k < 9; k++) {
      const int plane = (PH == PH_AA_A) ? OPP[k] : k;
      const int row = SHIFT ? y - CY[k] : y;
      const long long base = (long long)plane * a.plane + (long long)row * a.pitch + x0;
      w[j][k] = inner ? __ldg((const unsigned *)(s + base)) : 0u;
      if (SHIFT && CX[k] == 1 && lane == 0 && inner) edge[j][edge_slot(k)] = __ldg(s + base - 1);
      if (SHIFT && CX[k] == -1 && lane == 31 && inner) edge[j][edge_slot(k)] = __ldg(s + base + 2);
    }
  }
  // ---- per row: assemble the pulled pairs, collide, store
#pragma unroll
  for (int j = 0; j < NPT; j++) {
    const int y = y0 + j;
    if (!(y >= 1 && y < a.m - 1)) continue;
    float2 F[9];
#pragma unroll
    for (int k = 0; k < 9; k++) {
      uint32_t word = w[j][k];
      if (SHIFT && CX[k] == 1) {
        uint32_t prev = __shfl_up_sync(FULL, word, 1);
        if (lane == 0) {
          uint16_t h;
          memcpy(&h, &edge[j][edge_slot(k)], 2);
          prev = (uint32_t)h << 16;
        }
        word = __byte_perm(prev, word, 0x5432);  // (x0-1, x0)
      } else if (SHIFT && CX[k] == -1) {
        uint32_t next = __shfl_down_sync(FULL, word, 1);
        if (lane == 31) {
          uint16_t h;
          memcpy(&h, &edge[j][edge_slot(k)], 2);
          next = (uint32_t)h;
        }
        word = __byte_perm(word, next, 0x5432);  // (x0+1, x0+2)
      }
      // MRT works on raw storage values (no scaling), other models on deviations
      F[k] = MODEL == 3 ? raw2<ST>(word) : unpack2v<ST>(word, k, a);
    }
    float2 M[9];
    if constexpr (MODEL == 3) {
      collide_mrt_pair_raw(F, a, M);
    } else {
      float F0[9], F1[9], M0[9], M1[9];
#pragma unroll
      for (int k = 0; k < 9; k++) {
        F0[k] = F[k].x;
        F1[k] = F[k].y;
      }
      collide_bulk_dev<MODEL, ST>(F0, a, M0);
      collide_bulk_dev<MODEL, ST>(F1, a, M1);
#pragma unroll
      for (int k = 0; k < 9; k++) M[k] = make_float2(M0[k], M1[k]);
    }
    // a solid node of the pair keeps zero deviations
    if (cl[j][0] == CLS_SOLID)
#pragma unroll
      for (int k = 0; k < 9; k++) M[k].x = 0.f;
    if (cl[j][1] == CLS_SOLID)
#pragma unroll
      for (int k = 0; k < 9; k++) M[k].y = 0.f;
    if constexpr (MODEL == 3) flag_nonfinite(a, M[0].x + M[0].y);
    const long long node0 = (long long)y * a.pitch + x0;
#pragma unroll
    for (int i = 0; i < 2; i++)
      if (PH != PH_AB && cl[j][i] == CLS_BULK_REC) {
        const uint32_t sbi = a.aux[node0 + i];
#pragma unroll
        for (int k = 0; k < 9; k++) {
          const float dv = (i ? M[k].y : M[k].x) * (MODEL == 3 ? a.inv_scale[k] : 1.f);
          a.sb_dst[(size_t)sbi * 9 + k] = (double)dv + wgt<double>(k) * a.rho0;
        }
      }
#pragma unroll
    for (int k = 0; k < 9; k++) {
      if (PH == PH_AA_A) {
        // neighbour write x + e_k, element-wise for fluid nodes
        T *q = d + (long long)k * a.plane + node0 + nb(k, a.pitch);
        if constexpr (MODEL == 3) {
          if (cl[j][0] != CLS_SOLID) q[0] = to_raw<ST>(M[k].x);
          if (cl[j][1] != CLS_SOLID) q[1] = to_raw<ST>(M[k].y);
        } else {
          if (cl[j][0] != CLS_SOLID) st_dev<ST>(q, k, M[k].x, a);
          if (cl[j][1] != CLS_SOLID) st_dev<ST>(q + 1, k, M[k].y, a);
        }
      } else {
        const int plane = (PH == PH_AB) ? k : OPP[k];
        const uint32_t wd = MODEL == 3 ? pack_raw2<ST>(M[k]) : pack2v<ST>(M[k], k, a);
        __stcs((unsigned *)(d + (long long)plane * a.plane + node0), wd);
      }
    }
  }
}

// ------------------------------------------------------------- TMA pipeline

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  uint64_t state;
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;"
               : "=l"(state)
               : "r"(smem_addr(bar)), "r"(bytes)
               : "memory");
  asm volatile("" ::"l"(state));
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: gives up after `polls` polls (each poll may suspend briefly).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, int polls) {
  for (int i = 0; i < polls; i++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
// One contiguous global -> shared copy by the bulk-copy (TMA) engine; both
// addresses 16-byte aligned, size a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// Fused step with TMA-staged sources.  The grid is persistent; a block walks
// tiles of TX x TY nodes (rows 1..m-2, which hold every fluid node).  For each
// tile warp 0 issues 10*TY bulk copies -- for every population plane the TY
// source rows, TX + 2H elements wide (H = one 16-byte granule of halo on each
// side, so every copy starts and ends on a 16-byte boundary), and the TY rows
// of class bytes -- into one stage of a ring of shared-memory stages;
// completion arrives on the stage's mbarrier.  Copies run a.tma_stages - 1
// tiles ahead of the computation, so the bytes in flight are bounded by
// shared memory, not registers, and the node loop reads its 9 inputs from
// shared memory at fixed offsets.  Nodes with boundary work take the per-node
// path with global loads (in the AA pattern their inputs live in the side
// buffer anyway).  Shared-memory stage layout: populations [k][j][W], then
// class bytes [j][TX].
template <class T, int TX, int TY>
struct TmaStage {
  static constexpr int H = 16 / (int)sizeof(T);
  static constexpr int W = TX + 2 * H;
  static constexpr int POP_BYTES = 9 * TY * W * (int)sizeof(T);
  static constexpr int BYTES = (POP_BYTES + TY * TX + 127) / 128 * 128;
};

template <class ST, int MODEL, int PH, int TX, int TY, int RPT>
__global__ void __launch_bounds__(TX * TY / RPT, 3) k_step_tma(const __grid_constant__ StepArgs a) {
  using R = typename ST::R;
  using T = typename ST::T;
  using G = TmaStage<T, TX, TY>;
  constexpr int H = G::H, W = G::W;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  uint64_t *bars = (uint64_t *)smem_raw;
  unsigned char *stages = smem_raw + 128;
  const int S = a.tma_stages;
  const int ntx = a.tma_tiles_x;
  const int ntiles = ntx * a.tma_tiles_y;
  const int tid = threadIdx.x, lane = tid & 31;
  const bool producer = tid < 32;
  const T *src = (const T *)a.src;
  if (tid == 0) {
    for (int st = 0; st < S; st++) mbar_init(&bars[st], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  // executed by the 32 lanes of warp 0
  auto issue = [&](int tile, int st) {
    const int tx0 = (tile % ntx) * TX;
    const int ty0 = 1 + (tile / ntx) * TY;
    const int rows = min(TY, (a.m - 1) - ty0);
    if (lane == 0) mbar_arrive_expect_tx(&bars[st], (uint32_t)(rows * (9 * W * sizeof(T) + TX)));
    __syncwarp();
    unsigned char *base = stages + (size_t)st * G::BYTES;
    for (int q = lane; q < 10 * rows; q += 32) {
      if (q < 9 * rows) {
        const int k = q / rows, j = q - k * rows;
        const int plane = (PH == PH_AA_A) ? OPP[k] : k;
        const int dy = (PH == PH_AA_B) ? 0 : -CY[k];
        const T *g = src + (long long)plane * a.plane + (long long)(ty0 + j + dy) * a.pitch + tx0 - H;
        bulk_g2s(base + (size_t)(k * TY + j) * W * sizeof(T), g, (uint32_t)(W * sizeof(T)), &bars[st]);
      } else {
        const int j = q - 9 * rows;
        bulk_g2s(base + G::POP_BYTES + j * TX, a.cls + (long long)(ty0 + j) * a.pitch + tx0,
                 (uint32_t)TX, &bars[st]);
      }
    }
  };

  int issued = 0, consumed = 0;
  if (producer)
    for (int q = 0; q < S - 1; q++) {
      const int t = blockIdx.x + q * gridDim.x;
      if (t < ntiles) issue(t, q), issued++;
    }
  const int col = tid % TX, rgrp = tid / TX;
  for (int tile = blockIdx.x, it = 0; tile < ntiles; tile += gridDim.x, it++) {
    const int st = it % S;
    if (producer) {
      const int ahead = tile + (S - 1) * gridDim.x;
      if (ahead < ntiles) {
        // the stage being refilled was read through the generic proxy in the
        // previous iteration (ordered by its trailing __syncthreads)
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        issue(ahead, (it + S - 1) % S);
        issued++;
      }
    }
    const bool ok = mbar_wait_bounded(&bars[st], (uint32_t)((it / S) & 1), 1 << 18);
    if (__syncthreads_or(!ok)) {
      if (tid == 0) {
        atomicExch(a.err, 1);
        // let the copies still in flight land before the block's shared memory goes away
        for (int q = consumed; q < issued; q++)
          mbar_wait_bounded(&bars[q % S], (uint32_t)((q / S) & 1), 1 << 16);
      }
      return;
    }
    consumed++;
    const int tx0 = (tile % ntx) * TX;
    const int ty0 = 1 + (tile / ntx) * TY;
    const unsigned char *base = stages + (size_t)st * G::BYTES;
    const T *sb = (const T *)base;
    const uint8_t *scls = base + G::POP_BYTES;
    const int x = tx0 + col;
#pragma unroll
    for (int r = 0; r < RPT; r++) {
      const int j = rgrp * RPT + r;
      const int y = ty0 + j;
      if (x >= a.n || y > a.m - 2) continue;
      const uint8_t c = scls[j * TX + col];
      if (c == CLS_SOLID) continue;
      const long long node = (long long)y * a.pitch + x;
      if (c == CLS_SPECIAL) {
        step_one<ST, MODEL, PH>(a, node, c);
        continue;
      }
      R F[9];
#pragma unroll
      for (int k = 0; k < 9; k++) {
        const int dx = (PH == PH_AA_B) ? 0 : -CX[k];
        F[k] = ST::cvt_dev(sb[(k * TY + j) * W + H + col + dx], k, a);
      }
      bulk_store<ST, MODEL, PH>(a, node, c, F);
    }
    __syncthreads();
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
// Blocks stride over rows (grid.y may be smaller than m).  Per-cell terms are
// formed in the storage's arithmetic type; with FP32/16-bit storage they are
// summed in FP32 over at most 8 rows per thread and then in FP64, so that the
// reductions are FP64 without an FP64 operation per term (GB300's FP64 rate
// is a small fraction of its FP32 rate).
template <class ST, int L>
__global__ void __launch_bounds__(128) k_finish(const __grid_constant__ StepArgs a, const FinishOut o) {
  using R = typename ST::R;
  using T = typename ST::T;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[NSUM];
  R part[NSUM];
#pragma unroll
  for (int i = 0; i < NSUM; i++) acc[i] = 0.0, part[i] = R(0);
  const T *src = (const T *)a.src;
  constexpr bool SH = ST::SHIFT;  // populations handled as deviations, see moments_form
  AccMain<ST, L, SH> acc_m(a, a.src);
  int chunk = 0;
  for (int y = blockIdx.y; y < a.m && x < a.n; y += gridDim.y) {
    const long long node = (long long)y * a.pitch + x;
    const long long cell = (long long)y * a.n + x;
    const uint8_t c = a.cls[node];
    if (c == CLS_SOLID) {
      if (o.f)
        for (int k = 0; k < 9; k++) o.f[cell * 9 + k] = 0.0;
      if (o.metaf)
        for (int k = 0; k < 9; k++) o.metaf[cell * 9 + k] = 0.0;
      if (o.rho) o.rho[cell] = o.rho_solid[cell];
      if (o.u) o.u[cell] = o.u_solid[cell];
      if (o.v) o.v[cell] = o.v_solid[cell];
      continue;
    }
    R F[9], M[9], rho, u, v;
    if (c != CLS_SPECIAL) {
      // bulk: all neighbours fluid, plain loads in the state's layout
#pragma unroll
      for (int k = 0; k < 9; k++) {
        F[k] = ST::cvt_dev(__ldg(src + slot_of<L>(k, node - nb(k, a.pitch), a)), k, a);
        M[k] = ST::cvt_dev(__ldg(src + slot_of<L>(k, node, a)), k, a);
      }
      moments_form<ST>(F, a, rho, u, v);
    } else {
      R mac[3];
      special_node<R>(a, acc_m, node, F, mac);
      rho = mac[0];
      u = mac[1];
      v = mac[2];
#pragma unroll
      for (int k = 0; k < 9; k++) M[k] = acc_m.meta(node, k);
    }
    R l2 = R(0);
#pragma unroll
    for (int k = 0; k < 9; k++) {
      R dk = F[k] - M[k];
      l2 += dk * dk;
    }
    if (o.f)
      for (int k = 0; k < 9; k++) o.f[cell * 9 + k] = (double)F[k] + (SH ? wgt<double>(k) * a.rho0 : 0.0);
    if (o.metaf)
      for (int k = 0; k < 9; k++) o.metaf[cell * 9 + k] = (double)M[k] + (SH ? wgt<double>(k) * a.rho0 : 0.0);
    if (o.rho) o.rho[cell] = (double)rho;
    if (o.u) o.u[cell] = (double)u;
    if (o.v) o.v[cell] = (double)v;
    const R uu = u * u + v * v;
    part[S_L2] += l2;
    part[S_MASS] += rho;
    part[S_MX] += rho * u;
    part[S_MY] += rho * v;
    part[S_UU] += uu;
    part[S_VMAX] = fmax(part[S_VMAX], sqrt(uu));
    if (rho != rho || u != u || v != v) part[S_NAN] += R(1);
    if (o.uprev) {
      const R pu = (R)o.uprev[cell], pv = (R)o.vprev[cell];
      part[S_DU] += (u - pu) * (u - pu) + (v - pv) * (v - pv);
      o.uprev[cell] = (float)u;
      o.vprev[cell] = (float)v;
    }
    if (c == CLS_SPECIAL) {
      const BRec &r = a.rec[a.aux[node]];
      if (r.flags & FL_DRAG) {
        // momentum exchange over the wall links of this cell, in FP64
        const uint32_t wall = (r.flags >> FL_WALL_SHIFT) & 0x1FFu;
        for (int k = 1; k < 9; k++)
          if ((wall >> k) & 1u) {
            double g = (double)M[k] + (double)F[OPP[k]] + (SH ? 2.0 * wgt<double>(k) * a.rho0 : 0.0);
            acc[S_FX] += g * CX[k];
            acc[S_FY] += g * CY[k];
          }
      }
    }
    if (std::is_same<R, double>::value || ++chunk == 8) {
      chunk = 0;
#pragma unroll
      for (int i = 0; i < NSUM; i++) {
        if (i == S_VMAX) acc[i] = fmax(acc[i], (double)part[i]);
        else if (i != S_FX && i != S_FY) acc[i] += (double)part[i];
        part[i] = R(0);
      }
    }
  }
#pragma unroll
  for (int i = 0; i < NSUM; i++) {
    if (i == S_VMAX) acc[i] = fmax(acc[i], (double)part[i]);
    else if (i != S_FX && i != S_FY) acc[i] += (double)part[i];
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
template <class ACC>
__device__ __forceinline__ void resid_body(const StepArgs &a, const ACC &acc_m, double *out) {
  using R = typename ACC::R;
  __shared__ double sh[3][256];
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

template <class ST, int L>
__global__ void __launch_bounds__(256) k_resid_ref(const __grid_constant__ StepArgs a, double *out) {
  resid_body<AccMain<ST, L>>(a, AccMain<ST, L>(a, a.src), out);
}

}  // namespace lbm
