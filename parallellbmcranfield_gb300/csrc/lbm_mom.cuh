// Moment storage (LBM_FP16NEQ): the state between launches is each node's
// post-collision moments instead of its nine post-collision populations.
//
// Why.  With 16-bit populations the rounding of every store lands in the
// conserved moments (mass and momentum), which no collision relaxes: the slow
// viscous modes sum those errors up and the steady state ends 1e-3..1e-2 off
// the FP64 one.  Stored as moments, the conserved ones keep 24 bits and only
// the six non-conserved moments are 16-bit; a rounding error there is
// relaxed by the next collision and reaches the momentum equation only as
// the divergence of a stress error.
//
// Per node (A-B pattern, 21 bytes):
//   planes 0..2   int16  high 16 bits of Q(rho - rho0), Q(j_x), Q(j_y)
//   planes 3..8   FP16   n_i = (m*_i - b_i) * neq_scale, i = 1, 2, 4, 6, 7, 8
//   bytes  0..2   uint8  low 8 bits of the three fixed-point values
// Layout: chunks of 64 consecutive nodes of a row (the pitch is a multiple
// of 256), 1344 bytes each, in node order; inside a chunk the nine 16-bit
// planes (128 bytes each) and then the three byte planes (64 bytes each).
// A node's twelve values are then at fixed offsets from one pointer, so a
// thread addresses a whole row with one pointer and immediate offsets.
// Q(x) = floor(x / step + u) is a 24-bit signed fixed-point number with a
// per-node, per-generation dither u in [0, 1) (unbiased rounding; steps from
// the host: the density range +-0.5 rho0, the momentum range +-0.25 rho0); a value
// beyond the range is not stored and sets the step's flag (value 2).  b_i is
// a storage reference, a polynomial of the stored conserved moments
// (b1 = -2 rho~ + 3 |j|^2, b2 = rho~ - 3 |j|^2, b4 = -j_x, b6 = -j_y,
// b7 = (j_x^2 - j_y^2) / rho0, b8 = j_x j_y / rho0; rho~ = rho - rho0), so that
// the stored n_i are the small non-equilibrium parts.  Moments are those of
// the reference's MRT transform (serial/CellFunctions.c:37-47) applied to the
// deviations d_k = f_k - w_k rho0.
//
// Nodes with boundary work (class 3) keep their post-collision populations
// in FP32 in a side array indexed by their record instead (the boundary
// treatment reads populations, and the corners' large non-equilibrium parts
// lose most to 16 bits).  Fluid nodes next to them (class 2 in this mode)
// are updated together with them by k_special_mom, so the bulk kernel never
// reads a class-3 node.
#pragma once
#include "lbm_device.cuh"

namespace lbm {

constexpr int MOM_QMAX = (1 << 23) - 1;     // largest fixed-point magnitude

constexpr int MOM_CH = 64;                // nodes per chunk
constexpr int MOM_CHB = 21 * MOM_CH;      // bytes per chunk
constexpr int MOM_LO_OFF = 18 * MOM_CH;   // first byte plane inside a chunk

// Byte offset of node z's 16-bit slot in plane 0 (the node's chunk plus
// two bytes per node before it in the chunk); plane p lies 128 p bytes on.
__device__ __forceinline__ long long mom_off(long long z) {
  return 21LL * (z & ~(long long)(MOM_CH - 1)) + 2 * (z & (MOM_CH - 1));
}
// Byte offset of node z's slot in byte plane 0; byte plane p lies 64 p on.
__device__ __forceinline__ long long mom_off_lo(long long z) {
  return 21LL * (z & ~(long long)(MOM_CH - 1)) + MOM_LO_OFF + (z & (MOM_CH - 1));
}
__device__ __forceinline__ const int16_t *mom_hi(const void *b, long long z, int p) {
  return (const int16_t *)((const char *)b + mom_off(z) + 2 * MOM_CH * p);
}
__device__ __forceinline__ const __half *mom_n(const void *b, long long z, int i) {
  return (const __half *)((const char *)b + mom_off(z) + 2 * MOM_CH * (3 + i));
}
__device__ __forceinline__ const uint8_t *mom_lo(const void *b, long long z, int p) {
  return (const uint8_t *)b + mom_off_lo(z) + MOM_CH * p;
}

// The stored moment set of one node in deviation form: r = rho - rho0,
// x = j_x, y = j_y, n[6] = m*_i - b_i (i = 1, 2, 4, 6, 7, 8).
struct MomSet {
  float r, x, y, n[6];
};

// Post-collision deviations d*_k = (Minv m*)_k of a stored moment set
// (Minv = (1/36) x integers, serial/CellFunctions.c:49-59).
__device__ __forceinline__ void mom_to_pops(const MomSet &s, const StepArgs &a, float d[9]) {
  const float jj = s.x * s.x + s.y * s.y, i0 = a.fx_irho0;
  const float m1 = fmaf(3.f, jj, -2.f * s.r) + s.n[0];
  const float m2 = fmaf(-3.f, jj, s.r) + s.n[1];
  const float m4 = s.n[2] - s.x, m6 = s.n[3] - s.y;
  const float m7 = (s.x * s.x - s.y * s.y) * i0 + s.n[4];
  const float m8 = s.x * s.y * i0 + s.n[5];
  const float c = 1.f / 36.f;
  const float ax = 4.f * s.r - m1 - 2.f * m2, dg = 4.f * s.r + 2.f * m1 + m2;
  const float P = 9.f * m7;
  const float Xd = fmaf(3.f, m4, 6.f * s.x), Yd = fmaf(3.f, m6, 6.f * s.y), Q = 9.f * m8;
  d[5] = c * (dg + Xd + Yd + Q);
  d[6] = c * (dg - Xd + Yd - Q);
  d[7] = c * (dg - Xd - Yd + Q);
  d[8] = c * (dg + Xd - Yd - Q);
  // c = 1/36 is not exact in FP32: Minv applied as above would scale mass and
  // momentum by 36 c = 1 + 7.5e-9 every step, a bias the slow modes sum up.
  // So only the non-conserved shape comes from Minv; the axis pairs take the
  // momentum that the diagonals leave and the rest population the mass, which
  // makes sum d = r and sum c d = j up to one rounding each.
  const float s13 = c * (2.f * ax + 2.f * P), s24 = c * (2.f * ax - 2.f * P);
  const float dx = s.x - ((d[5] - d[7]) + (d[8] - d[6]));
  const float dy = s.y - ((d[5] - d[7]) + (d[6] - d[8]));
  d[1] = 0.5f * (s13 + dx);
  d[3] = 0.5f * (s13 - dx);
  d[2] = 0.5f * (s24 + dy);
  d[4] = 0.5f * (s24 - dy);
  d[0] = s.r - (((d[1] + d[3]) + (d[2] + d[4])) + ((d[5] + d[7]) + (d[6] + d[8])));
}

// Fixed point <-> float of one conserved moment (p: 0 density, 1 and 2 momentum).
__device__ __forceinline__ float fx_step(const StepArgs &a, int p) { return p == 0 ? a.fx_rho : a.fx_j; }
__device__ __forceinline__ float fx_istep(const StepArgs &a, int p) { return p == 0 ? a.fx_irho : a.fx_ij; }

// Stored moment set of node z (any class but special; solid and padding
// nodes read as all zero, i.e. f = w rho0).
__device__ __forceinline__ MomSet mom_load(const StepArgs &a, const void *b, long long z) {
  MomSet s;
  float q[3];
#pragma unroll
  for (int p = 0; p < 3; p++) {
    const int hi = __ldg(mom_hi(b, z, p));
    const int lo = __ldg(mom_lo(b, z, p));
    q[p] = (float)(hi * 256 + lo) * fx_step(a, p);
  }
  s.r = q[0];
  s.x = q[1];
  s.y = q[2];
#pragma unroll
  for (int i = 0; i < 6; i++) s.n[i] = __half2float(__ldg(mom_n(b, z, i))) * a.neq_is;
  return s;
}

// Moments (deviation form) of deviation populations d: r, j and the six
// non-conserved ones in the order 1, 2, 4, 6, 7, 8.
__device__ __forceinline__ void pops_to_mom(const float d[9], float &r, float &jx, float &jy,
                                            float m[6]) {
  const float a13 = d[1] + d[3], a24 = d[2] + d[4], a14 = a13 + a24;
  const float p57 = d[5] + d[7], p68 = d[6] + d[8], a58 = p57 + p68;
  r = (d[0] + a14) + a58;
  const float d13 = d[1] - d[3], d24 = d[2] - d[4];
  const float e57 = d[5] - d[7], e86 = d[8] - d[6];
  const float x58 = e57 + e86, y58 = e57 - e86;
  jx = d13 + x58;
  jy = d24 + y58;
  m[0] = 2.f * a58 - a14 - 4.f * d[0];
  m[1] = (4.f * d[0] + a58) - 2.f * a14;
  m[2] = x58 - 2.f * d13;
  m[3] = y58 - 2.f * d24;
  m[4] = a13 - a24;
  m[5] = p57 - p68;
}

// Collision in moment space (deviation form; rho = rho0 + r).  MRT is the
// reference's operator (serial/CellFunctions.c:401-438: meq_1 = -2 rho +
// 3 |j|^2, meq_2 = rho - 3 |j|^2, s = 1.4, 1.4, 1.2, 1.2, omega, omega);
// BGK and TRT are the same relaxation of M f toward M f_eq with the
// second-order f_eq (meq_1 = -2 rho + 3 |j|^2 / rho, meq_2 = rho -
// 3 |j|^2 / rho), at rates omega (BGK) or omega for the even and omegaA for
// the odd moments 4, 6 (TRT, serial/CellFunctions.c:372-395).  m[] becomes
// the post-collision moments; r and j are conserved.
template <int MODEL>
__device__ __forceinline__ void collide_mom(float r, float jx, float jy, float m[6],
                                           const StepArgs &a) {
  const float rho = (float)a.rho0 + r;
  const float inv = 1.f / rho;
  const float jj = jx * jx + jy * jy;
  const float q = MODEL == 3 ? jj : jj * inv;
  const float e1 = fmaf(3.f, q, -2.f * r), e2 = fmaf(-3.f, q, r);
  const float e7 = (jx * jx - jy * jy) * inv, e8 = jx * jy * inv;
  const float om = (float)a.omega;
  const float s12 = MODEL == 3 ? 1.4f : om;
  const float s46 = MODEL == 3 ? 1.2f : (MODEL == 2 ? (float)a.omegaA : om);
  m[0] -= s12 * (m[0] - e1);
  m[1] -= s12 * (m[1] - e2);
  m[2] -= s46 * (m[2] + jx);
  m[3] -= s46 * (m[3] + jy);
  m[4] -= om * (m[4] - e7);
  m[5] -= om * (m[5] - e8);
}

// Fixed-point code of a conserved moment, rounded with a dither u in [0, 1):
// floor(v / step + u).  Rounding to nearest would give a node at steady state
// the same error every step, and the mass of the domain would drift by their
// sum each step; with the dither the expected code is v / step and the errors
// of successive steps are independent.  `ok` turns false out of range.
__device__ __forceinline__ int fx_code(float v, float istep, float u, bool &ok) {
  // x + u would round to the grid of x (1/8 at |x| ~ 2^20) and bias the
  // dither; the integer part and the fraction of x are exact instead
  const float x = v * istep;
  const float xi = floorf(x);
  const float t = xi + ((x - xi) > u ? 1.f : 0.f);
  ok = ok && fabsf(t) <= (float)MOM_QMAX;
  return (int)fminf(fmaxf(t, -(float)MOM_QMAX), (float)MOM_QMAX);
}

// 32-bit integer hash (the "lowbias32" finaliser of C. Wellons' hash-prospector
// search: xor-shift / multiply rounds); three 10-bit dithers per node and
// generation.
__device__ __forceinline__ uint32_t mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}
__device__ __forceinline__ void dithers(long long z, unsigned gen, float u[3]) {
  const uint32_t h = mix32((uint32_t)z ^ mix32(gen * 0x9e3779b9u + 0x632be5abu));
#pragma unroll
  for (int p = 0; p < 3; p++) u[p] = (float)((h >> (10 * p)) & 1023u) * (1.f / 1024.f) + (1.f / 2048.f);
}

// Encoded moment set (codes and FP16 non-equilibrium parts) of post-collision
// moments; the references b_i come from the stored (rounded) r and j.
struct MomCode {
  int q[3];
  __half n[6];
};
__device__ __forceinline__ MomCode mom_encode(float r, float jx, float jy, const float m[6],
                                              const StepArgs &a, long long z, bool &ok) {
  MomCode c;
  float u[3];
  dithers(z, a.gen, u);
  c.q[0] = fx_code(r, a.fx_irho, u[0], ok);
  c.q[1] = fx_code(jx, a.fx_ij, u[1], ok);
  c.q[2] = fx_code(jy, a.fx_ij, u[2], ok);
  const float rs = (float)c.q[0] * a.fx_rho, xs = (float)c.q[1] * a.fx_j,
              ys = (float)c.q[2] * a.fx_j;
  const float jj = xs * xs + ys * ys, i0 = a.fx_irho0;
  const float b[6] = {fmaf(3.f, jj, -2.f * rs), fmaf(-3.f, jj, rs), -xs, -ys,
                      (xs * xs - ys * ys) * i0, xs * ys * i0};
#pragma unroll
  for (int i = 0; i < 6; i++) c.n[i] = __float2half_rn((m[i] - b[i]) * a.neq_s);
  return c;
}

__device__ __forceinline__ void mom_store(const StepArgs &a, void *b, long long z,
                                          const MomCode &c) {
#pragma unroll
  for (int p = 0; p < 3; p++) {
    *(int16_t *)mom_hi(b, z, p) = (int16_t)(c.q[p] >> 8);
    *(uint8_t *)mom_lo(b, z, p) = (uint8_t)(c.q[p] & 0xff);
  }
#pragma unroll
  for (int i = 0; i < 6; i++) *(__half *)mom_n(b, z, i) = c.n[i];
}

// Out-of-range or non-finite result: the step's flag (checked by the host).
__device__ __forceinline__ void mom_flag(const StepArgs &a, bool ok, float probe) {
  if (a.nanflag) {
    if (!(fabsf(probe) <= 3.0e38f)) *a.nanflag = 1;
    else if (!ok) *a.nanflag = 2;
  }
}

// METAF of any node in deviation form (DEV) or absolute: class 3 from the
// FP32 side array of the current parity, solid as zero, others decoded.
template <bool DEV>
struct AccMom {
  using R = float;
  static constexpr bool dev = DEV;
  const StepArgs &a;
  __device__ AccMom(const StepArgs &a_, const void *) : a(a_) {}
  __device__ __forceinline__ float meta(long long z, int k) const {
    const uint8_t c = a.cls[z];
    const float w0 = wgt<float>(k) * (float)a.rho0;
    float d;
    if (c == CLS_SOLID) {
      d = -w0;
    } else if (c == CLS_SPECIAL) {
      d = a.ss_src[(size_t)a.aux[z] * 9 + k];
    } else {
      float p[9];
      mom_to_pops(mom_load(a, a.src, z), a, p);
      d = p[k];
    }
    return DEV ? d : d + w0;
  }
  // All nine METAF of a non-solid node (deviation form).
  __device__ __forceinline__ void all(long long z, float d[9]) const {
    if (a.cls[z] == CLS_SPECIAL) {
#pragma unroll
      for (int k = 0; k < 9; k++) d[k] = a.ss_src[(size_t)a.aux[z] * 9 + k];
    } else {
      mom_to_pops(mom_load(a, a.src, z), a, d);
    }
  }
};

// ------------------------------------------------------------------ bulk step
//
// The two nodes of a pair (x0, x0+1) travel together: their 32-bit words of
// the 16-bit planes, the 16-bit word of each byte plane, and packed FP32x2
// arithmetic (one FFMA2 / FADD2 / FMUL2 for both nodes).

// Raw stored words of one pair of one row.
struct MomRaw {
  uint32_t h[3];  // two int16 high parts
  uint32_t l[3];  // two low bytes (in the low 16 bits)
  uint32_t n[6];  // two FP16 non-equilibrium moments
};

// p16 / plo: the pair's slots in 16-bit plane 0 and byte plane 0 (mom_off,
// mom_off_lo of its first node, which is even: both nodes share a chunk).
__device__ __forceinline__ void mom_raw_load(const char *p16, const char *plo, MomRaw &w) {
#pragma unroll
  for (int p = 0; p < 3; p++) {
    w.h[p] = __ldg((const unsigned *)(p16 + 2 * MOM_CH * p));
    w.l[p] = (uint32_t)__ldg((const unsigned short *)(plo + MOM_CH * p));
  }
#pragma unroll
  for (int i = 0; i < 6; i++) w.n[i] = __ldg((const unsigned *)(p16 + 2 * MOM_CH * (3 + i)));
}

// Byte permute with the PTX default mode: a selector nibble with bit 3 set
// replicates the sign bit of the byte it selects (the __byte_perm intrinsic
// keeps only 3 bits per selector).
__device__ __forceinline__ int prmt_s(uint32_t a, uint32_t b, uint32_t sel) {
  uint32_t d;
  asm("prmt.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(sel));
  return (int)d;
}

// Post-collision deviations of both nodes of a pair (mom_to_pops on FP32
// pairs): each 24-bit code is the low byte, then the int16 high part, then
// the high part's sign replicated, in one permute.  The factor 1/36 of Minv
// and the storage scale of the n_i are folded into the constants, so that
// each diagonal population is two sums of terms formed by one multiply-add:
//   36 d_5..8 = (r + 3|j|^2 + 2 N1 + N2) +- 3 (x + N4) +- 3 (y + N6) +- 9 (x y / rho0 + N8)
//   36 (d_1 + d_3) / 2 = (4 r + 3|j|^2 - N1 - 2 N2) + 9 ((x^2 - y^2) / rho0 + N7)
// (N_i = n_i / neq_s; the axis pairs and d_0 as in mom_to_pops, so that mass
// and momentum are exact up to one rounding each).
__device__ __forceinline__ void mom_decode2(const StepArgs &a, const MomRaw &w, float2 d[9]) {
  float2 q[3];
#pragma unroll
  for (int p = 0; p < 3; p++) {
    const int q0 = prmt_s(w.l[p], w.h[p], 0xD540u);  // l.b0, h.b0, h.b1, sign(h.b1)
    const int q1 = prmt_s(w.l[p], w.h[p], 0xF761u);  // l.b1, h.b2, h.b3, sign(h.b3)
    q[p] = mul2(make_float2((float)q0, (float)q1), bc2(fx_step(a, p)));
  }
  float2 n[6];  // stored units (n_i * neq_s)
#pragma unroll
  for (int i = 0; i < 6; i++) {
    __half2 h;
    memcpy(&h, &w.n[i], 4);
    n[i] = __half22float2(h);
  }
  constexpr float is = 1.f / MOM_NEQ_S;
  const float2 r = q[0], x = q[1], y = q[2];
  const float2 yy = mul2(y, y);
  const float2 jj = fma2(x, x, yy);
  const float2 xmy = fma2(bc2(-2.f), yy, jj);  // x^2 - y^2
  const float2 xy = mul2(x, y);
  const float2 i4 = bc2(a.f_i4rho0);            // 1 / (4 rho0)
  // the four diagonal populations, already divided by 36
  const float2 dg = fma2(n[1], bc2(is / 36.f),
                         fma2(n[0], bc2(2.f * is / 36.f),
                              fma2(jj, bc2(1.f / 12.f), mul2(r, bc2(1.f / 36.f)))));
  const float2 Q = fma2(n[5], bc2(is / 4.f), mul2(xy, i4));
  const float2 Xd = fma2(n[2], bc2(is / 12.f), mul2(x, bc2(1.f / 12.f)));
  const float2 Yd = fma2(n[3], bc2(is / 12.f), mul2(y, bc2(1.f / 12.f)));
  const float2 gp = add2(dg, Q), gm = sub2(dg, Q), sp = add2(Xd, Yd), sm = sub2(Xd, Yd);
  d[5] = add2(gp, sp);
  d[6] = sub2(gm, sm);
  d[7] = sub2(gp, sp);
  d[8] = add2(gm, sm);
  // half the axis pairs' sums, divided by 36
  const float2 ax = fma2(n[1], bc2(-2.f * is / 36.f),
                         fma2(n[0], bc2(-is / 36.f),
                              fma2(jj, bc2(3.f / 36.f), mul2(r, bc2(4.f / 36.f)))));
  const float2 P = fma2(n[4], bc2(is / 4.f), mul2(xmy, i4));
  const float2 s13 = add2(ax, P), s24 = sub2(ax, P);
  // the momentum the diagonals leave goes to the axis pairs (see mom_to_pops)
  const float2 e57 = sub2(d[5], d[7]), e86 = sub2(d[8], d[6]);
  const float2 dx = sub2(x, add2(e57, e86));
  const float2 dy = sub2(y, sub2(e57, e86));
  d[1] = fma2(dx, bc2(0.5f), s13);
  d[3] = fma2(dx, bc2(-0.5f), s13);
  d[2] = fma2(dy, bc2(0.5f), s24);
  d[4] = fma2(dy, bc2(-0.5f), s24);
  d[0] = sub2(r, add2(add2(add2(d[1], d[3]), add2(d[2], d[4])),
                      add2(add2(d[5], d[7]), add2(d[6], d[8]))));
}

// Moments of pulled deviations (pops_to_mom on pairs).
__device__ __forceinline__ void pops_to_mom2(const float2 d[9], float2 &r, float2 &jx, float2 &jy,
                                             float2 m[6]) {
  const float2 a13 = add2(d[1], d[3]), a24 = add2(d[2], d[4]), a14 = add2(a13, a24);
  const float2 p57 = add2(d[5], d[7]), p68 = add2(d[6], d[8]), a58 = add2(p57, p68);
  r = add2(add2(d[0], a14), a58);
  const float2 d13 = sub2(d[1], d[3]), d24 = sub2(d[2], d[4]);
  const float2 e57 = sub2(d[5], d[7]), e86 = sub2(d[8], d[6]);
  const float2 x58 = add2(e57, e86), y58 = sub2(e57, e86);
  jx = add2(d13, x58);
  jy = add2(d24, y58);
  m[0] = sub2(fma2(bc2(2.f), a58, mul2(bc2(-4.f), d[0])), a14);
  m[1] = fma2(bc2(-2.f), a14, fma2(bc2(4.f), d[0], a58));
  m[2] = fma2(bc2(-2.f), d13, x58);
  m[3] = fma2(bc2(-2.f), d24, y58);
  m[4] = sub2(a13, a24);
  m[5] = sub2(p57, p68);
}

// Collision (collide_mom on pairs) and encoding of a pair's pulled moments
// (r, j and the pre-collision non-equilibrium moments m), and the stores of
// the nodes whose `own` flag is set (both: full words; one: its own
// elements).  Each stored value is one expression: with the relaxation rate
// s_i, the equilibrium e_i of the pulled r, j and the storage reference b_i
// of the stored (rounded) r, j,
//   n_i = S (m_i - s_i (m_i - e_i) - b_i) = S (1 - s_i) m_i + S s_i e_i - S b_i
// (S = neq_s; the products S s_i and S (1 - s_i) come from the host).  The
// largest |rho - rho0| and |j| of the stored nodes go to rmax / jmax (the
// caller compares them with the fixed-point range once, at the end of its
// walk), their density deviation and stored n_7 to the NaN probe.
template <int MODEL>
__device__ __forceinline__ void mom_collide_store2(const StepArgs &a, char *p16, char *plo,
                                                   long long z, uint32_t hseed, float2 r,
                                                   float2 jx, float2 jy, const float2 m[6],
                                                   bool own0, bool own1, float &rmax, float &jmax,
                                                   float &probe) {
  // Dithered codes in integers: R = round(2^D v / step), t = (R + u) >> D
  // with u uniform in 0 .. 2^D - 1, so that E[t] = R / 2^D, within 2^-(D+1)
  // of v / step.  The pair's dithers come from one hash: node 0 in bits
  // 0..15, node 1 in 16..31; D = 6 for rho, 5 for each j.  Values beyond the
  // range show in rmax / jmax; a NaN converts to 0 and is caught by the
  // caller's probe instead.
  const uint32_t h = mix32((uint32_t)z ^ hseed);
  const float2 v[3] = {r, jx, jy};
  const int sh[3] = {0, 6, 11}, nb[3] = {6, 5, 5};
  int q0[3], q1[3];
  float2 qf[3];
#pragma unroll
  for (int p = 0; p < 3; p++) {
    const uint32_t mask = (1u << nb[p]) - 1u;
    const float2 x = mul2(v[p], bc2(a.fx_enc[p == 0 ? 0 : 1]));
    const uint32_t R0 = (uint32_t)__float2int_rn(x.x), R1 = (uint32_t)__float2int_rn(x.y);
    q0[p] = (int)(R0 + ((h >> sh[p]) & mask)) >> nb[p];
    q1[p] = (int)(R1 + ((h >> (16 + sh[p])) & mask)) >> nb[p];
    qf[p] = make_float2((float)q0[p], (float)q1[p]);
  }
  if (own0) {
    rmax = fmaxf(rmax, fabsf(r.x));
    jmax = fmaxf(jmax, fmaxf(fabsf(jx.x), fabsf(jy.x)));
  }
  if (own1) {
    rmax = fmaxf(rmax, fabsf(r.y));
    jmax = fmaxf(jmax, fmaxf(fabsf(jx.y), fabsf(jy.y)));
  }
  // -S b_i of the stored conserved moments, from the codes with the
  // fixed-point steps folded into the constants (enc_c)
  const float2 qr = qf[0], qx = qf[1], qy = qf[2];
  const float2 qyy = mul2(qy, qy);
  const float2 qjj = fma2(qx, qx, qyy);
  const float2 qxmy = fma2(bc2(-2.f), qyy, qjj);
  const float2 c5 = bc2(a.enc_c[5]), c4 = bc2(a.enc_c[4]);
  const float2 mref[6] = {fma2(qjj, bc2(a.enc_c[1]), mul2(qr, bc2(a.enc_c[0]))),
                          fma2(qjj, bc2(a.enc_c[3]), mul2(qr, bc2(a.enc_c[2]))), mul2(qx, c4),
                          mul2(qy, c4), mul2(qxmy, c5), mul2(mul2(qx, qy), c5)};
  // equilibria of the pulled r, j (the reference's MRT: e_1 = -2 r + 3 |j|^2,
  // e_2 = r - 3 |j|^2, e_4 = -j_x, e_6 = -j_y, e_7 = (j_x^2 - j_y^2) / rho,
  // e_8 = j_x j_y / rho; BGK and TRT with |j|^2 / rho).  1 / rho enters only
  // the equilibria of the non-conserved moments, whose stored form keeps 11
  // bits: the approximate reciprocal is ample
  const float2 rho = add2(bc2(a.f_rho0), r);
  const float2 inv = make_float2(__fdividef(1.f, rho.x), __fdividef(1.f, rho.y));
  const float2 jyy = mul2(jy, jy);
  const float2 jj = fma2(jx, jx, jyy);
  const float2 q = MODEL == 3 ? jj : mul2(jj, inv);
  const float2 e7 = mul2(fma2(bc2(-2.f), jyy, jj), inv), e8 = mul2(mul2(jx, jy), inv);
  const float *es = a.enc_s;  // S s_12 x (3, -2, 1, -3), S (1 - s_12), -S s_46, S (1 - s_46), S om, S (1 - om)
  float2 n[6];
  n[0] = fma2(m[0], bc2(es[4]), fma2(q, bc2(es[0]), fma2(r, bc2(es[1]), mref[0])));
  n[1] = fma2(m[1], bc2(es[4]), fma2(q, bc2(es[3]), fma2(r, bc2(es[2]), mref[1])));
  n[2] = fma2(m[2], bc2(es[6]), fma2(jx, bc2(es[5]), mref[2]));
  n[3] = fma2(m[3], bc2(es[6]), fma2(jy, bc2(es[5]), mref[3]));
  n[4] = fma2(m[4], bc2(es[8]), fma2(e7, bc2(es[7]), mref[4]));
  n[5] = fma2(m[5], bc2(es[8]), fma2(e8, bc2(es[7]), mref[5]));
  if (own0) probe += r.x + n[4].x;
  if (own1) probe += r.y + n[4].y;
  uint32_t nw[6];
#pragma unroll
  for (int i = 0; i < 6; i++) {
    const __half2 hh = __float22half2_rn(n[i]);
    memcpy(&nw[i], &hh, 4);
  }
  if (own0 && own1) {
#pragma unroll
    for (int p = 0; p < 3; p++) {
      *(uint32_t *)(p16 + 2 * MOM_CH * p) = __byte_perm((uint32_t)q0[p], (uint32_t)q1[p], 0x6521);
      *(unsigned short *)(plo + MOM_CH * p) =
          (unsigned short)__byte_perm((uint32_t)q0[p], (uint32_t)q1[p], 0x0040);
    }
#pragma unroll
    for (int i = 0; i < 6; i++) *(uint32_t *)(p16 + 2 * MOM_CH * (3 + i)) = nw[i];
  } else if (own0 || own1) {
    const int e = own0 ? 0 : 1;
#pragma unroll
    for (int p = 0; p < 3; p++) {
      const int q = e ? q1[p] : q0[p];
      *(int16_t *)(p16 + 2 * MOM_CH * p + 2 * e) = (int16_t)(q >> 8);
      *(uint8_t *)(plo + MOM_CH * p + e) = (uint8_t)(q & 0xff);
    }
#pragma unroll
    for (int i = 0; i < 6; i++)
      *(unsigned short *)(p16 + 2 * MOM_CH * (3 + i) + 2 * e) =
          (unsigned short)(e ? nw[i] >> 16 : nw[i] & 0xffffu);
  }
}

// Bulk step of the moment storage (A-B).  A warp covers 60 columns: lane l
// holds the pair (x0, x0+1), x0 = 60 w - 2 + 2 l; lanes 1..30 own their
// destination nodes and lanes 0 and 31 decode the pairs just outside, so
// that every +-1 x-shift is a warp shuffle and all lanes run the same
// instructions (no divergent halo path).  Each thread walks NPT destination
// rows: source row r, decoded once, hands its populations with c_y = +1 to
// destination row r+1, c_y = 0 to row r and c_y = -1 to row r-1, which is
// then complete: it collides and stores (class-1 nodes only; class 2 and 3
// belong to k_special_mom, solid nodes are never written).  The raw words of
// source rows are loaded one or two rows ahead (LD) into a ring of three,
// from addresses clamped into the domain, and lanes 0..23 prefetch the
// warp's span of row r + MOM_PF and its class bytes into L2 (a hint: nothing
// waits for it, every prefetched address lies inside the row).  Rows are
// addressed by one pointer per thread and row (the chunked layout), each
// value at an immediate offset from it.  Every lane runs the collision and
// the encoding; only the nodes a lane owns are stored.
// The row walk is a loop over groups of three rows, the period of the ring
// and of the three population rows, so that the code stays small.
constexpr int MOM_PF = 6;

struct MomWalk {
  MomRaw raw[3];
  float2 Fa[9], Fb[9], Fc[9];
  float rmax, jmax;        // largest |rho - rho0|, |j| stored (range check at the end)
  float probe;
  int rowb;                // bytes per row of a moment buffer (21 x pitch)
  int o16, olo;            // the pair's slot offsets within a row (mom_off, mom_off_lo of x0)
  int pf0, pf1;            // the warp's span of a row, [pf0, pf1) bytes within the row
};

// Row j of the walk (source row y0 + j); PH = (j + 1) mod 3 selects the ring
// slots: row j decodes slot PH and loads row j + LD into slot (PH + LD) mod 3
// (LD = 1 or 2 rows ahead: 12 or 24 registers of loads in flight).
template <int MODEL, int NPT, bool PF, int LD, int PH>
__device__ __forceinline__ void mom_walk_row(const StepArgs &a, MomWalk &w, int j, int y0, int wx,
                                             int x0, int lane, bool owner,
                                             uint32_t hseed) {
  const unsigned FULL = 0xffffffffu;
  const int r = y0 + j;
  const char *src = (const char *)a.src;
  if (j + LD <= NPT) {
    const long long rb = (long long)min(r + LD, a.m - 1) * w.rowb;
    mom_raw_load(src + rb + w.o16, src + rb + w.olo, w.raw[(PH + LD) % 3]);
  }
  // class word of this row's destination row r - 1, loaded before the
  // decode so that the arithmetic covers its latency
  const int y = r - 1;
  const uint32_t cw = j >= 1 && owner && y < a.m
                          ? __ldg((const unsigned short *)(a.cls + (long long)y * a.pitch + x0))
                          : 0u;
  if (PF) {
    // one 128-byte line per lane: the warp's span of a row is one or two
    // whole chunks (at most 2688 bytes, 22 lines at a 64-byte offset) for
    // lanes 0..21, the span's class bytes (64 bytes, at most two lines) for
    // lanes 22 and 23; the last address of each is clamped into the span.
    // A predicated instruction, not a branch: lanes 24..31 and rows past
    // the domain issue nothing (their addresses are formed, not used).
    const int rp = r + MOM_PF;
    const bool go = lane < 24 && rp < a.m && j + MOM_PF <= NPT;
    const char *p = lane < 22 ? src + (long long)rp * w.rowb + min(w.pf0 + 128 * lane, w.pf1 - 1)
                              : (const char *)a.cls + (long long)rp * a.pitch +
                                    (lane == 22 ? max(wx - 2, 0) : min(wx + 61, a.pitch - 1));
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %1, 0;\n\t@p prefetch.global.L2 [%0];\n\t}" ::"l"(p),
        "r"((unsigned)go));
  }
  float2 d[9];
  mom_decode2(a, w.raw[PH], d);
#pragma unroll
  for (int k = 0; k < 9; k++) {
    float2 v = d[k];
    if (CX[k] == 1) {
      const float left = __shfl_up_sync(FULL, d[k].y, 1);
      v = make_float2(left, d[k].x);
    } else if (CX[k] == -1) {
      const float right = __shfl_down_sync(FULL, d[k].x, 1);
      v = make_float2(d[k].y, right);
    }
    if (CY[k] == 1) w.Fc[k] = v;
    else if (CY[k] == 0) w.Fb[k] = v;
    else w.Fa[k] = v;
  }
  if (j >= 1) {  // destination row r - 1 is complete
    const bool own0 = (cw & 0xffu) == CLS_BULK;
    const bool own1 = (cw >> 8) == CLS_BULK && x0 + 1 < a.n;
    // every lane runs the arithmetic (no divergent branch around it); only
    // the nodes a lane owns are stored and counted
    float2 rr, jx, jy, m[6];
    pops_to_mom2(w.Fa, rr, jx, jy, m);
    char *dst = (char *)a.dst + (long long)y * w.rowb;
    mom_collide_store2<MODEL>(a, dst + w.o16, dst + w.olo, (long long)y * a.pitch + x0, hseed, rr,
                              jx, jy, m, own0, own1, w.rmax, w.jmax, w.probe);
  }
#pragma unroll
  for (int k = 0; k < 9; k++) {
    w.Fa[k] = w.Fb[k];
    w.Fb[k] = w.Fc[k];
  }
}

template <int MODEL, int NPT, int MINB, bool PF, int LD>
__global__ void __launch_bounds__(128, MINB) k_step_mom(const __grid_constant__ StepArgs a) {
  static_assert((NPT + 2) % 3 == 0, "the row walk runs in groups of three rows");
  static_assert(LD == 1 || LD == 2, "source rows are loaded one or two rows ahead");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wx = (blockIdx.x * 4 + warp) * 60;
  if (wx >= a.n) return;  // the whole warp lies past the row
  const int x0 = wx - 2 + 2 * lane;
  const bool owner = lane >= 1 && lane <= 30 && x0 < a.n;
  const int y0 = blockIdx.y * NPT;
  if (y0 - 1 >= a.m) return;
  const uint32_t hseed = mix32(a.gen * 0x9e3779b9u + 0x632be5abu);
  MomWalk w;
  w.rowb = 21 * a.pitch;  // the host keeps 21 x pitch below 2^31
  // Loads are unconditional: a pair left or right of the row (x0 = -2, or
  // x0 >= pitch) reads the row's first or last pair, a row above or below
  // the domain its first or last row.  Those values reach only nodes that
  // are not bulk nodes (the domain's edge columns and rows are never class
  // 1), which this kernel does not store.
  const int x0c = min(max(x0, 0), a.pitch - 2);
  w.o16 = (int)mom_off(x0c);
  w.olo = (int)mom_off_lo(x0c);
  // chunks met by the warp's columns wx - 2 .. wx + 61 (clamped to the row)
  w.pf0 = MOM_CHB * (max(wx - 2, 0) / MOM_CH);
  w.pf1 = MOM_CHB * (min(wx + 61, a.pitch - 1) / MOM_CH + 1);
  {
    const char *src = (const char *)a.src;
    const long long rm = (long long)min(max(y0 - 1, 0), a.m - 1) * w.rowb;
    const long long r0 = (long long)min(y0, a.m - 1) * w.rowb;
    mom_raw_load(src + rm + w.o16, src + rm + w.olo, w.raw[0]);
    if (LD == 2) mom_raw_load(src + r0 + w.o16, src + r0 + w.olo, w.raw[1]);
  }
#pragma unroll
  for (int k = 0; k < 9; k++) w.Fa[k] = w.Fb[k] = w.Fc[k] = make_float2(0.f, 0.f);
  w.rmax = w.jmax = 0.f;
  w.probe = 0.f;
  // the last group may run past the domain's last row: rows past it load
  // nothing and store nothing
#pragma unroll 1
  for (int j = -1; j <= NPT && y0 + j - 1 < a.m; j += 3) {
    mom_walk_row<MODEL, NPT, PF, LD, 0>(a, w, j, y0, wx, x0, lane, owner, hseed);
    mom_walk_row<MODEL, NPT, PF, LD, 1>(a, w, j + 1, y0, wx, x0, lane, owner, hseed);
    mom_walk_row<MODEL, NPT, PF, LD, 2>(a, w, j + 2, y0, wx, x0, lane, owner, hseed);
  }
  mom_flag(a, w.rmax <= a.fx_rlim && w.jmax <= a.fx_jlim, w.probe);
}

// Nodes with boundary work (class 3) and their fluid neighbours (class 2),
// one thread each, from a compact list.  Class 3: the reference's boundary
// treatment (special_node, on the populations the accessor reconstructs),
// collision, FP32 side array.  Class 2: pull (from side array or decoded
// moments), collision, moment store.
template <int MODEL>
__global__ void __launch_bounds__(128) k_special_mom(const __grid_constant__ StepArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.mlist_n) return;
  const long long node = a.mlist[i];
  const uint8_t c = a.cls[node];
  AccMom<true> acc(a, nullptr);
  float F[9], M[9];
  if (c == CLS_SPECIAL) {
    float mac[3];
    special_node<float>(a, acc, node, F, mac);
    collide_dev<MODEL>(F, mac[0], mac[1], mac[2], a, M);
    float *o = a.ss_dst + (size_t)a.aux[node] * 9;
#pragma unroll
    for (int k = 0; k < 9; k++) o[k] = M[k];
    return;
  }
#pragma unroll
  for (int k = 0; k < 9; k++) F[k] = acc.meta(node - nb(k, a.pitch), k);
  float rr, jx, jy, m[6];
  pops_to_mom(F, rr, jx, jy, m);
  collide_mom<MODEL>(rr, jx, jy, m, a);
  bool ok = true;
  const MomCode code = mom_encode(rr, jx, jy, m, a, node, ok);
  mom_flag(a, ok, rr + m[4]);
  mom_store(a, a.dst, node, code);
}

// First collision after lbm_set_state: f = f0 or f_eq(rho, u, v), collided,
// stored in the moment form (class 3 in the side array).
template <int MODEL>
__global__ void __launch_bounds__(128) k_init_mom(const __grid_constant__ StepArgs a,
                                                  const double *f0, const double *rho0,
                                                  const double *u0, const double *v0) {
  int x, y;
  if (!node_xy(a, x, y)) return;
  const long long node = (long long)y * a.pitch + x;
  const long long cell = (long long)y * a.n + x;
  const uint8_t c = a.cls[node];
  if (c == CLS_SOLID) return;
  const double rho = rho0[cell], u = u0[cell], v = v0[cell];
  double fe[9];
  if (f0) {
#pragma unroll
    for (int k = 0; k < 9; k++) fe[k] = f0[cell * 9 + k];
  } else {
    equilibrium<double>(rho, u, v, fe);
  }
  float F[9], M[9];
#pragma unroll
  for (int k = 0; k < 9; k++) F[k] = (float)(fe[k] - wgt<double>(k) * a.rho0);
  collide_dev<MODEL>(F, (float)rho, (float)u, (float)v, a, M);
  if (c == CLS_SPECIAL) {
    float *o = a.ss_dst + (size_t)a.aux[node] * 9;
#pragma unroll
    for (int k = 0; k < 9; k++) o[k] = M[k];
    return;
  }
  float rr, jx, jy, m[6];
  pops_to_mom(M, rr, jx, jy, m);
  bool ok = true;
  const MomCode code = mom_encode(rr, jx, jy, m, a, node, ok);
  mom_flag(a, ok, rr + m[4]);
  mom_store(a, a.dst, node, code);
}

// Read-only: F_{t+1}, macroscopic fields and FP64 diagnostics (the sums of
// k_finish, same lanes and launch shape) through the moment accessor.
__global__ void __launch_bounds__(128) k_finish_mom(const __grid_constant__ StepArgs a,
                                                    const FinishOut o) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[NSUM];
  float part[NSUM];
#pragma unroll
  for (int i = 0; i < NSUM; i++) acc[i] = 0.0, part[i] = 0.f;
  AccMom<true> am(a, nullptr);
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
    float F[9], M[9], rho, u, v;
    if (c != CLS_SPECIAL) {
#pragma unroll
      for (int k = 0; k < 9; k++) F[k] = am.meta(node - nb(k, a.pitch), k);
      const float rt = ((F[0] + F[1]) + (F[2] + F[3])) + ((F[4] + F[5]) + (F[6] + F[7])) + F[8];
      const float jx = (F[1] - F[3]) + (F[5] - F[6]) + (F[8] - F[7]);
      const float jy = (F[2] - F[4]) + (F[5] - F[7]) + (F[6] - F[8]);
      rho = (float)a.rho0 + rt;
      u = jx / rho;
      v = jy / rho;
    } else {
      float mac[3];
      special_node<float>(a, am, node, F, mac);
      rho = mac[0];
      u = mac[1];
      v = mac[2];
    }
    am.all(node, M);
    float l2 = 0.f;
#pragma unroll
    for (int k = 0; k < 9; k++) {
      const float dk = F[k] - M[k];
      l2 += dk * dk;
    }
    if (o.f)
      for (int k = 0; k < 9; k++) o.f[cell * 9 + k] = (double)F[k] + wgt<double>(k) * a.rho0;
    if (o.metaf)
      for (int k = 0; k < 9; k++) o.metaf[cell * 9 + k] = (double)M[k] + wgt<double>(k) * a.rho0;
    if (o.rho) o.rho[cell] = (double)rho;
    if (o.u) o.u[cell] = (double)u;
    if (o.v) o.v[cell] = (double)v;
    const float uu = u * u + v * v;
    part[S_L2] += l2;
    part[S_MASS] += rho;
    part[S_MX] += rho * u;
    part[S_MY] += rho * v;
    part[S_UU] += uu;
    part[S_VMAX] = fmaxf(part[S_VMAX], sqrtf(uu));
    if (rho != rho || u != u || v != v) part[S_NAN] += 1.f;
    if (o.uprev) {
      const float pu = o.uprev[cell], pv = o.vprev[cell];
      part[S_DU] += (u - pu) * (u - pu) + (v - pv) * (v - pv);
      o.uprev[cell] = u;
      o.vprev[cell] = v;
    }
    if (c == CLS_SPECIAL) {
      const BRec &r = a.rec[a.aux[node]];
      if (r.flags & FL_DRAG) {
        const uint32_t wall = (r.flags >> FL_WALL_SHIFT) & 0x1FFu;
        for (int k = 1; k < 9; k++)
          if ((wall >> k) & 1u) {
            const double g = (double)M[k] + (double)F[OPP[k]] + 2.0 * wgt<double>(k) * a.rho0;
            acc[S_FX] += g * CX[k];
            acc[S_FY] += g * CY[k];
          }
      }
    }
    if (++chunk == 8) {
      chunk = 0;
#pragma unroll
      for (int i = 0; i < NSUM; i++) {
        if (i == S_VMAX) acc[i] = fmax(acc[i], (double)part[i]);
        else if (i != S_FX && i != S_FY) acc[i] += (double)part[i];
        part[i] = 0.f;
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

}  // namespace lbm
