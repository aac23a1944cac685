// Surrogate network for warm starts: a 4-level convolutional encoder-decoder
// (U-Net with skip connections) mapping (geometry mask, boundary-velocity
// map, Re, velocity scale) on an H x W grid to the steady (rho, u, v).
//
// Everything runs in this file's kernels: activations and weights in BF16
// (NHWC), every product on the tensor cores (mma.sync m16n8k16 BF16 with FP32
// accumulation) through an explicit im2col + GEMM formulation, FP32 master
// weights, bias/ReLU/pool/upsample/concat/loss kernels and Adam.
//
// Convolution as GEMM (pixels p = B*H*W rows, K = 9*Cin padded to 32):
//   forward       Y[p][co]   = relu(sum_k A[p][k] Wt[co][k] + b[co]),  A = im2col(X)
//   input grad    dX[p][ci]  = sum_k A'[p][k] Wd[ci][k],  A' = im2col(dZ), Wd = flipped W
//   weight grad   dW[co][k]  = sum_p dZ[p][co] A[p][k]   (split-K over p, FP32 atomics)
// The GEMM kernel takes both operands K-contiguous (A[M][K], Bt[N][K]).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "lbm_internal.h"
#include "lbm_tc.cuh"

using lbm::fail;
typedef __nv_bfloat16 bf16;

namespace {

// ------------------------------------------------------------------ kernels

constexpr int GBM = 128, GBK = 32, GPAD = 8, GSTAGES = 3;

enum Epi : int {
  EPI_BIAS_RELU_BF16 = 0,  // forward conv with ReLU
  EPI_BIAS_BF16 = 1,       // forward conv without activation (output layer)
  EPI_BF16 = 2,            // plain product to BF16 (input gradients)
  EPI_ATOMIC_F32 = 3       // split-K accumulation into FP32 (weight gradients)
};

struct GemmArgs {
  const bf16 *A;   // [M][K] (explicit operand)
  const bf16 *X;   // [B][H][W][C] source of the implicit im2col operand
  int H, W, C, taps;
  const bf16 *Bt;  // [N][K]
  int M, N, K;     // K multiple of GBK
  int kchunk;      // K range per blockIdx.z (multiple of GBK)
  const float *bias;
  bf16 *out_bf16;  // [M][N]
  float *out_f32;  // [M][N]
};

__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], const uint32_t b[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// 16-byte global -> shared copy; with pred false the 16 bytes are zero-filled
// and nothing is read (src-size 0).
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, bool pred) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  const int n = pred ? 16 : 0;
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(gmem), "r"(n));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

// Four transposed 8x8 BF16 matrices from shared memory (one row address per lane).
__device__ __forceinline__ void ldsm_x4_t(uint32_t r[4], const void *row) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(row);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(sa));
}

// C[M][N] = A[M][K] x Bt[N][K]^T.  256 threads: 8 warps as 4 (M) x 2 (N), each
// warp 32 x BN/2; K in tiles of 32 through a GSTAGES-deep cp.async ring.  With
// GATHER the A operand is the im2col of X, formed while loading: row p is a
// pixel, column k = r*C + c is channel c of the pixel at tap offset r (3x3,
// pad 1, or 1x1), zero for k >= taps*C; C is a multiple of 8, so every
// 16-byte chunk of a row lies within one tap.
template <int EPI, bool GATHER, int BN>
__global__ void __launch_bounds__(256) k_gemm(const GemmArgs g) {
  constexpr int NJ = BN / 16;  // n8 tiles per warp
  __shared__ __align__(16) bf16 As[GSTAGES][GBM][GBK + GPAD];
  __shared__ __align__(16) bf16 Bs[GSTAGES][BN][GBK + GPAD];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp & 3, wn = warp >> 2;
  const int m0 = blockIdx.x * GBM, n0 = blockIdx.y * BN;
  const int kbeg = blockIdx.z * g.kchunk;
  const int kend = min(g.K, kbeg + g.kchunk);
  const int nk = (kend - kbeg) / GBK;
  // the two A chunks (row, 8-column group) this thread loads in every stage
  int arow[2], ac8[2], ay[2] = {0, 0}, ax[2] = {0, 0};
  bool aok[2];
#pragma unroll
  for (int it = 0; it < 2; it++) {
    const int ch = tid + it * 256;
    arow[it] = ch >> 2;
    ac8[it] = (ch & 3) * 8;
    const int p = m0 + arow[it];
    aok[it] = p < g.M;
    if (GATHER) {
      ax[it] = p % g.W;
      ay[it] = (p / g.W) % g.H;
    }
  }
  auto load = [&](int stage, int k0) {
#pragma unroll
    for (int it = 0; it < 2; it++) {
      const int p = m0 + arow[it];
      const bf16 *src = g.Bt;  // any valid address when nothing is read
      bool ok = aok[it];
      if (GATHER) {
        const int kk = k0 + ac8[it];
        const int r = kk / g.C, c = kk - r * g.C;
        const int dy = g.taps == 9 ? r / 3 - 1 : 0, dx = g.taps == 9 ? r % 3 - 1 : 0;
        const int yy = ay[it] + dy, xx = ax[it] + dx;
        ok = ok && r < g.taps && yy >= 0 && yy < g.H && xx >= 0 && xx < g.W;
        if (ok) src = g.X + (size_t)(p + dy * g.W + dx) * g.C + c;
      } else if (ok) {
        src = g.A + (size_t)p * g.K + k0 + ac8[it];
      }
      cp_async16(&As[stage][arow[it]][ac8[it]], src, ok);
    }
    if (tid < BN * 4) {
      const int r = tid >> 2, c8 = (tid & 3) * 8;
      const bool ok = n0 + r < g.N;
      cp_async16(&Bs[stage][r][c8], ok ? g.Bt + (size_t)(n0 + r) * g.K + k0 + c8 : g.Bt, ok);
    }
  };
  float acc[2][NJ][4];
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < NJ; j++)
#pragma unroll
      for (int r = 0; r < 4; r++) acc[i][j][r] = 0.f;
  const int gq = lane >> 2, tq = lane & 3;
#pragma unroll
  for (int st = 0; st < GSTAGES - 1; st++) {
    if (st < nk) load(st, kbeg + st * GBK);
    cp_async_commit();
  }
  for (int kt = 0; kt < nk; kt++) {
    cp_async_wait<GSTAGES - 2>();
    __syncthreads();
    if (kt + GSTAGES - 1 < nk) load((kt + GSTAGES - 1) % GSTAGES, kbeg + (kt + GSTAGES - 1) * GBK);
    cp_async_commit();
    const int stg = kt % GSTAGES;
#pragma unroll
    for (int kk = 0; kk < GBK; kk += 16) {
      uint32_t af[2][4], bfr[NJ][2];
#pragma unroll
      for (int i = 0; i < 2; i++) {
        const int r = wm * 32 + i * 16 + gq;
        af[i][0] = *(const uint32_t *)&As[stg][r][kk + 2 * tq];
        af[i][1] = *(const uint32_t *)&As[stg][r + 8][kk + 2 * tq];
        af[i][2] = *(const uint32_t *)&As[stg][r][kk + 2 * tq + 8];
        af[i][3] = *(const uint32_t *)&As[stg][r + 8][kk + 2 * tq + 8];
      }
#pragma unroll
      for (int j = 0; j < NJ; j++) {
        const int c = wn * (BN / 2) + j * 8 + gq;
        bfr[j][0] = *(const uint32_t *)&Bs[stg][c][kk + 2 * tq];
        bfr[j][1] = *(const uint32_t *)&Bs[stg][c][kk + 2 * tq + 8];
      }
#pragma unroll
      for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < NJ; j++) mma_bf16(acc[i][j], af[i], bfr[j]);
    }
  }
  cp_async_wait<0>();
  // epilogue: c0,c1 at (row gq, cols 2tq, 2tq+1), c2,c3 at row gq+8
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < NJ; j++)
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int row = m0 + wm * 32 + i * 16 + gq + h * 8;
        if (row >= g.M) continue;
        const int col = n0 + wn * (BN / 2) + j * 8 + 2 * tq;
        const size_t o = (size_t)row * g.N + col;
        float v0 = acc[i][j][h * 2], v1 = acc[i][j][h * 2 + 1];
        if (EPI == EPI_ATOMIC_F32) {
          if (col < g.N) atomicAdd(g.out_f32 + o, v0);
          if (col + 1 < g.N) atomicAdd(g.out_f32 + o + 1, v1);
          continue;
        }
        if (EPI != EPI_BF16) {
          if (col < g.N) v0 += g.bias[col];
          if (col + 1 < g.N) v1 += g.bias[col + 1];
        }
        if (EPI == EPI_BIAS_RELU_BF16) {
          v0 = fmaxf(v0, 0.f);
          v1 = fmaxf(v1, 0.f);
        }
        if (col + 1 < g.N && (g.N & 1) == 0) {
          *(__nv_bfloat162 *)(g.out_bf16 + o) = __floats2bfloat162_rn(v0, v1);
        } else {
          if (col < g.N) g.out_bf16[o] = __float2bfloat16_rn(v0);
          if (col + 1 < g.N) g.out_bf16[o + 1] = __float2bfloat16_rn(v1);
        }
      }
}

// Weight gradient of a convolution without im2col in memory:
// dW[co][k] += sum over pixels p of dZ[p][co] * X[p at tap r(k)][c(k)],
// k = r*C + c < taps*C, C and Cout multiples of 8.  128 threads as 2 (Cout) x
// 2 (k) warps of 32 x 32; K runs over pixels in tiles of 32 (split over
// blockIdx.z, FP32 atomics into dW whose rows are ldw long).  Both tiles are
// held pixel-major in shared memory and read with transposing ldmatrix.
constexpr int DWM = 64, DWN = 64, DWK = 32, DWPAD = 8;
__global__ void __launch_bounds__(128) k_gemm_dw(const bf16 *dZ, const bf16 *X, float *dW, int P,
                                                 int H, int W, int C, int taps, int Cout, int ldw,
                                                 int pchunk) {
  __shared__ __align__(16) bf16 Zs[GSTAGES][DWK][DWM + DWPAD];
  __shared__ __align__(16) bf16 Xs[GSTAGES][DWK][DWN + DWPAD];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp & 1, wn = warp >> 1;
  const int m0 = blockIdx.x * DWM, n0 = blockIdx.y * DWN;
  const int pbeg = blockIdx.z * pchunk, pend = min(P, pbeg + pchunk);
  const int nk = (pend - pbeg + DWK - 1) / DWK;
  const int KC = taps * C;
  // per thread: two (pixel row, 8-column group) chunks of each tile
  int zr[2], zc[2], xdy[2], xdx[2], xcol[2];
  bool zok[2], xok[2];
#pragma unroll
  for (int it = 0; it < 2; it++) {
    const int ch = tid + it * 128;
    zr[it] = ch >> 3;
    zc[it] = (ch & 7) * 8;
    zok[it] = m0 + zc[it] < Cout;
    const int k = n0 + zc[it];
    xok[it] = k < KC;
    const int r = xok[it] ? k / C : 0;
    xdy[it] = taps == 9 ? r / 3 - 1 : 0;
    xdx[it] = taps == 9 ? r % 3 - 1 : 0;
    xcol[it] = k - r * C;
  }
  auto load = [&](int stage, int p0) {
#pragma unroll
    for (int it = 0; it < 2; it++) {
      const int p = p0 + zr[it];
      const bool pin = p < pend;
      const bool zk = pin && zok[it];
      cp_async16(&Zs[stage][zr[it]][zc[it]], zk ? dZ + (size_t)p * Cout + m0 + zc[it] : dZ, zk);
      bool xk = pin && xok[it];
      const bf16 *src = X;
      if (xk) {
        const int x = p % W, y = (p / W) % H;
        const int yy = y + xdy[it], xx = x + xdx[it];
        xk = yy >= 0 && yy < H && xx >= 0 && xx < W;
        if (xk) src = X + (size_t)(p + xdy[it] * W + xdx[it]) * C + xcol[it];
      }
      cp_async16(&Xs[stage][zr[it]][zc[it]], src, xk);
    }
  };
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int r = 0; r < 4; r++) acc[i][j][r] = 0.f;
#pragma unroll
  for (int st = 0; st < GSTAGES - 1; st++) {
    if (st < nk) load(st, pbeg + st * DWK);
    cp_async_commit();
  }
  const int l8 = lane & 7, lb3 = (lane >> 3) & 1, lb4 = (lane >> 4) & 1;
  for (int kt = 0; kt < nk; kt++) {
    cp_async_wait<GSTAGES - 2>();
    __syncthreads();
    if (kt + GSTAGES - 1 < nk) load((kt + GSTAGES - 1) % GSTAGES, pbeg + (kt + GSTAGES - 1) * DWK);
    cp_async_commit();
    const int stg = kt % GSTAGES;
#pragma unroll
    for (int kk = 0; kk < DWK; kk += 16) {
      uint32_t af[2][4], bfr[4][2];
#pragma unroll
      for (int i = 0; i < 2; i++)  // A[m][k] = Zs[k][m]: matrices (m, k), (m+8, k), (m, k+8), (m+8, k+8)
        ldsm_x4_t(af[i], &Zs[stg][kk + l8 + lb4 * 8][wm * 32 + i * 16 + lb3 * 8]);
#pragma unroll
      for (int j = 0; j < 4; j += 2) {  // B[k][n] = Xs[k][n]: (k, n), (k+8, n), (k, n+8), (k+8, n+8)
        uint32_t r[4];
        ldsm_x4_t(r, &Xs[stg][kk + l8 + lb3 * 8][wn * 32 + j * 8 + lb4 * 8]);
        bfr[j][0] = r[0];
        bfr[j][1] = r[1];
        bfr[j + 1][0] = r[2];
        bfr[j + 1][1] = r[3];
      }
#pragma unroll
      for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) mma_bf16(acc[i][j], af[i], bfr[j]);
    }
  }
  cp_async_wait<0>();
  const int gq = lane >> 2, tq = lane & 3;
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int row = m0 + wm * 32 + i * 16 + gq + h * 8;
        if (row >= Cout) continue;
#pragma unroll
        for (int e = 0; e < 2; e++) {
          const int col = n0 + wn * 32 + j * 8 + 2 * tq + e;
          if (col < KC) atomicAdd(dW + (size_t)row * ldw + col, acc[i][j][h * 2 + e]);
        }
      }
}

// dZ = dY * (Y > 0) for ReLU layers (in place, when RELU) and db[c] += sum
// over pixels of dZ[p][c]; C a multiple of 8, each thread 8 channels of a pixel.
template <bool RELU>
__global__ void __launch_bounds__(256) k_relu_bias_back(bf16 *dY, const bf16 *Y, float *db, size_t P, int C) {
  __shared__ float sh[256][9];
  const int G = C / 8;              // channel groups of a pixel
  const int per = blockDim.x / G;   // pixels per block pass
  const int grp = threadIdx.x % G, pl = threadIdx.x / G;
  float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (pl < per) {
    for (size_t p = (size_t)blockIdx.x * per + pl; p < P; p += (size_t)gridDim.x * per) {
      uint4 d = *(const uint4 *)(dY + p * C + grp * 8);
      bf16 *dv = (bf16 *)&d;
      if (RELU) {
        const uint4 y = *(const uint4 *)(Y + p * C + grp * 8);
        const bf16 *yv = (const bf16 *)&y;
#pragma unroll
        for (int e = 0; e < 8; e++)
          if (!(__bfloat162float(yv[e]) > 0.f)) dv[e] = __float2bfloat16_rn(0.f);
        *(uint4 *)(dY + p * C + grp * 8) = d;
      }
#pragma unroll
      for (int e = 0; e < 8; e++) acc[e] += __bfloat162float(dv[e]);
    }
  }
#pragma unroll
  for (int e = 0; e < 8; e++) sh[threadIdx.x][e] = acc[e];
  __syncthreads();
  if (threadIdx.x < C) {
    const int gi = threadIdx.x / 8, e = threadIdx.x % 8;
    float s = 0.f;
    for (int t = gi; t < per * G; t += G) s += sh[t][e];
    atomicAdd(db + threadIdx.x, s);
  }
}

// im2col of a taps = 9 (3x3, pad 1) or taps = 1 convolution:
// A[p][r*C + c] = X[p + offset r][c], zero outside the image and in the K
// padding (k >= taps*C).  X is [B][H][W][C], A is [B*H*W][Kp].
__global__ void k_im2col(const bf16 *X, bf16 *A, int B, int H, int W, int C, int taps, int Kp) {
  const size_t total = (size_t)B * H * W * Kp;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(i % Kp);
    const size_t p = i / Kp;
    bf16 v = __float2bfloat16_rn(0.f);
    if (k < taps * C) {
      const int r = k / C, c = k - r * C;
      if (taps == 1) {
        v = X[p * C + c];
      } else {
        const int x = (int)(p % W), y = (int)((p / W) % H), b = (int)(p / ((size_t)W * H));
        const int xx = x + r % 3 - 1, yy = y + r / 3 - 1;
        if (xx >= 0 && xx < W && yy >= 0 && yy < H) v = X[(((size_t)b * H + yy) * W + xx) * C + c];
      }
    }
    A[i] = v;
  }
}

// Transpose of a [R][Cc] BF16 matrix into [Cc][ldo] (ldo >= R; columns R..ldo-1 zero).
__global__ void k_transpose(const bf16 *in, bf16 *out, int R, int Cc, int ldo) {
  __shared__ bf16 t[32][33];
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  for (int i = threadIdx.y; i < 32; i += 8) {
    const int r = r0 + i, c = c0 + threadIdx.x;
    t[i][threadIdx.x] = (r < R && c < Cc) ? in[(size_t)r * Cc + c] : __float2bfloat16_rn(0.f);
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += 8) {
    const int c = c0 + i, r = r0 + threadIdx.x;
    if (c < Cc && r < ldo) out[(size_t)c * ldo + r] = t[threadIdx.x][i];
  }
}

__device__ __forceinline__ float bf(bf16 v) { return __bfloat162float(v); }

// dZ = dY * (Y > 0) for ReLU layers (in place on dY).
__global__ void k_relu_back(bf16 *dY, const bf16 *Y, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    if (!(bf(Y[i]) > 0.f)) dY[i] = __float2bfloat16_rn(0.f);
}

// db[c] += sum over pixels of dZ[p][c] for C <= 8 channels (the output
// layer): per-thread sums over a pixel stride, then a warp reduction.
// Sum of v over the block's threads (blocks of up to 32 warps), in thread 0;
// a block-level sum first, so that a kernel adds one value per block into
// global memory instead of one per warp (the adds to one address serialise).
template <class T>
__device__ __forceinline__ T block_sum(T v) {
  __shared__ T part[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();  // part[] may still be read by a previous call
  if ((threadIdx.x & 31) == 0) part[w] = v;
  __syncthreads();
  T s = 0;
  if (threadIdx.x == 0)
    for (int i = 0; i < nw; i++) s += part[i];
  return s;
}

__global__ void k_bias_grad(const bf16 *dZ, float *db, size_t P, int C) {
  float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < P; p += (size_t)gridDim.x * blockDim.x)
#pragma unroll
    for (int c = 0; c < 8; c++)
      if (c < C) acc[c] += bf(dZ[p * C + c]);
#pragma unroll
  for (int c = 0; c < 8; c++) {
    if (c >= C) break;  // C is uniform
    const float v = block_sum(acc[c]);
    if (threadIdx.x == 0) atomicAdd(db + c, v);
  }
}

// The channel-layout kernels below move 8 channels (16 bytes) per thread when
// every channel count and offset is a multiple of 8 (all feature maps of the
// network), with 32-bit index arithmetic; the sums and roundings are those of
// one channel at a time.  The scalar loops remain for other shapes.
__device__ __forceinline__ void ld8(const bf16 *p, float v[8]) {
  const uint4 u = *(const uint4 *)p;
  const __nv_bfloat162 *h = (const __nv_bfloat162 *)&u;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const float2 f = __bfloat1622float2(h[i]);
    v[2 * i] = f.x;
    v[2 * i + 1] = f.y;
  }
}
__device__ __forceinline__ void st8(bf16 *p, const float v[8]) {
  uint4 u;
  __nv_bfloat162 *h = (__nv_bfloat162 *)&u;
#pragma unroll
  for (int i = 0; i < 4; i++) h[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
  *(uint4 *)p = u;
}
__host__ __device__ __forceinline__ bool vec8(int C, int Ctot, int coff, const void *a,
                                              const void *b) {
  return (C % 8) == 0 && (Ctot % 8) == 0 && (coff % 8) == 0 && ((uintptr_t)a & 15) == 0 &&
         ((uintptr_t)b & 15) == 0;
}

// 2x2 average pool of X [B][H][W][C] into Y [B][H/2][W/2][C].
__global__ void k_pool(const bf16 *X, bf16 *Y, int B, int H, int W, int C) {
  if (vec8(C, C, 0, X, Y) && (size_t)B * H * W * C < (1u << 31)) {
    const int C8 = C / 8, W2 = W / 2, H2 = H / 2;
    const int total = B * H2 * W2 * C8;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
      const int c = (i % C8) * 8, q = i / C8;
      const int x = q % W2, y = (q / W2) % H2, b = q / (W2 * H2);
      const size_t base = (((size_t)b * H + 2 * y) * W + 2 * x) * C + c;
      float a[8], e[8], f[8], g[8], o[8];
      ld8(X + base, a);
      ld8(X + base + C, e);
      ld8(X + base + (size_t)W * C, f);
      ld8(X + base + (size_t)W * C + C, g);
#pragma unroll
      for (int k = 0; k < 8; k++) o[k] = 0.25f * (a[k] + e[k] + f[k] + g[k]);
      st8(Y + (size_t)q * C + c, o);
    }
    return;
  }
  const size_t total = (size_t)B * (H / 2) * (W / 2) * C;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    size_t q = i / C;
    const int x = (int)(q % (W / 2)), y = (int)((q / (W / 2)) % (H / 2)), b = (int)(q / ((size_t)(W / 2) * (H / 2)));
    const size_t base = (((size_t)b * H + 2 * y) * W + 2 * x) * C + c;
    const float s = bf(X[base]) + bf(X[base + C]) + bf(X[base + (size_t)W * C]) + bf(X[base + (size_t)W * C + C]);
    Y[i] = __float2bfloat16_rn(0.25f * s);
  }
}
// Gradient of the pool, written into channels [coff, coff+C) of a [.., Ctot] tensor (adds when acc).
__global__ void k_pool_back(const bf16 *dY, bf16 *dX, int B, int H, int W, int C, int Ctot, int coff, int accum) {
  if (vec8(C, Ctot, coff, dY, dX) && (size_t)B * H * W * Ctot < (1u << 31)) {
    const int C8 = C / 8;
    const int total = B * H * W * C8;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
      const int c = (i % C8) * 8, q = i / C8;
      const int x = q % W, y = (q / W) % H, b = q / (W * H);
      float g[8], o[8];
      ld8(dY + (((size_t)b * (H / 2) + y / 2) * (W / 2) + x / 2) * C + c, g);
      bf16 *po = dX + (size_t)q * Ctot + coff + c;
      if (accum) ld8(po, o);
#pragma unroll
      for (int k = 0; k < 8; k++) o[k] = accum ? o[k] + 0.25f * g[k] : 0.25f * g[k];
      st8(po, o);
    }
    return;
  }
  const size_t total = (size_t)B * H * W * C;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    size_t q = i / C;
    const int x = (int)(q % W), y = (int)((q / W) % H), b = (int)(q / ((size_t)W * H));
    const float g = 0.25f * bf(dY[(((size_t)b * (H / 2) + y / 2) * (W / 2) + x / 2) * C + c]);
    bf16 *o = dX + q * Ctot + coff + c;
    *o = __float2bfloat16_rn(accum ? bf(*o) + g : g);
  }
}

// Nearest 2x upsample of X [B][h][w][C] into channels [0, C) of Y [B][2h][2w][Ctot].
__global__ void k_upsample(const bf16 *X, bf16 *Y, int B, int h, int w, int C, int Ctot) {
  if (vec8(C, Ctot, 0, X, Y) && (size_t)B * 4 * h * w * Ctot < (1u << 31)) {
    const int C8 = C / 8, W2 = 2 * w, H2 = 2 * h;
    const int total = B * H2 * W2 * C8;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
      const int c = (i % C8) * 8, q = i / C8;
      const int x = q % W2, y = (q / W2) % H2, b = q / (W2 * H2);
      *(uint4 *)(Y + (size_t)q * Ctot + c) =
          *(const uint4 *)(X + (((size_t)b * h + y / 2) * w + x / 2) * C + c);
    }
    return;
  }
  const size_t total = (size_t)B * 2 * h * 2 * w * C;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    size_t q = i / C;
    const int x = (int)(q % (2 * w)), y = (int)((q / (2 * w)) % (2 * h)), b = (int)(q / ((size_t)4 * w * h));
    Y[q * Ctot + c] = X[(((size_t)b * h + y / 2) * w + x / 2) * C + c];
  }
}
// Gradient of the upsample: dX[b][y][x][c] = sum of the 4 children in channels [0, C) of dY.
__global__ void k_upsample_back(const bf16 *dY, bf16 *dX, int B, int h, int w, int C, int Ctot) {
  if (vec8(C, Ctot, 0, dY, dX) && (size_t)B * 4 * h * w * Ctot < (1u << 31)) {
    const int C8 = C / 8;
    const int total = B * h * w * C8;
    const size_t W2 = 2 * w;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
      const int c = (i % C8) * 8, q = i / C8;
      const int x = q % w, y = (q / w) % h, b = q / (w * h);
      const size_t base = (((size_t)b * 2 * h + 2 * y) * W2 + 2 * x) * Ctot + c;
      float a[8], e[8], f[8], g[8], o[8];
      ld8(dY + base, a);
      ld8(dY + base + Ctot, e);
      ld8(dY + base + W2 * Ctot, f);
      ld8(dY + base + W2 * Ctot + Ctot, g);
#pragma unroll
      for (int k = 0; k < 8; k++) o[k] = a[k] + e[k] + f[k] + g[k];
      st8(dX + (size_t)q * C + c, o);
    }
    return;
  }
  const size_t total = (size_t)B * h * w * C;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    size_t q = i / C;
    const int x = (int)(q % w), y = (int)((q / w) % h), b = (int)(q / ((size_t)w * h));
    const size_t W2 = 2 * w;
    const size_t base = (((size_t)b * 2 * h + 2 * y) * W2 + 2 * x) * Ctot + c;
    const float s = bf(dY[base]) + bf(dY[base + Ctot]) + bf(dY[base + W2 * Ctot]) + bf(dY[base + W2 * Ctot + Ctot]);
    dX[i] = __float2bfloat16_rn(s);
  }
}

// Copy X [P][C] into channels [coff, coff+C) of Y [P][Ctot] (and the reverse).
__global__ void k_copy_ch(const bf16 *X, bf16 *Y, size_t P, int C, int Ctot, int coff) {
  if (vec8(C, Ctot, coff, X, Y) && P * Ctot < (1u << 31)) {
    const int C8 = C / 8, total = (int)P * C8;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
      const int c = (i % C8) * 8, q = i / C8;
      *(uint4 *)(Y + (size_t)q * Ctot + coff + c) = *(const uint4 *)(X + (size_t)q * C + c);
    }
    return;
  }
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < P * C; i += (size_t)gridDim.x * blockDim.x)
    Y[(i / C) * Ctot + coff + i % C] = X[i];
}
// dX[p][c] += dY[p][coff + c] (gradient of a skip tensor used in a concat).
__global__ void k_add_ch(const bf16 *dY, bf16 *dX, size_t P, int C, int Ctot, int coff) {
  if (vec8(C, Ctot, coff, dY, dX) && P * Ctot < (1u << 31)) {
    const int C8 = C / 8, total = (int)P * C8;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
      const int c = (i % C8) * 8, q = i / C8;
      float a[8], d[8];
      ld8(dX + (size_t)q * C + c, a);
      ld8(dY + (size_t)q * Ctot + coff + c, d);
#pragma unroll
      for (int k = 0; k < 8; k++) a[k] = a[k] + d[k];
      st8(dX + (size_t)q * C + c, a);
    }
    return;
  }
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < P * C; i += (size_t)gridDim.x * blockDim.x)
    dX[i] = __float2bfloat16_rn(bf(dX[i]) + bf(dY[(i / C) * Ctot + coff + i % C]));
}

__global__ void k_f32_to_bf16(const float *x, bf16 *y, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] = __float2bfloat16_rn(x[i]);
}
__global__ void k_bf16_to_f32(const bf16 *x, float *y, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] = __bfloat162float(x[i]);
}

// Sum of the loss mask (FP64, one atomic per warp).
__global__ void k_mask_sum(const float *mask, size_t P, double *out) {
  double s = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < P; i += (size_t)gridDim.x * blockDim.x)
    s += mask[i];
  s = block_sum(s);
  if (threadIdx.x == 0) atomicAdd(out, s);
}

// Masked mean-squared error: loss = sum m (y - t)^2 / (sum m * C); dY in BF16.
// msum = sum of the mask (k_mask_sum).
// (P * C < 2^31: the host checks; 32-bit indices, the division by C per
// element being the costly part in 64 bits)
__global__ void k_mse(const bf16 *Y, const float *T, const float *mask, bf16 *dY, size_t P, int C,
                      const double *msum, double *loss) {
  const double inv_count = *msum > 0 ? 1.0 / (*msum * C) : 0.0;
  const float g2 = (float)(2.0 * inv_count);
  const unsigned n = (unsigned)(P * C), uc = (unsigned)C;
  double s = 0.0;
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float m = mask[i / uc];
    const float d = bf(Y[i]) - T[i];
    s += (double)m * d * d;
    dY[i] = __float2bfloat16_rn(g2 * m * d);
  }
  s = block_sum(s);
  if (threadIdx.x == 0) atomicAdd(loss, s * inv_count);
}

// Block-mean term of the loss: the masked means of output and target over
// s x s blocks (per sample and channel) are compared as well, so that errors
// of the large scales weigh more than their share of single cells.
// Pass 1, one thread per (block, channel): D = mean_m(y) - mean_m(t), the
// block's mask weight, and the count of blocks with any weight (channel 0).
__global__ void k_coarse_stats(const bf16 *Y, const float *T, const float *mask, int B, int H, int W,
                               int C, int s, float *D, float *wsum, double *nblk) {
  const int nbx = W / s, nby = H / s, nb = B * nby * nbx;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nb * C; i += gridDim.x * blockDim.x) {
    const int c = i % C, blk = i / C;
    const int bx = blk % nbx, by = (blk / nbx) % nby, b = blk / (nbx * nby);
    float sy = 0.f, st = 0.f, sw = 0.f;
    for (int yy = 0; yy < s; yy++)
      for (int xx = 0; xx < s; xx++) {
        const size_t p = ((size_t)b * H + by * s + yy) * W + bx * s + xx;
        const float m = mask[p];
        sy += m * bf(Y[p * C + c]);
        st += m * T[p * C + c];
        sw += m;
      }
    D[i] = sw > 0.f ? (sy - st) / sw : 0.f;
    if (c == 0) {
      wsum[blk] = sw;
      if (sw > 0.f) atomicAdd(nblk, 1.0);
    }
  }
}
// Pass 2: loss += lambda * sum D^2 / (nblk * C) over blocks with weight, and
// dY[p][c] += lambda * 2 D m_p / (w nblk C) (dY in BF16).
__global__ void k_coarse_apply(bf16 *dY, const float *mask, int B, int H, int W, int C, int s,
                               const float *D, const float *wsum, const double *nblk, float lambda,
                               double *loss) {
  const double inv = *nblk > 0 ? 1.0 / (*nblk * C) : 0.0;
  const int nbx = W / s, nby = H / s;
  const size_t P = (size_t)B * H * W, nbc = (size_t)B * nby * nbx * C;
  double acc = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < P * C; i += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    const size_t p = i / C;
    const int x = (int)(p % W), y = (int)((p / W) % H), b = (int)(p / ((size_t)W * H));
    const int blk = (b * nby + y / s) * nbx + x / s;
    const float w = wsum[blk];
    if (w > 0.f) {
      const float g = lambda * 2.f * D[(size_t)blk * C + c] * mask[p] / w * (float)inv;
      dY[i] = __float2bfloat16_rn(bf(dY[i]) + g);
    }
    if (i < nbc && wsum[i / C] > 0.f) acc += (double)D[i] * D[i];
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, lambda * acc * inv);
}

// Adam on FP32 master weights, with decoupled weight decay wd (AdamW).
__global__ void k_adam(float *w, const float *g, float *m, float *v, size_t n, float lr, float b1,
                       float b2, float eps, float c1, float c2, float wd) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * ((mi / c1) / (sqrtf(vi / c2) + eps) + wd * w[i]);
  }
}

// BF16 copies of one layer's FP32 master weights W[co][Kp] (k = r*Cin + ci,
// zero beyond taps*Cin): Wt = W for the forward product, and the flipped,
// transposed Wd[ci][k'] (k' = r*Cout + co, r -> taps-1-r) for the input gradient.
// The BF16 weights of every layer in one launch: blockIdx.y is the layer.
struct WeightJob {
  const float *W;
  bf16 *Wt, *Wd;
  int Cout, Cin, taps, Kp, Kpd;
};
__global__ void k_weights(const WeightJob *__restrict__ jobs) {
  const WeightJob j = jobs[blockIdx.y];
  const float *W = j.W;
  bf16 *Wt = j.Wt, *Wd = j.Wd;
  const int Cout = j.Cout, Cin = j.Cin, taps = j.taps, Kp = j.Kp, Kpd = j.Kpd;
  const int n = Cout * Kp;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    Wt[i] = __float2bfloat16_rn(W[i]);
  const int nd = Cin * Kpd;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nd; i += gridDim.x * blockDim.x) {
    const int ci = i / Kpd, k = i % Kpd;
    float v = 0.f;
    if (k < taps * Cout) {
      const int r = k / Cout, co = k % Cout;
      v = W[(size_t)co * Kp + (taps - 1 - r) * Cin + ci];
    }
    Wd[i] = __float2bfloat16_rn(v);
  }
}

}  // namespace

// ------------------------------------------------------------------- network

namespace {

int rup(int x, int a) { return (x + a - 1) / a * a; }
int grid_for(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 152 * 32); }
// Reductions into one address: two blocks per SM, so that the per-block adds
// (which serialise on that address) stay few.
int grid_sum(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 152 * 2); }

struct Conv {
  int cin, cout, taps, Kp, Kpd;
  bool relu;
  size_t woff, boff;  // master weights W[cout][Kp] and bias b[cout] in the parameter vector
  bf16 *Wt, *Wd;
};

struct Act {
  int h = 0, w = 0, c = 0;
  bf16 *x = nullptr, *dx = nullptr;
};

// activation ids
enum {
  A_IN, A_E0A, A_E0, A_P0, A_E1A, A_E1, A_P1, A_E2A, A_E2, A_P2, A_E3A, A_E3, A_C2, A_D2A, A_D2,
  A_C1, A_D1A, A_D1, A_C0, A_D0A, A_D0, A_OUT, A_COUNT
};

}  // namespace

struct lbm_sg {
  lbm_sg_config cfg{};
  std::vector<Conv> conv;
  Act act[A_COUNT];
  size_t nparam = 0;
  float *w = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
  bf16 *col = nullptr, *colT = nullptr, *dzT = nullptr;
  float *tgt = nullptr, *msk = nullptr, *xin = nullptr, *yout = nullptr;
  float *coarse_d = nullptr, *coarse_w = nullptr;  // block-mean loss term scratch
  double *loss = nullptr;
  int64_t step = 0;
  cudaStream_t stream = nullptr;
  std::vector<void *> allocs;
  float *ds_x = nullptr, *ds_y = nullptr, *ds_m = nullptr;
  int ds_count = 0;
  int *d_err = nullptr;  // set by a tcgen05 kernel whose bounded wait gave up
  void *d_wjobs = nullptr;  // k_weights' per-layer jobs (one launch refreshes every layer)
};

namespace {

template <class T>
lbm_status salloc(lbm_sg *s, T **p, size_t count) {
  cudaError_t e = cudaMalloc((void **)p, std::max<size_t>(count * sizeof(T), 16));
  if (e != cudaSuccess)
    return fail(LBM_NOMEM, std::string("surrogate cudaMalloc: ") + cudaGetErrorString(e));
  s->allocs.push_back((void *)*p);
  return LBM_OK;
}

void sfree(lbm_sg *s) {
  for (void *p : s->allocs) cudaFree(p);
  s->allocs.clear();
  if (s->stream) cudaStreamDestroy(s->stream);
  s->stream = nullptr;
}

template <int EPI, bool GATHER>
const void *gemm_fn(int bn) {
  return bn == 32 ? (const void *)k_gemm<EPI, GATHER, 32> : (const void *)k_gemm<EPI, GATHER, 64>;
}

// After a synchronisation: a tcgen05 kernel whose bounded wait gave up set
// the error word; report it (and clear it for the next call).
lbm_status tc_status(lbm_sg *s) {
  int h = 0;
  if (cudaMemcpy(&h, s->d_err, sizeof h, cudaMemcpyDeviceToHost) != cudaSuccess)
    return fail(LBM_CUDA, "surrogate error word read-back");
  if (h != 0) {
    cudaMemset(s->d_err, 0, sizeof(int));
    return fail(LBM_TIMEOUT, "a bounded wait of a tcgen05 product gave up");
  }
  return LBM_OK;
}

// tcgen05 convolution product (lbm_tc.cuh) of one epilogue and tile width.
template <int EPI, int BN>
cudaError_t tc_conv_launch(lbm_sg *s, const bf16 *X, int P, int H, int W, int C, int taps,
                           const bf16 *Bt, int N, int Kp, const float *bias, bf16 *out) {
  using S = sgtc::TcSmem<BN>;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(sgtc::k_tc_conv<EPI, BN>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, S::ALLOC);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  dim3 grid((P + sgtc::TC_BM - 1) / sgtc::TC_BM, (N + BN - 1) / BN);
  sgtc::k_tc_conv<EPI, BN><<<grid, sgtc::TC_THREADS, S::ALLOC, s->stream>>>(
      X, P, H, W, C, taps, Bt, N, Kp, bias, out, s->d_err);
  return cudaGetLastError();
}

// cuTensorMapEncodeTiled from the driver (resolved once; null if absent).
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                   const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                   const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return (EncodeTiledFn) nullptr;
    return (EncodeTiledFn)p;
  }();
  return fn;
}

// The halo-tile tcgen05 convolution (k_tc_conv3h): 3x3, W a multiple of 128,
// C a multiple of 32, N a multiple of BN (N / BN output tiles).  Returns false (nothing launched) when the
// tensor maps cannot be encoded, so the caller takes the gather kernel.
template <int EPI, int BN>
bool tc_conv3h(lbm_sg *s, const bf16 *X, int P, int H, int W, int C, const bf16 *Bt, int N, int Kp,
               const float *bias, bf16 *out, cudaError_t *err) {
  using T = sgtc::TcHalo<BN>;
  EncodeTiledFn enc = encode_tiled();
  if (!enc || ((uintptr_t)X & 15) || ((uintptr_t)Bt & 15)) return false;
  const int imgs = P / (H * W);
  CUtensorMap ma, mb;
  const cuuint64_t da[5] = {8, (cuuint64_t)W, (cuuint64_t)(C / 8), (cuuint64_t)H, (cuuint64_t)imgs};
  const cuuint64_t sa[4] = {(cuuint64_t)C * 2, 16, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2};
  const cuuint32_t ba[5] = {8, 130, 4, 3, 1}, ea[5] = {1, 1, 1, 1, 1};
  const cuuint64_t db[4] = {8, (cuuint64_t)N, (cuuint64_t)(C / 8), 9};
  const cuuint64_t sb[3] = {(cuuint64_t)Kp * 2, 16, (cuuint64_t)C * 2};
  const cuuint32_t bb[4] = {8, (cuuint32_t)BN, 4, 9}, eb[4] = {1, 1, 1, 1};
  if (enc(&ma, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, (void *)X, da, sa, ba, ea,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS ||
      enc(&mb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void *)Bt, db, sb, bb, eb,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  static bool attr = false;
  if (!attr) {
    *err = cudaFuncSetAttribute(sgtc::k_tc_conv3h<EPI, BN>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, T::bytes(2));
    if (*err != cudaSuccess) return true;
    attr = true;
  }
  const int S = C / 32 >= 2 ? 2 : 1;
  dim3 grid((unsigned)(W / sgtc::TC_BM * (N / BN)), (unsigned)H, (unsigned)imgs);
  sgtc::k_tc_conv3h<EPI, BN><<<grid, sgtc::TC_THREADS, T::bytes(S), s->stream>>>(
      ma, mb, H, W, C, N, S, bias, out, s->d_err);
  *err = cudaGetLastError();
  return true;
}

// The same product with several row segments per block (k_tc_conv3m): H a
// multiple of TC_SEGS as well, out 16-byte aligned.  Returns false (nothing
// launched) when the tensor maps cannot be encoded.
template <int EPI, int BN>
bool tc_conv3m(lbm_sg *s, const bf16 *X, int P, int H, int W, int C, const bf16 *Bt, int N, int Kp,
               const float *bias, bf16 *out, cudaError_t *err) {
  using M = sgtc::TcHaloM<BN>;
  EncodeTiledFn enc = encode_tiled();
  if (!enc || ((uintptr_t)X & 15) || ((uintptr_t)Bt & 15) || ((uintptr_t)out & 15)) return false;
  // halo ring depth: the most halo loads in flight per SM (stages used, at
  // most the block's TC_SEGS x nch loads, times resident blocks: shared
  // memory and 2 BN tensor-memory columns per block; fewer stages on a tie),
  // at least two stages (a stage is refilled while the next one is read)
  const int nch = C / 32;
  constexpr int kSmemSM = 233472, kSmemBlock = 232448;  // per SM, per block (bytes)
  int S = 0, best = 0;
  for (int st = 2; st <= sgtc::TC3M_MAX_STAGES; st++) {
    const int bytes = M::bytes(st, nch);
    if (bytes > kSmemBlock) break;
    const int blocks = std::min(kSmemSM / (bytes + 1024), 512 / (2 * BN));
    if (std::min(st, sgtc::TC_SEGS * nch) * blocks > best) {
      best = std::min(st, sgtc::TC_SEGS * nch) * blocks;
      S = st;
    }
  }
  if (S == 0) return false;
  const int imgs = P / (H * W);
  CUtensorMap ma, mb;
  const cuuint64_t da[5] = {8, (cuuint64_t)W, (cuuint64_t)(C / 8), (cuuint64_t)H, (cuuint64_t)imgs};
  const cuuint64_t sa[4] = {(cuuint64_t)C * 2, 16, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2};
  const cuuint32_t ba[5] = {8, 130, 4, 3, 1}, ea[5] = {1, 1, 1, 1, 1};
  const cuuint64_t db[4] = {8, (cuuint64_t)N, (cuuint64_t)(C / 8), 9};
  const cuuint64_t sb[3] = {(cuuint64_t)Kp * 2, 16, (cuuint64_t)C * 2};
  const cuuint32_t bb[4] = {8, (cuuint32_t)BN, 4, 9}, eb[4] = {1, 1, 1, 1};
  if (enc(&ma, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, (void *)X, da, sa, ba, ea,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS ||
      enc(&mb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void *)Bt, db, sb, bb, eb,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  static bool attr = false;
  if (!attr) {
    *err = cudaFuncSetAttribute(sgtc::k_tc_conv3m<EPI, BN>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBlock);
    if (*err != cudaSuccess) return true;
    attr = true;
  }
  dim3 grid((unsigned)(W / sgtc::TC_BM * (N / BN)), (unsigned)(H / sgtc::TC_SEGS), (unsigned)imgs);
  sgtc::k_tc_conv3m<EPI, BN><<<grid, sgtc::TC3M_THREADS, M::bytes(S, nch), s->stream>>>(
      ma, mb, H, W, C, N, S, bias, out, s->d_err);
  *err = cudaGetLastError();
  return true;
}

template <int EPI>
cudaError_t tc_conv(lbm_sg *s, const bf16 *X, int P, int H, int W, int C, int taps,
                    const bf16 *Bt, int N, int Kp, const float *bias, bf16 *out) {
  if (taps == 9 && W % sgtc::TC_BM == 0 && C % 32 == 0 && Kp >= 9 * C && Kp % 8 == 0 &&
      P % (H * W) == 0 && s->cfg.products == 0 && H % sgtc::TC_SEGS == 0) {
    cudaError_t e = cudaSuccess;
    bool done = false;
    if (N % 128 == 0) done = tc_conv3m<EPI, 128>(s, X, P, H, W, C, Bt, N, Kp, bias, out, &e);
    else if (N % 64 == 0) done = tc_conv3m<EPI, 64>(s, X, P, H, W, C, Bt, N, Kp, bias, out, &e);
    else if (N % 32 == 0) done = tc_conv3m<EPI, 32>(s, X, P, H, W, C, Bt, N, Kp, bias, out, &e);
    if (done) return e;
  }
  if (taps == 9 && W % sgtc::TC_BM == 0 && C % 32 == 0 && Kp >= 9 * C && Kp % 8 == 0 &&
      P % (H * W) == 0 && (s->cfg.products == 0 || s->cfg.products == 3)) {
    cudaError_t e = cudaSuccess;
    bool done = false;
    if (N % 128 == 0) done = tc_conv3h<EPI, 128>(s, X, P, H, W, C, Bt, N, Kp, bias, out, &e);
    else if (N % 64 == 0) done = tc_conv3h<EPI, 64>(s, X, P, H, W, C, Bt, N, Kp, bias, out, &e);
    else if (N % 32 == 0) done = tc_conv3h<EPI, 32>(s, X, P, H, W, C, Bt, N, Kp, bias, out, &e);
    if (done) return e;
  }
  if (N <= 32) return tc_conv_launch<EPI, 32>(s, X, P, H, W, C, taps, Bt, N, Kp, bias, out);
  if (N <= 64) return tc_conv_launch<EPI, 64>(s, X, P, H, W, C, taps, Bt, N, Kp, bias, out);
  return tc_conv_launch<EPI, 128>(s, X, P, H, W, C, taps, Bt, N, Kp, bias, out);
}

// The halo-tile tcgen05 weight gradient (k_tc_wgrad3h): 3x3, W a multiple
// of 128, C a multiple of 32, N a multiple of 8; one block per SM in all (the
// row segments split over blocks).  Returns false (nothing launched) when the
// tensor maps cannot be encoded.
bool tc_wgrad3h(lbm_sg *s, const bf16 *dZ, const bf16 *X, int P, int H, int W, int C, int N,
                float *dW, int ldw, cudaError_t *err) {
  using T = sgtc::TcHaloW;
  EncodeTiledFn enc = encode_tiled();
  if (!enc || ((uintptr_t)X & 15) || ((uintptr_t)dZ & 15)) return false;
  const int imgs = P / (H * W);
  CUtensorMap mx, mz;
  const cuuint64_t dx[5] = {8, (cuuint64_t)W, (cuuint64_t)(C / 8), (cuuint64_t)H, (cuuint64_t)imgs};
  const cuuint64_t sx[4] = {(cuuint64_t)C * 2, 16, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2};
  const cuuint32_t bx[5] = {8, 130, 4, 3, 1}, e5[5] = {1, 1, 1, 1, 1};
  const cuuint64_t dz[5] = {8, (cuuint64_t)W, (cuuint64_t)(N / 8), (cuuint64_t)H, (cuuint64_t)imgs};
  const cuuint64_t sz[4] = {(cuuint64_t)N * 2, 16, (cuuint64_t)W * N * 2, (cuuint64_t)H * W * N * 2};
  const cuuint32_t bz[5] = {8, 128, (cuuint32_t)std::min(16, N / 8), 1, 1};
  if (enc(&mx, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, (void *)X, dx, sx, bx, e5,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS ||
      enc(&mz, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, (void *)dZ, dz, sz, bz, e5,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  static bool attr = false;
  if (!attr) {
    *err = cudaFuncSetAttribute(sgtc::k_tc_wgrad3h, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                T::BYTES);
    if (*err != cudaSuccess) return true;
    attr = true;
  }
  const int nseg = imgs * H * (W / sgtc::TC_BM);
  const int bx_ = C / 32, by_ = (N + 127) / 128;
  const int splits = std::max(1, std::min(nseg, (152 + bx_ * by_ - 1) / (bx_ * by_)));
  const int spb = (nseg + splits - 1) / splits;
  dim3 grid((unsigned)bx_, (unsigned)by_, (unsigned)((nseg + spb - 1) / spb));
  sgtc::k_tc_wgrad3h<<<grid, sgtc::TC_THREADS, T::BYTES, s->stream>>>(mx, mz, H, W, C, N, nseg, spb,
                                                                      dW, ldw, s->d_err);
  *err = cudaGetLastError();
  return true;
}

// tcgen05 weight gradient (lbm_tc.cuh), pixels split so that about four
// blocks per SM run in all, at least 256 pixels each.
template <int BN>
cudaError_t tc_wgrad_launch(lbm_sg *s, const bf16 *dZ, const bf16 *X, int P, int H, int W, int C,
                            int taps, int N, float *dW, int ldw) {
  using S = sgtc::TcSmem<BN>;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(sgtc::k_tc_wgrad<BN>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, S::ALLOC);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const int bm = (taps * C + sgtc::TC_BM - 1) / sgtc::TC_BM, bn = (N + BN - 1) / BN;
  const int splits = std::max(1, std::min(P / 256, (152 * 4) / (bm * bn) + 1));
  const int pchunk = rup((P + splits - 1) / splits, sgtc::TC_BK);
  dim3 grid(bm, bn, (P + pchunk - 1) / pchunk);
  sgtc::k_tc_wgrad<BN><<<grid, sgtc::TC_THREADS, S::ALLOC, s->stream>>>(
      dZ, X, P, H, W, C, taps, N, dW, ldw, pchunk, s->d_err);
  return cudaGetLastError();
}

// C = A x Bt^T with A explicit ([M][K]) or, when X is given, the implicit
// im2col of X ([M pixels][H][W][C], K = taps * C).
lbm_status gemm(lbm_sg *s, int epi, const bf16 *A, const bf16 *Bt, int M, int N, int K,
                const float *bias, bf16 *ob, float *of, int splits, const bf16 *X = nullptr,
                int H = 0, int W = 0, int C = 0, int taps = 0) {
  GemmArgs g;
  g.A = A;
  g.X = X;
  g.H = H;
  g.W = W;
  g.C = C;
  g.taps = taps;
  g.Bt = Bt;
  g.M = M;
  g.N = N;
  g.K = K;
  g.kchunk = rup((K + splits - 1) / splits, GBK);
  g.bias = bias;
  g.out_bf16 = ob;
  g.out_f32 = of;
  if (X && s->cfg.products != 1 && splits == 1 && K % 8 == 0 && K <= sgtc::TC_KTAB * 8 &&
      (epi == EPI_BIAS_RELU_BF16 || epi == EPI_BIAS_BF16 || epi == EPI_BF16)) {
    // the implicit-GEMM convolution on tcgen05
    cudaError_t e;
    if (epi == EPI_BIAS_RELU_BF16)
      e = tc_conv<sgtc::TC_BIAS_RELU>(s, X, M, H, W, C, taps, Bt, N, K, bias, ob);
    else if (epi == EPI_BIAS_BF16)
      e = tc_conv<sgtc::TC_BIAS>(s, X, M, H, W, C, taps, Bt, N, K, bias, ob);
    else
      e = tc_conv<sgtc::TC_PLAIN>(s, X, M, H, W, C, taps, Bt, N, K, nullptr, ob);
    if (e != cudaSuccess)
      return fail(LBM_CUDA, std::string("surrogate tcgen05 conv: ") + cudaGetErrorString(e));
    return LBM_OK;
  }
  const int bn = N <= 32 ? 32 : 64;
  dim3 grid((M + GBM - 1) / GBM, (N + bn - 1) / bn, (K + g.kchunk - 1) / g.kchunk);
  void *args[] = {&g};
  const bool ga = X != nullptr;
  const void *fn = nullptr;
  switch (epi) {
    case EPI_BIAS_RELU_BF16:
      fn = ga ? gemm_fn<EPI_BIAS_RELU_BF16, true>(bn) : gemm_fn<EPI_BIAS_RELU_BF16, false>(bn);
      break;
    case EPI_BIAS_BF16:
      fn = ga ? gemm_fn<EPI_BIAS_BF16, true>(bn) : gemm_fn<EPI_BIAS_BF16, false>(bn);
      break;
    case EPI_BF16:
      fn = ga ? gemm_fn<EPI_BF16, true>(bn) : gemm_fn<EPI_BF16, false>(bn);
      break;
    default:
      fn = gemm_fn<EPI_ATOMIC_F32, false>(bn);
      break;
  }
  cudaError_t e = cudaLaunchKernel(fn, grid, dim3(256), args, 0, s->stream);
  if (e != cudaSuccess) return fail(LBM_CUDA, std::string("surrogate gemm: ") + cudaGetErrorString(e));
  return LBM_OK;
}

void refresh_weights(lbm_sg *s) {
  k_weights<<<dim3(64, (unsigned)s->conv.size()), 256, 0, s->stream>>>(
      (const WeightJob *)s->d_wjobs);
}

// The implicit im2col needs every 16-byte chunk inside one tap.
bool gather_ok(int C) { return C % 8 == 0; }

lbm_status conv_fwd(lbm_sg *s, int li, int xi, int yi, int B) {
  const Conv &c = s->conv[li];
  const Act &X = s->act[xi];
  Act &Y = s->act[yi];
  const int M = B * X.h * X.w;
  const int epi = c.relu ? EPI_BIAS_RELU_BF16 : EPI_BIAS_BF16;
  if (gather_ok(X.c))
    return gemm(s, epi, nullptr, c.Wt, M, c.cout, c.Kp, s->w + c.boff, Y.x, nullptr, 1, X.x, X.h,
                X.w, X.c, c.taps);
  const size_t n = (size_t)M * c.Kp;
  k_im2col<<<grid_for(n), 256, 0, s->stream>>>(X.x, s->col, B, X.h, X.w, X.c, c.taps, c.Kp);
  return gemm(s, epi, s->col, c.Wt, M, c.cout, c.Kp, s->w + c.boff, Y.x, nullptr, 1);
}

// Given Y.dx (gradient of the layer output), accumulates the weight and bias
// gradients and, when need_dx, writes the input gradient into X.dx.
lbm_status conv_bwd(lbm_sg *s, int li, int xi, int yi, int B, bool need_dx) {
  const Conv &c = s->conv[li];
  Act &X = s->act[xi];
  Act &Y = s->act[yi];
  const int M = B * X.h * X.w, Mp = rup(M, GBK);
  const size_t ny = (size_t)M * c.cout;
  if (c.cout % 8 == 0) {
    const int G = c.cout / 8, per = 256 / G;
    const int grid = (int)std::min<size_t>(((size_t)M + per - 1) / per, 152 * 8);
    if (c.relu)
      k_relu_bias_back<true><<<grid, 256, 0, s->stream>>>(Y.dx, Y.x, s->g + c.boff, (size_t)M, c.cout);
    else
      k_relu_bias_back<false><<<grid, 256, 0, s->stream>>>(Y.dx, Y.x, s->g + c.boff, (size_t)M, c.cout);
  } else {
    if (c.cout > 8) return fail(LBM_INVALID, "surrogate: output channels must be <= 8 or a multiple of 8");
    if (c.relu) k_relu_back<<<grid_for(ny), 256, 0, s->stream>>>(Y.dx, Y.x, ny);
    k_bias_grad<<<grid_sum((size_t)M), 256, 0, s->stream>>>(Y.dx, s->g + c.boff, (size_t)M, c.cout);
  }
  lbm_status st = LBM_OK;
  bool halo_done = false;
  if ((s->cfg.products == 0 || s->cfg.products == 3) && c.taps == 9 && X.w % sgtc::TC_BM == 0 &&
      X.c % 32 == 0 && c.cout % 8 == 0 && c.Kp >= 9 * X.c && M % (X.h * X.w) == 0) {
    cudaError_t e = cudaSuccess;
    halo_done = tc_wgrad3h(s, Y.dx, X.x, M, X.h, X.w, X.c, c.cout, s->g + c.woff, c.Kp, &e);
    if (halo_done && e != cudaSuccess)
      return fail(LBM_CUDA, std::string("surrogate tcgen05 wgrad: ") + cudaGetErrorString(e));
  }
  if (halo_done) {
  } else if (X.c % 8 == 0 && c.cout % 8 == 0 && s->cfg.products != 1) {
    cudaError_t e;
    if (c.cout <= 32)
      e = tc_wgrad_launch<32>(s, Y.dx, X.x, M, X.h, X.w, X.c, c.taps, c.cout, s->g + c.woff, c.Kp);
    else if (c.cout <= 64)
      e = tc_wgrad_launch<64>(s, Y.dx, X.x, M, X.h, X.w, X.c, c.taps, c.cout, s->g + c.woff, c.Kp);
    else
      e = tc_wgrad_launch<128>(s, Y.dx, X.x, M, X.h, X.w, X.c, c.taps, c.cout, s->g + c.woff, c.Kp);
    if (e != cudaSuccess)
      return fail(LBM_CUDA, std::string("surrogate tcgen05 wgrad: ") + cudaGetErrorString(e));
  } else if (X.c % 8 == 0 && c.cout % 8 == 0) {
    const int bm = (c.cout + DWM - 1) / DWM, bn = (c.Kp + DWN - 1) / DWN;
    const int splits = std::max(1, std::min(M / (DWK * 8), (152 * 6) / (bm * bn) + 1));
    const int pchunk = rup((M + splits - 1) / splits, DWK);
    dim3 grid(bm, bn, (M + pchunk - 1) / pchunk);
    k_gemm_dw<<<grid, 128, 0, s->stream>>>(Y.dx, X.x, s->g + c.woff, M, X.h, X.w, X.c, c.taps,
                                           c.cout, c.Kp, pchunk);
  } else {
    k_im2col<<<grid_for((size_t)M * c.Kp), 256, 0, s->stream>>>(X.x, s->col, B, X.h, X.w, X.c, c.taps, c.Kp);
    k_transpose<<<dim3((c.Kp + 31) / 32, Mp / 32), dim3(32, 8), 0, s->stream>>>(s->col, s->colT, M, c.Kp, Mp);
    k_transpose<<<dim3((c.cout + 31) / 32, Mp / 32), dim3(32, 8), 0, s->stream>>>(Y.dx, s->dzT, M, c.cout, Mp);
    const int splits = std::max(1, std::min(256, Mp / 4096));
    st = gemm(s, EPI_ATOMIC_F32, s->dzT, s->colT, c.cout, c.Kp, Mp, nullptr, nullptr, s->g + c.woff,
              splits);
  }
  if (st != LBM_OK || !need_dx) return st;
  if (gather_ok(c.cout))
    return gemm(s, EPI_BF16, nullptr, c.Wd, M, c.cin, c.Kpd, nullptr, X.dx, nullptr, 1, Y.dx, X.h,
                X.w, c.cout, c.taps);
  k_im2col<<<grid_for((size_t)M * c.Kpd), 256, 0, s->stream>>>(Y.dx, s->col, B, X.h, X.w, c.cout, c.taps, c.Kpd);
  return gemm(s, EPI_BF16, s->col, c.Wd, M, c.cin, c.Kpd, nullptr, X.dx, nullptr, 1);
}

lbm_status forward(lbm_sg *s, int B) {
  lbm_status st;
  const int b = s->cfg.base;
  auto cf = [&](int li, int xi, int yi) { return conv_fwd(s, li, xi, yi, B); };
  auto pool = [&](int xi, int yi) {
    const Act &X = s->act[xi];
    const size_t n = (size_t)B * (X.h / 2) * (X.w / 2) * X.c;
    k_pool<<<grid_for(n), 256, 0, s->stream>>>(X.x, s->act[yi].x, B, X.h, X.w, X.c);
  };
  auto cat = [&](int lowi, int skipi, int yi) {
    const Act &L = s->act[lowi], &K = s->act[skipi];
    Act &Y = s->act[yi];
    const size_t n = (size_t)B * Y.h * Y.w * L.c;
    k_upsample<<<grid_for(n), 256, 0, s->stream>>>(L.x, Y.x, B, L.h, L.w, L.c, Y.c);
    const size_t P = (size_t)B * Y.h * Y.w;
    k_copy_ch<<<grid_for(P * K.c), 256, 0, s->stream>>>(K.x, Y.x, P, K.c, Y.c, L.c);
  };
  (void)b;
  if ((st = cf(0, A_IN, A_E0A)) || (st = cf(1, A_E0A, A_E0))) return st;
  pool(A_E0, A_P0);
  if ((st = cf(2, A_P0, A_E1A)) || (st = cf(3, A_E1A, A_E1))) return st;
  pool(A_E1, A_P1);
  if ((st = cf(4, A_P1, A_E2A)) || (st = cf(5, A_E2A, A_E2))) return st;
  pool(A_E2, A_P2);
  if ((st = cf(6, A_P2, A_E3A)) || (st = cf(7, A_E3A, A_E3))) return st;
  cat(A_E3, A_E2, A_C2);
  if ((st = cf(8, A_C2, A_D2A)) || (st = cf(9, A_D2A, A_D2))) return st;
  cat(A_D2, A_E1, A_C1);
  if ((st = cf(10, A_C1, A_D1A)) || (st = cf(11, A_D1A, A_D1))) return st;
  cat(A_D1, A_E0, A_C0);
  if ((st = cf(12, A_C0, A_D0A)) || (st = cf(13, A_D0A, A_D0))) return st;
  return cf(14, A_D0, A_OUT);
}

lbm_status backward(lbm_sg *s, int B) {
  lbm_status st;
  auto cb = [&](int li, int xi, int yi, bool need) { return conv_bwd(s, li, xi, yi, B, need); };
  // concat split: low part -> upsample gradient into the low tensor (write),
  // skip part -> skip tensor gradient (write)
  auto uncat = [&](int lowi, int skipi, int yi) {
    const Act &L = s->act[lowi], &K = s->act[skipi], &Y = s->act[yi];
    const size_t nl = (size_t)B * L.h * L.w * L.c;
    k_upsample_back<<<grid_for(nl), 256, 0, s->stream>>>(Y.dx, L.dx, B, L.h, L.w, L.c, Y.c);
    const size_t P = (size_t)B * Y.h * Y.w;
    cudaMemsetAsync(K.dx, 0, P * K.c * sizeof(bf16), s->stream);
    k_add_ch<<<grid_for(P * K.c), 256, 0, s->stream>>>(Y.dx, K.dx, P, K.c, Y.c, L.c);
  };
  auto unpool = [&](int xi, int yi) {  // adds the pool gradient into X.dx
    const Act &X = s->act[xi];
    const size_t n = (size_t)B * X.h * X.w * X.c;
    k_pool_back<<<grid_for(n), 256, 0, s->stream>>>(s->act[yi].dx, s->act[xi].dx, B, X.h, X.w, X.c, X.c, 0, 1);
  };
  if ((st = cb(14, A_D0, A_OUT, true)) || (st = cb(13, A_D0A, A_D0, true)) ||
      (st = cb(12, A_C0, A_D0A, true)))
    return st;
  uncat(A_D1, A_E0, A_C0);
  if ((st = cb(11, A_D1A, A_D1, true)) || (st = cb(10, A_C1, A_D1A, true))) return st;
  uncat(A_D2, A_E1, A_C1);
  if ((st = cb(9, A_D2A, A_D2, true)) || (st = cb(8, A_C2, A_D2A, true))) return st;
  uncat(A_E3, A_E2, A_C2);
  if ((st = cb(7, A_E3A, A_E3, true)) || (st = cb(6, A_P2, A_E3A, true))) return st;
  unpool(A_E2, A_P2);
  if ((st = cb(5, A_E2A, A_E2, true)) || (st = cb(4, A_P1, A_E2A, true))) return st;
  unpool(A_E1, A_P1);
  if ((st = cb(3, A_E1A, A_E1, true)) || (st = cb(2, A_P0, A_E1A, true))) return st;
  unpool(A_E0, A_P0);
  if ((st = cb(1, A_E0A, A_E0, true)) || (st = cb(0, A_IN, A_E0A, false))) return st;
  return LBM_OK;
}

// Loss and gradients of one batch whose FP32 inputs are at s->xin, targets at
// s->tgt and masks at s->msk (device).
lbm_status loss_grads(lbm_sg *s, int B, double *loss_out) {
  const lbm_sg_config &c = s->cfg;
  const size_t P = (size_t)B * c.height * c.width;
  k_f32_to_bf16<<<grid_for(P * c.in_channels), 256, 0, s->stream>>>(s->xin, s->act[A_IN].x, P * c.in_channels);
  lbm_status st = forward(s, B);
  if (st != LBM_OK) return st;
  cudaMemsetAsync(s->g, 0, s->nparam * sizeof(float), s->stream);
  cudaMemsetAsync(s->loss, 0, 3 * sizeof(double), s->stream);  // loss, mask sum, block count
  if (P * c.out_channels >= (1ull << 31))
    return fail(LBM_INVALID, "surrogate: batch x height x width x outputs must stay below 2^31");
  k_mask_sum<<<grid_sum(P), 256, 0, s->stream>>>(s->msk, P, s->loss + 1);
  k_mse<<<grid_sum(P * c.out_channels), 256, 0, s->stream>>>(s->act[A_OUT].x, s->tgt, s->msk, s->act[A_OUT].dx, P,
                                                           c.out_channels, s->loss + 1, s->loss);
  if (c.coarse_weight > 0.f) {
    const int sb = c.coarse_block, nbc = B * (c.height / sb) * (c.width / sb) * c.out_channels;
    k_coarse_stats<<<grid_for((size_t)nbc), 256, 0, s->stream>>>(
        s->act[A_OUT].x, s->tgt, s->msk, B, c.height, c.width, c.out_channels, sb, s->coarse_d,
        s->coarse_w, s->loss + 2);
    k_coarse_apply<<<grid_for(P * c.out_channels), 256, 0, s->stream>>>(
        s->act[A_OUT].dx, s->msk, B, c.height, c.width, c.out_channels, sb, s->coarse_d,
        s->coarse_w, s->loss + 2, c.coarse_weight, s->loss);
  }
  if ((st = backward(s, B)) != LBM_OK) return st;
  double h = 0;
  cudaMemcpyAsync(&h, s->loss, sizeof h, cudaMemcpyDeviceToHost, s->stream);
  if (cudaStreamSynchronize(s->stream) != cudaSuccess || cudaGetLastError() != cudaSuccess)
    return fail(LBM_CUDA, "surrogate step failed");
  if ((st = tc_status(s)) != LBM_OK) return st;
  if (loss_out) *loss_out = h;
  return LBM_OK;
}

void adam(lbm_sg *s) {
  s->step++;
  const lbm_sg_config &c = s->cfg;
  const float c1 = 1.f - std::pow(c.beta1, (float)s->step), c2 = 1.f - std::pow(c.beta2, (float)s->step);
  k_adam<<<grid_for(s->nparam), 256, 0, s->stream>>>(s->w, s->g, s->m, s->v, s->nparam, c.lr, c.beta1,
                                                     c.beta2, c.eps, c1, c2, c.weight_decay);
  refresh_weights(s);
}

}  // namespace

extern "C" {

lbm_status lbm_sg_create(const lbm_sg_config *cfg, lbm_sg **out) {
  if (!cfg || !out) return fail(LBM_INVALID, "null argument");
  *out = nullptr;
  const int H = cfg->height, W = cfg->width, b = cfg->base;
  if (H < 16 || W < 16 || H % 8 || W % 8 || b < 8 || b % 8 || cfg->in_channels < 1 ||
      cfg->out_channels < 1 || cfg->out_channels > 64 || (cfg->out_channels > 8 && cfg->out_channels % 8) ||
      cfg->max_batch < 1)
    return fail(LBM_INVALID,
                "surrogate: H, W multiples of 8 (>= 16), base multiple of 8, outputs <= 8 or a multiple of 8");
  if (cfg->coarse_weight < 0.f ||
      (cfg->coarse_weight > 0.f && (cfg->coarse_block < 1 || H % cfg->coarse_block || W % cfg->coarse_block)))
    return fail(LBM_INVALID, "surrogate: coarse_block must divide height and width");
  lbm_sg *s = new lbm_sg();
  s->cfg = *cfg;
  auto bail = [&](lbm_status st) {
    sfree(s);
    delete s;
    return st;
  };
  if (cudaSetDevice(cfg->device) != cudaSuccess) return bail(fail(LBM_CUDA, "cudaSetDevice failed"));
  cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  const int ci = cfg->in_channels, co = cfg->out_channels;
  // (cin, cout, taps, relu) in forward order
  const int L[15][4] = {{ci, b, 9, 1},          {b, b, 9, 1},          {b, 2 * b, 9, 1},
                        {2 * b, 2 * b, 9, 1},   {2 * b, 4 * b, 9, 1},  {4 * b, 4 * b, 9, 1},
                        {4 * b, 4 * b, 9, 1},   {4 * b, 4 * b, 9, 1},  {8 * b, 4 * b, 9, 1},
                        {4 * b, 4 * b, 9, 1},   {6 * b, 2 * b, 9, 1},  {2 * b, 2 * b, 9, 1},
                        {3 * b, b, 9, 1},       {b, b, 9, 1},          {b, co, 1, 0}};
  size_t off = 0;
  for (auto &l : L) {
    Conv c;
    c.cin = l[0];
    c.cout = l[1];
    c.taps = l[2];
    c.relu = l[3] != 0;
    c.Kp = rup(c.taps * c.cin, GBK);
    c.Kpd = rup(c.taps * c.cout, GBK);
    c.woff = off;
    off += (size_t)c.cout * c.Kp;
    c.boff = off;
    off += c.cout;
    s->conv.push_back(c);
  }
  s->nparam = off;
  lbm_status st;
  if ((st = salloc(s, &s->w, off)) || (st = salloc(s, &s->g, off)) || (st = salloc(s, &s->m, off)) ||
      (st = salloc(s, &s->v, off)))
    return bail(st);
  for (Conv &c : s->conv)
    if ((st = salloc(s, &c.Wt, (size_t)c.cout * c.Kp)) || (st = salloc(s, &c.Wd, (size_t)c.cin * c.Kpd)))
      return bail(st);
  // He-normal initial weights (padding columns and biases zero)
  std::vector<float> hw(off, 0.f);
  std::mt19937_64 rng(cfg->seed);
  for (const Conv &c : s->conv) {
    std::normal_distribution<float> nd(0.f, std::sqrt(2.f / (c.taps * c.cin)));
    for (int o = 0; o < c.cout; o++)
      for (int k = 0; k < c.taps * c.cin; k++) hw[c.woff + (size_t)o * c.Kp + k] = nd(rng);
  }
  cudaMemcpy(s->w, hw.data(), off * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemset(s->m, 0, off * sizeof(float));
  cudaMemset(s->v, 0, off * sizeof(float));
  // activations
  const int B = cfg->max_batch;
  const int sh[A_COUNT][3] = {
      {0, 0, ci},     {0, 0, b},      {0, 0, b},      {1, 1, b},      {1, 1, 2 * b},
      {1, 1, 2 * b},  {2, 2, 2 * b},  {2, 2, 4 * b},  {2, 2, 4 * b},  {3, 3, 4 * b},
      {3, 3, 4 * b},  {3, 3, 4 * b},  {2, 2, 8 * b},  {2, 2, 4 * b},  {2, 2, 4 * b},
      {1, 1, 6 * b},  {1, 1, 2 * b},  {1, 1, 2 * b},  {0, 0, 3 * b},  {0, 0, b},
      {0, 0, b},      {0, 0, co}};
  size_t max_col = 0, max_colT = 0, max_dz = 0;
  for (int a = 0; a < A_COUNT; a++) {
    Act &A = s->act[a];
    A.h = H >> sh[a][0];
    A.w = W >> sh[a][1];
    A.c = sh[a][2];
    const size_t n = (size_t)B * A.h * A.w * A.c;
    if ((st = salloc(s, &A.x, n)) || (st = salloc(s, &A.dx, n))) return bail(st);
  }
  const int xs[15] = {A_IN, A_E0A, A_P0, A_E1A, A_P1, A_E2A, A_P2, A_E3A, A_C2, A_D2A, A_C1, A_D1A, A_C0, A_D0A, A_D0};
  for (int li = 0; li < 15; li++) {
    const Conv &c = s->conv[li];
    const Act &X = s->act[xs[li]];
    const size_t M = (size_t)B * X.h * X.w, Mp = (size_t)rup((int)M, GBK);
    max_col = std::max(max_col, M * std::max(c.Kp, c.Kpd));
    max_colT = std::max(max_colT, Mp * c.Kp);
    max_dz = std::max(max_dz, Mp * c.cout);
  }
  const size_t P = (size_t)B * H * W;
  if ((st = salloc(s, &s->col, max_col)) || (st = salloc(s, &s->colT, max_colT)) ||
      (st = salloc(s, &s->dzT, max_dz)) || (st = salloc(s, &s->tgt, P * co)) ||
      (st = salloc(s, &s->msk, P)) || (st = salloc(s, &s->xin, P * ci)) ||
      (st = salloc(s, &s->yout, P * co)) || (st = salloc(s, &s->loss, 3)))
    return bail(st);
  if (cfg->products < 0 || cfg->products > 3)
    return bail(fail(LBM_INVALID,
                     "surrogate: products must be 0 (tcgen05), 1 (mma.sync), 2 (tcgen05, gather only) or 3 "
                     "(tcgen05, one row segment per halo-tile block)"));
  if ((st = salloc(s, &s->d_err, 1)) != LBM_OK) return bail(st);
  cudaMemset(s->d_err, 0, sizeof(int));
  {
    std::vector<WeightJob> jobs;
    for (const Conv &c : s->conv)
      jobs.push_back(WeightJob{s->w + c.woff, c.Wt, c.Wd, c.cout, c.cin, c.taps, c.Kp, c.Kpd});
    WeightJob *d = nullptr;
    if ((st = salloc(s, &d, jobs.size())) != LBM_OK) return bail(st);
    if (cudaMemcpy(d, jobs.data(), jobs.size() * sizeof(WeightJob), cudaMemcpyHostToDevice) !=
        cudaSuccess)
      return bail(fail(LBM_CUDA, "surrogate: upload of the weight jobs failed"));
    s->d_wjobs = d;
  }
  if (cfg->coarse_weight > 0.f) {
    const size_t nb = (size_t)B * (H / cfg->coarse_block) * (W / cfg->coarse_block);
    if ((st = salloc(s, &s->coarse_d, nb * co)) || (st = salloc(s, &s->coarse_w, nb))) return bail(st);
  }
  refresh_weights(s);
  if (cudaStreamSynchronize(s->stream) != cudaSuccess || cudaGetLastError() != cudaSuccess)
    return bail(fail(LBM_CUDA, "surrogate set-up failed"));
  *out = s;
  return LBM_OK;
}

void lbm_sg_destroy(lbm_sg *s) {
  if (!s) return;
  sfree(s);
  delete s;
}

lbm_status lbm_sg_num_params(const lbm_sg *s, int64_t *n) {
  if (!s || !n) return fail(LBM_INVALID, "null argument");
  *n = (int64_t)s->nparam;
  return LBM_OK;
}

lbm_status lbm_sg_get_params(lbm_sg *s, float *out) {
  if (!s || !out) return fail(LBM_INVALID, "null argument");
  if (cudaMemcpy(out, s->w, s->nparam * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
    return fail(LBM_CUDA, "surrogate parameter read-back");
  return LBM_OK;
}

lbm_status lbm_sg_set_params(lbm_sg *s, const float *in) {
  if (!s || !in) return fail(LBM_INVALID, "null argument");
  if (cudaMemcpy(s->w, in, s->nparam * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
    return fail(LBM_CUDA, "surrogate parameter upload");
  refresh_weights(s);
  cudaStreamSynchronize(s->stream);
  return LBM_OK;
}

lbm_status lbm_sg_forward(lbm_sg *s, int32_t batch, const float *x, float *y) {
  if (!s || !x || !y || batch < 1 || batch > s->cfg.max_batch) return fail(LBM_INVALID, "bad batch");
  const lbm_sg_config &c = s->cfg;
  const size_t P = (size_t)batch * c.height * c.width;
  cudaMemcpyAsync(s->xin, x, P * c.in_channels * sizeof(float), cudaMemcpyHostToDevice, s->stream);
  k_f32_to_bf16<<<grid_for(P * c.in_channels), 256, 0, s->stream>>>(s->xin, s->act[A_IN].x, P * c.in_channels);
  lbm_status st = forward(s, batch);
  if (st != LBM_OK) return st;
  k_bf16_to_f32<<<grid_for(P * c.out_channels), 256, 0, s->stream>>>(s->act[A_OUT].x, s->yout, P * c.out_channels);
  cudaMemcpyAsync(y, s->yout, P * c.out_channels * sizeof(float), cudaMemcpyDeviceToHost, s->stream);
  if (cudaStreamSynchronize(s->stream) != cudaSuccess) return fail(LBM_CUDA, "surrogate forward failed");
  return tc_status(s);
}

lbm_status lbm_sg_loss_grads(lbm_sg *s, int32_t batch, const float *x, const float *target,
                             const float *mask, double *loss, float *grads) {
  if (!s || !x || !target || batch < 1 || batch > s->cfg.max_batch) return fail(LBM_INVALID, "bad batch");
  const lbm_sg_config &c = s->cfg;
  const size_t P = (size_t)batch * c.height * c.width;
  cudaMemcpyAsync(s->xin, x, P * c.in_channels * sizeof(float), cudaMemcpyHostToDevice, s->stream);
  cudaMemcpyAsync(s->tgt, target, P * c.out_channels * sizeof(float), cudaMemcpyHostToDevice, s->stream);
  if (mask) cudaMemcpyAsync(s->msk, mask, P * sizeof(float), cudaMemcpyHostToDevice, s->stream);
  else {
    std::vector<float> ones(P, 1.f);
    cudaMemcpyAsync(s->msk, ones.data(), P * sizeof(float), cudaMemcpyHostToDevice, s->stream);
    cudaStreamSynchronize(s->stream);
  }
  lbm_status st = loss_grads(s, batch, loss);
  if (st != LBM_OK) return st;
  if (grads && cudaMemcpy(grads, s->g, s->nparam * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
    return fail(LBM_CUDA, "surrogate gradient read-back");
  return LBM_OK;
}

lbm_status lbm_sg_set_dataset(lbm_sg *s, int32_t count, const float *x, const float *y,
                              const float *mask) {
  if (!s || count < 1 || !x || !y || !mask) return fail(LBM_INVALID, "bad dataset");
  const lbm_sg_config &c = s->cfg;
  const size_t P = (size_t)c.height * c.width;
  lbm_status st;
  if (s->ds_x) {
    cudaFree(s->ds_x);
    cudaFree(s->ds_y);
    cudaFree(s->ds_m);
    s->ds_x = s->ds_y = s->ds_m = nullptr;
  }
  if (cudaMalloc((void **)&s->ds_x, count * P * c.in_channels * sizeof(float)) != cudaSuccess ||
      cudaMalloc((void **)&s->ds_y, count * P * c.out_channels * sizeof(float)) != cudaSuccess ||
      cudaMalloc((void **)&s->ds_m, count * P * sizeof(float)) != cudaSuccess)
    return fail(LBM_NOMEM, "surrogate dataset allocation");
  (void)st;
  cudaMemcpy(s->ds_x, x, count * P * c.in_channels * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemcpy(s->ds_y, y, count * P * c.out_channels * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemcpy(s->ds_m, mask, count * P * sizeof(float), cudaMemcpyHostToDevice);
  s->ds_count = count;
  return LBM_OK;
}

lbm_status lbm_sg_train(lbm_sg *s, int32_t batch, const int32_t *order, int32_t n, double *mean_loss) {
  if (!s || !order || n < 1 || batch < 1 || batch > s->cfg.max_batch || !s->ds_x)
    return fail(LBM_INVALID, "bad training call");
  const lbm_sg_config &c = s->cfg;
  const size_t P = (size_t)c.height * c.width;
  double total = 0;
  int steps = 0;
  for (int i0 = 0; i0 + batch <= n; i0 += batch) {
    for (int j = 0; j < batch; j++) {
      const int idx = order[i0 + j];
      if (idx < 0 || idx >= s->ds_count) return fail(LBM_INVALID, "sample index out of range");
      cudaMemcpyAsync(s->xin + j * P * c.in_channels, s->ds_x + (size_t)idx * P * c.in_channels,
                      P * c.in_channels * sizeof(float), cudaMemcpyDeviceToDevice, s->stream);
      cudaMemcpyAsync(s->tgt + j * P * c.out_channels, s->ds_y + (size_t)idx * P * c.out_channels,
                      P * c.out_channels * sizeof(float), cudaMemcpyDeviceToDevice, s->stream);
      cudaMemcpyAsync(s->msk + j * P, s->ds_m + (size_t)idx * P, P * sizeof(float),
                      cudaMemcpyDeviceToDevice, s->stream);
    }
    double l = 0;
    lbm_status st = loss_grads(s, batch, &l);
    if (st != LBM_OK) return st;
    adam(s);
    total += l;
    steps++;
  }
  if (cudaStreamSynchronize(s->stream) != cudaSuccess) return fail(LBM_CUDA, "surrogate training failed");
  if (lbm_status ts = tc_status(s)) return ts;
  if (mean_loss) *mean_loss = steps ? total / steps : 0.0;
  return LBM_OK;
}

lbm_status lbm_sg_set_lr(lbm_sg *s, float lr) {
  if (!s || !(lr > 0.f)) return fail(LBM_INVALID, "bad learning rate");
  s->cfg.lr = lr;
  return LBM_OK;
}

lbm_status lbm_sg_adam_step(lbm_sg *s) {
  if (!s) return fail(LBM_INVALID, "null argument");
  adam(s);
  if (cudaStreamSynchronize(s->stream) != cudaSuccess) return fail(LBM_CUDA, "adam failed");
  return LBM_OK;
}

}  // extern "C"
