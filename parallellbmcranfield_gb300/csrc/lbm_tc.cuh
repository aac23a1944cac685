// tcgen05 products of the warm-start network (5th-generation tensor cores:
// accumulators in tensor memory, operands read from shared memory by the
// MMA unit, one thread issuing the MMAs).
//
//   k_tc_conv   C[p][n] = sum_k A[p][k] Bt[n][k] with A the implicit im2col
//               of an NHWC tensor (forward: X and W; input gradient: dZ and
//               the flipped W).  M = 128 pixels per block, N = BN outputs.
//   k_tc_wgrad  dW[n][k] += sum_p im2col(X)[p][k] dZ[p][n], computed as the
//               transposed product dW^T[k][n] (M = 128 values of k = tap*C + c
//               per block, N = BN output channels), pixels split over
//               blockIdx.z, FP32 atomics into dW.
//
// Pipeline: 3 or 4 shared-memory stages of TC_BK = 64 K values; all 128
// threads fill a stage with 16-byte cp.async copies (zero-filled where the
// im2col or the tile runs out), fence them to the async proxy, and thread 0
// issues four 128 x BN x 16 MMAs (kind::f16, BF16 in, FP32 accumulate) and a
// tcgen05.commit to the stage's mbarrier; a stage is refilled only after that
// mbarrier reports the MMAs reading it complete.  Every mbarrier wait is
// bounded: on expiry the block sets *err, stops issuing, waits (bounded) for
// the MMAs in flight, frees its tensor memory and returns.
//
// Shared-memory operand layout (no swizzle, "interleaved"): 8 x 16-byte core
// matrices of 128 contiguous bytes.
//   K-major (row r of M or N, column k):   (r/8)*1024 + (k/8)*128 + (r%8)*16 + (k%8)*2
//            descriptor LBO = 128 (next 8 k), SBO = 1024 (next 8 rows)
//   MN-major (element r of M or N, k):     (k/8)*(R*16) + (r/8)*128 + (k%8)*16 + (r%8)*2
//            descriptor LBO = R*16 (next 8 k), SBO = 128 (next 8 r): in the
//            no-swizzle MN-major form the two offsets swap roles against the
//            swizzled MN-major forms
// (R = rows of the tile.)  Tensor memory holds D with row i of the tile in
// lane i and column j in column j; warp w reads lanes 32w..32w+31.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace sgtc {

using bf16 = __nv_bfloat16;

constexpr int TC_BM = 128;
constexpr int TC_BK = 64;
constexpr int TC_THREADS = 128;
constexpr long long TC_POLLS = 1ll << 20;  // mbarrier polls before a wait gives up (about a second)

__device__ __forceinline__ uint32_t saddr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// tcgen05 shared-memory matrix descriptor without swizzling: start address,
// leading and stride byte offsets (16-byte units), version field 0b001 at
// bits 46-48, base offset 0, swizzle mode 0.
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo & 0x3FFFFu) >> 4) << 16) |
         ((uint64_t)((sbo & 0x3FFFFu) >> 4) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9, 10-12 = 1), A / B major (bit 15 / 16: 0 K-major, 1 MN-major),
// N >> 3 (bits 17-22), M >> 4 (bits 24-28).
__host__ __device__ constexpr uint32_t tc_idesc(int n, int a_mn, int b_mn) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)a_mn << 15) | ((uint32_t)b_mn << 16) |
         ((uint32_t)(n >> 3) << 17) | ((uint32_t)(TC_BM >> 4) << 24);
}

__device__ __forceinline__ void cp16(uint32_t dst, const void *src, bool pred) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src),
               "r"(pred ? 16 : 0));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

__device__ __forceinline__ void mb_init(uint64_t *b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(saddr(b)), "r"(count));
}
__device__ __forceinline__ bool mb_try(uint64_t *b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(saddr(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mb_wait(uint64_t *b, uint32_t parity) {
  for (long long i = 0; i < TC_POLLS; i++)
    if (mb_try(b, parity)) return true;
  return false;
}

// Tensor memory (warp-wide): allocate ncols columns (a power of two >= 32),
// the address lands in *slot.
__device__ __forceinline__ void tm_alloc(uint32_t *slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                   saddr(slot)),
               "r"(ncols));
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
}
__device__ __forceinline__ void tm_free(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols));
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

// D[tmem] (+)= A[desc] x B[desc]^T, one thread.
__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                       uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
// The mbarrier receives one arrival when every MMA this thread issued before is done.
__device__ __forceinline__ void tc_commit(uint64_t *b) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                   saddr(b))
               : "memory");
}
// 16 consecutive FP32 columns of this thread's lane.
__device__ __forceinline__ void tm_ld16(uint32_t taddr, float v[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
      "[%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// TMA: the mbarrier expects `bytes` more (this thread's arrival included);
// tiled tensor loads of 4 and 5 dimensions completing on that mbarrier.
__device__ __forceinline__ void mb_expect_tx(uint64_t *b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(saddr(b)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap *map, uint64_t *bar,
                                            int c0, int c1, int c2, int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%3, %4, %5, %6}], [%2];\n" ::"r"(dst),
      "l"((uint64_t)map), "r"(saddr(bar)), "r"(c0), "r"(c1), "r"(c2), "r"(c3)
      : "memory");
}
__device__ __forceinline__ void tma_load_5d(uint32_t dst, const CUtensorMap *map, uint64_t *bar,
                                            int c0, int c1, int c2, int c3, int c4) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%3, %4, %5, %6, %7}], [%2];\n" ::"r"(dst),
      "l"((uint64_t)map), "r"(saddr(bar)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4)
      : "memory");
}

// Dynamic shared memory of a block: the stages, then the mbarriers and the
// tensor-memory address (64 bytes), then the convolution's K table (one int
// per 8 K values, TC_KTAB entries), from a 1024-byte aligned base.
// Ring depth: 4 stages up to 64 columns (two blocks fit an SM), 3 at 128.
constexpr int TC_KTAB = 1024;  // K up to 8192
template <int BN>
struct TcSmem {
  static constexpr int STAGES = BN >= 128 ? 3 : 4;
  static constexpr int A_BYTES = TC_BM * TC_BK * 2;
  static constexpr int B_BYTES = BN * TC_BK * 2;
  static constexpr int STAGE = A_BYTES + B_BYTES;
  static constexpr int BYTES = STAGES * STAGE + 64 + TC_KTAB * 4;
  static constexpr int ALLOC = BYTES + 1024;  // room to align the base
};

// The main loop shared by both kernels.  load(stage_a, stage_b, kt) issues
// this thread's cp.async copies of K tile kt; a_k16 / b_k16 are the byte
// advances of the A / B descriptors per MMA (16 K values).  Returns false if
// a bounded wait gave up (the MMAs issued are complete or abandoned).
template <int BN, class Load>
__device__ __forceinline__ bool tc_mainloop(uint8_t *sm, uint32_t tmem, int nk, uint32_t idesc,
                                            uint32_t a_lbo, uint32_t a_sbo, uint32_t a_k16,
                                            uint32_t b_lbo, uint32_t b_sbo, uint32_t b_k16,
                                            Load load, int *err) {
  using S = TcSmem<BN>;
  uint64_t *bars = (uint64_t *)(sm + S::STAGES * S::STAGE);
  const int tid = threadIdx.x;
#pragma unroll
  for (int s = 0; s < S::STAGES - 1; s++) {
    if (s < nk) load(sm + s * S::STAGE, sm + s * S::STAGE + S::A_BYTES, s);
    cp_commit();
  }
  bool ok = true;
  for (int kt = 0; kt < nk; kt++) {
    const int s = kt % S::STAGES;
    cp_wait<S::STAGES - 2>();
    fence_async_smem();
    if (!__syncthreads_and(ok)) {
      ok = false;
      break;
    }
    if (tid == 0) {
      tc_fence_after();
      const uint32_t a0 = saddr(sm + s * S::STAGE), b0 = a0 + S::A_BYTES;
#pragma unroll
      for (int kk = 0; kk < TC_BK / 16; kk++)
        tc_mma(tmem, tc_desc(a0 + kk * a_k16, a_lbo, a_sbo), tc_desc(b0 + kk * b_k16, b_lbo, b_sbo),
               idesc, (kt | kk) != 0);
      tc_commit(&bars[s]);
    }
    const int nt = kt + S::STAGES - 1;
    if (nt < nk) {
      // stage nt % S was last read by the MMAs of tile kt - 1
      if (kt >= 1 && !mb_wait(&bars[(kt - 1) % S::STAGES], ((kt - 1) / S::STAGES) & 1)) ok = false;
      if (ok) load(sm + (nt % S::STAGES) * S::STAGE, sm + (nt % S::STAGES) * S::STAGE + S::A_BYTES, nt);
    }
    cp_commit();
  }
  cp_wait<0>();
  // the last commit covers every MMA issued before it
  if (nk > 0 && !mb_wait(&bars[(nk - 1) % S::STAGES], ((nk - 1) / S::STAGES) & 1)) ok = false;
  ok = __syncthreads_and(ok) != 0;
  __syncwarp();  // thread 0 issued the MMAs alone; the epilogue's tcgen05.ld needs the whole warp
  tc_fence_after();
  if (!ok && tid == 0) atomicExch(err, 1);
  return ok;
}

// Block set-up: mbarriers (thread 0) and BN columns of tensor memory (warp 0).
template <int BN>
__device__ __forceinline__ uint32_t tc_setup(uint8_t *sm) {
  using S = TcSmem<BN>;
  uint64_t *bars = (uint64_t *)(sm + S::STAGES * S::STAGE);
  uint32_t *slot = (uint32_t *)(bars + S::STAGES);
  if (threadIdx.x == 0)
    for (int s = 0; s < S::STAGES; s++) mb_init(&bars[s], 1);
  // tcgen05.alloc / ld / dealloc are .sync.aligned: the warp must arrive
  // converged, also after code that only one of its threads ran
  __syncwarp();
  if (threadIdx.x < 32) tm_alloc(slot, BN < 32 ? 32 : BN);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  return *slot;
}
template <int BN>
__device__ __forceinline__ void tc_teardown(uint32_t tmem) {
  tc_fence_before();
  __syncthreads();
  __syncwarp();
  if (threadIdx.x < 32) tm_free(tmem, BN < 32 ? 32 : BN);
}

__device__ __forceinline__ uint8_t *tc_smem_base() {
  extern __shared__ uint8_t tc_dyn[];
  return (uint8_t *)(((uintptr_t)tc_dyn + 1023) & ~(uintptr_t)1023);
}

enum TcEpi : int { TC_BIAS_RELU = 0, TC_BIAS = 1, TC_PLAIN = 2 };

// Epilogue through shared memory: each warp's 32 rows of the accumulator tile
// (tcgen05.ld), bias / ReLU, BF16, into `tile` (rows of BN * 2 + 16 bytes,
// freed stage memory), then 16-byte copies of whole row segments to
// out[row][n0 .. n0 + BN) (row length N): consecutive threads write
// consecutive 16 bytes instead of each thread writing 4 bytes of its own row.
// Needs N and n0 multiples of 8 and a 16-byte aligned `out`.
template <int EPI, int BN>
__device__ __forceinline__ void tc_epilogue_tile(uint32_t tmem, uint8_t *tile, long long row0,
                                                 int rows, int N, int n0,
                                                 const float *__restrict__ bias,
                                                 bf16 *__restrict__ out) {
  constexpr int RS = BN * 2 + 16;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  uint8_t *mine = tile + (warp * 32 + lane) * RS;
#pragma unroll
  for (int c0 = 0; c0 < BN; c0 += 16) {
    float v[16];
    tm_ld16(tmem + ((uint32_t)(warp * 32) << 16) + c0, v);
    uint32_t w[8];
#pragma unroll
    for (int j = 0; j < 16; j += 2) {
      const int n = n0 + c0 + j;
      float v0 = v[j], v1 = v[j + 1];
      if (EPI != TC_PLAIN) {
        if (n < N) v0 += bias[n];
        if (n + 1 < N) v1 += bias[n + 1];
      }
      if (EPI == TC_BIAS_RELU) {
        v0 = fmaxf(v0, 0.f);
        v1 = fmaxf(v1, 0.f);
      }
      const __nv_bfloat162 h = __floats2bfloat162_rn(v0, v1);
      memcpy(&w[j / 2], &h, 4);
    }
    *(uint4 *)(mine + c0 * 2) = make_uint4(w[0], w[1], w[2], w[3]);
    *(uint4 *)(mine + c0 * 2 + 16) = make_uint4(w[4], w[5], w[6], w[7]);
  }
  __syncthreads();
  constexpr int CPR = BN * 2 / 16;  // 16-byte chunks per row
  for (int i = tid; i < TC_BM * CPR; i += TC_THREADS) {
    const int r = i / CPR, ch = i - r * CPR;
    if (r < rows && n0 + ch * 8 < N)
      *(uint4 *)(out + (row0 + r) * N + n0 + ch * 8) = *(const uint4 *)(tile + r * RS + ch * 16);
  }
}

// Convolution as C[p][n] = im2col(X)[p][k] Bt[n][k]: X is [P][H][W][C] BF16
// (C a multiple of 8: a 16-byte chunk never straddles two taps), taps 9
// (3x3, pad 1) or 1, k = tap*C + c < taps*C, Bt is [N][Kp] (rows of Kp
// values, zero beyond taps*C).  Output [P][N] BF16 with bias and ReLU per EPI.
template <int EPI, int BN>
__global__ void __launch_bounds__(TC_THREADS) k_tc_conv(const bf16 *__restrict__ X, int P, int H,
                                                        int W, int C, int taps,
                                                        const bf16 *__restrict__ Bt, int N, int Kp,
                                                        const float *__restrict__ bias,
                                                        bf16 *__restrict__ out, int *err) {
  uint8_t *sm = tc_smem_base();
  const uint32_t tmem = tc_setup<BN>(sm);
  const int tid = threadIdx.x;
  const int m0 = blockIdx.x * TC_BM, n0 = blockIdx.y * BN;
  const int KC = taps * C;
  const int nk = (Kp + TC_BK - 1) / TC_BK;
  // Copy pattern: one warp instruction moves 8 rows x 4 consecutive 16-byte
  // chunks (64 contiguous bytes of a pixel's tap in global memory; in shared
  // memory 8 distinct row slots of 16 bytes, the minimum 4 wavefronts).
  // This thread's rows of the A tile: rb * 8 + lane / 4 for rb = 4 j + warp.
  const int lane = tid & 31, warp = tid >> 5, l4 = lane & 3, r8 = lane >> 2;
  int pp[4], px[4], py[4];
  bool pin[4];
#pragma unroll
  for (int j = 0; j < 4; j++) {
    pp[j] = m0 + (j * 4 + warp) * 8 + r8;
    pin[j] = pp[j] < P;
    px[j] = pin[j] ? pp[j] % W : 0;
    py[j] = pin[j] ? (pp[j] / W) % H : 0;
  }
  // K table: per 8 K values the tap offsets and the channel, or -1 past K
  // (no integer divisions in the copy loop)
  int *ktab = (int *)(sm + TcSmem<BN>::STAGES * TcSmem<BN>::STAGE + 64);
  for (int j = tid; j < Kp / 8; j += TC_THREADS) {
    const int k = j * 8;
    int e = -1;
    if (k < KC) {
      const int r = k / C, c = k - r * C;
      const int dy = taps == 9 ? r / 3 : 1, dx = taps == 9 ? r % 3 : 1;
      e = (c << 4) | (dy << 2) | dx;
    }
    ktab[j] = e;
  }
  __syncthreads();
  auto load = [&](uint8_t *sa, uint8_t *sb, int kt) {
    const uint32_t a = saddr(sa), b = saddr(sb);
    const int k0 = kt * TC_BK;
#pragma unroll
    for (int i = 0; i < 8; i++) {
      const int j = i >> 1, kc = (i & 1) * 4 + l4;
      const int k = k0 + kc * 8;
      const int e = k < Kp ? ktab[k >> 3] : -1;
      const int dy = ((e >> 2) & 3) - 1, dx = (e & 3) - 1, c = e >> 4;
      const int yy = py[j] + dy, xx = px[j] + dx;
      const bool ok = pin[j] && e >= 0 && yy >= 0 && yy < H && xx >= 0 && xx < W;
      const bf16 *src = ok ? X + ((size_t)(pp[j] + dy * W + dx) * C + c) : X;
      cp16(a + (j * 4 + warp) * 1024 + kc * 128 + r8 * 16, src, ok);
    }
    // B tile: BN rows x 8 chunks, row blocks of 8 by the same pattern
#pragma unroll
    for (int i = 0; i < BN / 16; i++) {
      const int rb = (i >> 1) * 4 + warp, kc = (i & 1) * 4 + l4;
      const int r = rb * 8 + r8;
      const int k = k0 + kc * 8;
      const bool ok = n0 + r < N && k < Kp;
      cp16(b + rb * 1024 + kc * 128 + r8 * 16, ok ? Bt + (size_t)(n0 + r) * Kp + k : Bt, ok);
    }
  };
  const bool ok = tc_mainloop<BN>(sm, tmem, nk, tc_idesc(BN, 0, 0), 128, 1024, 256, 128, 1024, 256,
                                  load, err);
  if (ok && (N & 7) == 0 && ((uintptr_t)out & 15) == 0) {
    // the stages are free: the main loop waited for every copy and MMA
    tc_epilogue_tile<EPI, BN>(tmem, sm, m0, min(TC_BM, P - m0), N, n0, bias, out);
  } else if (ok) {
    const int row = m0 + warp * 32 + lane;
#pragma unroll
    for (int c0 = 0; c0 < BN; c0 += 16) {
      float v[16];
      tm_ld16(tmem + ((uint32_t)(warp * 32) << 16) + c0, v);
      if (row < P) {
#pragma unroll
        for (int j = 0; j < 16; j += 2) {
          const int n = n0 + c0 + j;
          float v0 = v[j], v1 = v[j + 1];
          if (EPI != TC_PLAIN) {
            if (n < N) v0 += bias[n];
            if (n + 1 < N) v1 += bias[n + 1];
          }
          if (EPI == TC_BIAS_RELU) {
            v0 = fmaxf(v0, 0.f);
            v1 = fmaxf(v1, 0.f);
          }
          if (n + 1 < N && (N & 1) == 0)
            *(__nv_bfloat162 *)(out + (size_t)row * N + n) = __floats2bfloat162_rn(v0, v1);
          else {
            if (n < N) out[(size_t)row * N + n] = __float2bfloat16_rn(v0);
            if (n + 1 < N) out[(size_t)row * N + n + 1] = __float2bfloat16_rn(v1);
          }
        }
      }
    }
  }
  tc_teardown<BN>(tmem);
}

// Weight gradient dW[n][k] += sum over pixels p in [pbeg, pend) of
// im2col(X)[p][k] * dZ[p][n], as the product dW^T[k][n] with both operands
// MN-major in shared memory (pixels are the K of the MMA).  dZ is [P][N]
// (N a multiple of 8), dW rows are ldw long; k < taps*C and n < N are written.
template <int BN>
__global__ void __launch_bounds__(TC_THREADS) k_tc_wgrad(const bf16 *__restrict__ dZ,
                                                         const bf16 *__restrict__ X, int P, int H,
                                                         int W, int C, int taps, int N,
                                                         float *__restrict__ dW, int ldw,
                                                         int pchunk, int *err) {
  uint8_t *sm = tc_smem_base();
  const uint32_t tmem = tc_setup<BN>(sm);
  const int tid = threadIdx.x;
  const int m0 = blockIdx.x * TC_BM, n0 = blockIdx.y * BN;
  const int KC = taps * C;
  const int pbeg = blockIdx.z * pchunk, pend = min(P, pbeg + pchunk);
  const int nk = pend > pbeg ? (pend - pbeg + TC_BK - 1) / TC_BK : 0;
  // Copy pattern: one warp instruction moves 8 pixels x 4 consecutive
  // 16-byte chunks (64 contiguous bytes per pixel in global memory, 8 distinct
  // pixel slots in shared memory).  This thread's pixels of a K tile:
  // (2 warp + h) * 8 + lane / 4 for h = 0, 1.
  const int lane = tid & 31, warp = tid >> 5, l4 = lane & 3, r8 = lane >> 2;
  // This thread's four K chunks are the same in every K tile (the block's M
  // rows): their tap offsets and channels once, here.
  int kdy[4], kdx[4], kc0[4];
  bool kin[4];
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int k = m0 + (q * 4 + l4) * 8;
    const int r = k / C;
    kin[q] = k < KC;
    kc0[q] = k - r * C;
    kdy[q] = taps == 9 ? r / 3 - 1 : 0;
    kdx[q] = taps == 9 ? r % 3 - 1 : 0;
  }
  // pixel coordinates of the two pixels of this thread, advanced by one K
  // tile (64 pixels) per call: the loads are issued for kt = 0, 1, 2, ...
  int p[2], px[2], py[2];
#pragma unroll
  for (int h = 0; h < 2; h++) {
    p[h] = pbeg + (2 * warp + h) * 8 + r8;
    px[h] = p[h] % W;
    py[h] = (p[h] / W) % H;
  }
  int kt_at = 0;
  auto load = [&](uint8_t *sa, uint8_t *sb, int kt) {
    const uint32_t a = saddr(sa), b = saddr(sb);
    while (kt_at < kt) {
#pragma unroll
      for (int h = 0; h < 2; h++) {
        p[h] += TC_BK;
        px[h] += TC_BK;
        while (px[h] >= W) {
          px[h] -= W;
          if (++py[h] == H) py[h] = 0;
        }
      }
      kt_at++;
    }
    bool pin[2];
#pragma unroll
    for (int h = 0; h < 2; h++) pin[h] = p[h] < pend;
    // A: 16 chunks of 8 k values per pixel
#pragma unroll
    for (int i = 0; i < 8; i++) {
      const int h = i & 1, q = i >> 1, kc = q * 4 + l4;
      const int yy = py[h] + kdy[q], xx = px[h] + kdx[q];
      const bool ok = pin[h] && kin[q] && yy >= 0 && yy < H && xx >= 0 && xx < W;
      const bf16 *src = ok ? X + ((size_t)(p[h] + kdy[q] * W + kdx[q]) * C + kc0[q]) : X;
      cp16(a + (2 * warp + h) * (TC_BM * 16) + kc * 128 + r8 * 16, src, ok);
    }
    // B: BN / 8 chunks of 8 output channels per pixel
#pragma unroll
    for (int i = 0; i < BN / 16; i++) {
      const int h = i & 1, cc = (i >> 1) * 4 + l4;
      const int n = n0 + cc * 8;
      const bool ok = pin[h] && n < N;
      cp16(b + (2 * warp + h) * (BN * 16) + cc * 128 + r8 * 16, ok ? dZ + (size_t)p[h] * N + n : dZ,
           ok);
    }
  };
  // MN-major without swizzle: LBO is the K-direction stride of 8-row groups,
  // SBO the MN-direction stride of core matrices
  const bool ok = tc_mainloop<BN>(sm, tmem, nk, tc_idesc(BN, 1, 1), TC_BM * 16, 128, 2 * TC_BM * 16,
                                  BN * 16, 128, 2 * BN * 16, load, err);
  if (ok && nk > 0) {
    const int k = m0 + warp * 32 + lane;
#pragma unroll
    for (int c0 = 0; c0 < BN; c0 += 16) {
      float v[16];
      tm_ld16(tmem + ((uint32_t)(warp * 32) << 16) + c0, v);
      if (k < KC) {
#pragma unroll
        for (int j = 0; j < 16; j++) {
          const int n = n0 + c0 + j;
          if (n < N) atomicAdd(dW + (size_t)n * ldw + k, v[j]);
        }
      }
    }
  }
  tc_teardown<BN>(tmem);
}

// 3x3 convolution (pad 1) of an NHWC tensor with W a multiple of 128 and C a
// multiple of 32, N a multiple of BN outputs: the halo-tile form.  A block computes 128
// consecutive pixels of one image row.  Per 32-channel chunk one TMA load
// stages the halo -- rows y-1..y+1, pixels x0-1..x0+128, 4 groups of 8
// channels, zero outside the image -- as [row][group][pixel][8 channels]
// (16 bytes per pixel, so a one-pixel shift is a 16-byte shift of the
// descriptor's start address), and one TMA load stages the weights of all
// nine taps as [tap][group][output][8 channels].  The nine taps are then
// MMAs on offsets of the same halo: every input pixel crosses from L2 once
// per chunk instead of nine times.  Tensor maps (built by the host):
//   mapA: dims (8, W, C/8, H, images), strides (C*2, 16, W*C*2, H*W*C*2),
//         box (8, 130, 4, 3, 1)
//   mapB: dims (8, N, C/8, 9), strides (Kp*2, 16, C*2), box (8, BN, 4, 9) at n0
// S stages (1 or 2) of TcHalo<BN>::STAGE bytes; thread 0 issues the loads
// and the MMAs, every wait is bounded.
constexpr int TH_A_BYTES = 8 * 130 * 4 * 3 * 2;  // 24960
constexpr int TH_A_SLOT = 25600;                  // rounded up to 1024
template <int BN>
struct TcHalo {
  static constexpr int B_BYTES = 8 * BN * 4 * 9 * 2;
  static constexpr int STAGE = TH_A_SLOT + B_BYTES;
  static constexpr int bytes(int stages) { return stages * STAGE + 64 + 1024; }
};

template <int EPI, int BN>
__global__ void __launch_bounds__(TC_THREADS) k_tc_conv3h(const __grid_constant__ CUtensorMap mapA,
                                                          const __grid_constant__ CUtensorMap mapB,
                                                          int H, int W, int C, int N, int S,
                                                          const float *__restrict__ bias,
                                                          bf16 *__restrict__ out, int *err) {
  using T = TcHalo<BN>;
  uint8_t *sm = tc_smem_base();
  uint64_t *bars = (uint64_t *)(sm + S * T::STAGE);  // full[2], empty[2], done
  uint64_t *full = bars, *empty = bars + 2, *done = bars + 4;
  uint32_t *slot = (uint32_t *)(bars + 5);
  const int tid = threadIdx.x;
  // blockIdx.x: row segment (W / 128 of them) and output tile n0 = BN * tile
  const int segs = W / TC_BM;
  const int x0 = (blockIdx.x % segs) * TC_BM, n0 = (blockIdx.x / segs) * BN;
  const int y = blockIdx.y, img = blockIdx.z;
  const int nch = C / 32;
  if (tid == 0) {
    for (int i = 0; i < 5; i++) mb_init(&bars[i], 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    fence_async_smem();
  }
  __syncwarp();
  if (tid < 32) tm_alloc(slot, BN < 32 ? 32 : BN);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *slot;
  bool ok = true;
  // warp 0 issues, lane 0 alone; its other lanes wait at __syncwarp
  // instead of polling the mbarrier beside it
  if (tid < 32) {
    if (tid == 0) {
      const uint32_t idesc = tc_idesc(BN, 0, 0);
      int issued = 0, consumed = 0;  // chunks whose loads were issued / have landed
      auto issue = [&](int kc, int st) {
        const uint32_t a = saddr(sm + st * T::STAGE), b = a + TH_A_SLOT;
        mb_expect_tx(&full[st], TH_A_BYTES + T::B_BYTES);
        tma_load_5d(a, &mapA, &full[st], 0, x0 - 1, kc * 4, y - 1, img);
        tma_load_4d(b, &mapB, &full[st], 0, n0, kc * 4, 0);
        issued = kc + 1;
      };
      for (int i = 0; i < S && i < nch; i++) issue(i, i);
      for (int kc = 0; kc < nch && ok; kc++) {
        const int st = kc % S;
        const uint32_t ph = (uint32_t)(kc / S) & 1u;
        if (!mb_wait(&full[st], ph)) {
          ok = false;
          break;
        }
        consumed = kc + 1;
        tc_fence_after();
        const uint32_t a = saddr(sm + st * T::STAGE), b = a + TH_A_SLOT;
        // the taps are start-address offsets, added to the descriptors'
        // address field (16-byte units, no carry: shared addresses < 2^18)
        const uint64_t da = tc_desc(a, 2080, 128), db = tc_desc(b, BN * 16, 128);
  #pragma unroll
        for (int tap = 0; tap < 9; tap++) {
          const int dy = tap / 3, dx = tap % 3;  // offsets + 1
  #pragma unroll
          for (int k2 = 0; k2 < 2; k2++)
            tc_mma(tmem, da + (uint64_t)((dy * (4 * 2080) + (2 * k2) * 2080 + dx * 16) >> 4),
                   db + (uint64_t)((tap * (4 * BN * 16) + (2 * k2) * (BN * 16)) >> 4), idesc,
                   (kc | tap | k2) != 0);
        }
        tc_commit(&empty[st]);
        // refill the stage the previous chunk used: its MMAs complete ahead of
        // the ones just issued, which keep the tensor pipe busy meanwhile
        if (kc >= 1 && kc - 1 + S < nch) {
          const int pst = (kc - 1) % S;
          if (!mb_wait(&empty[pst], (uint32_t)((kc - 1) / S) & 1u)) {
            ok = false;
            break;
          }
          issue(kc - 1 + S, pst);
        }
      }
      tc_commit(done);  // arrives when every MMA issued above is complete
      if (!ok) {
        // loads still in flight land in this block's shared memory: wait for
        // them (bounded) before the block may exit
        for (int kc = consumed; kc < issued; kc++) mb_wait(&full[kc % S], (uint32_t)(kc / S) & 1u);
      }
    }
    __syncwarp();
  }
  if (!mb_wait(done, 0)) ok = false;
  ok = __syncthreads_and(ok) != 0;
  __syncwarp();
  tc_fence_after();
  if (!ok) {
    if (tid == 0) atomicExch(err, 1);
  } else {
    // the stages are free: every MMA has completed and every load landed
    tc_epilogue_tile<EPI, BN>(tmem, sm, ((long long)img * H + y) * W + x0, TC_BM, N, n0, bias, out);
  }
  tc_fence_before();
  __syncthreads();
  __syncwarp();
  if (tid < 32) tm_free(tmem, BN < 32 ? 32 : BN);
}

// The halo-tile convolution over several row segments per block: rows
// y0 .. y0 + TC_SEGS - 1 at the same x0, output tile and image, so that the
// loads, MMAs and epilogue of consecutive segments overlap instead of
// following one another as in k_tc_conv3h, and more halo loads are in
// flight per SM.  The weights of all 32-channel chunks (one TMA load each,
// tensor map as for k_tc_conv3h) stay in shared memory for the whole block;
// the halos (one TMA load per segment and chunk) go through a ring of S
// stages, S from the host.  Warp 4 (one lane) issues the loads and the MMAs,
// each segment into one of two tensor-memory accumulators; warps 0-3
// (tensor-memory lanes 0-127: warp w reads lanes 32w..32w+31) drain the
// other accumulator, each thread storing its pixel's BN outputs as 32-byte
// row pieces (two 16-byte stores per 16 columns, whole sectors).
// mbarriers: wfull (the weights landed), full / empty per stage (the halo
// landed / the MMAs reading it are done), accfull per accumulator (its
// segment's MMAs are done), accfree per accumulator (128 arrivals: the
// epilogue has read it), done (every MMA issued is done).  Every wait is
// bounded; on expiry the block sets *err, stops issuing, lets the loads and
// MMAs in flight finish (bounded) and frees its tensor memory.
constexpr int TC_SEGS = 4;
constexpr int TC3M_THREADS = 160;
constexpr int TC3M_MAX_STAGES = 8;
template <int BN>
struct TcHaloM {
  static constexpr int B_CHUNK = TcHalo<BN>::B_BYTES;  // weights of one 32-channel chunk
  // halo ring, weights, mbarriers and the tensor-memory slot (256 bytes), alignment slack
  static constexpr int bytes(int stages, int nch) {
    return stages * TH_A_SLOT + nch * B_CHUNK + 256 + 1024;
  }
};

__device__ __forceinline__ void mb_arrive(uint64_t *b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(saddr(b)) : "memory");
}

template <int EPI, int BN>
__global__ void __launch_bounds__(TC3M_THREADS) k_tc_conv3m(const __grid_constant__ CUtensorMap mapA,
                                                            const __grid_constant__ CUtensorMap mapB,
                                                            int H, int W, int C, int N, int S,
                                                            const float *__restrict__ bias,
                                                            bf16 *__restrict__ out, int *err) {
  static_assert(BN >= 32 && BN <= 128 && BN % 16 == 0, "accumulator width");
  using M = TcHaloM<BN>;
  uint8_t *sm = tc_smem_base();
  const int nch = C / 32;
  uint8_t *wts = sm + S * TH_A_SLOT;  // nch chunks of weights
  uint64_t *bars = (uint64_t *)(wts + nch * M::B_CHUNK);
  uint64_t *full = bars, *empty = bars + TC3M_MAX_STAGES;
  uint64_t *accfull = bars + 2 * TC3M_MAX_STAGES, *accfree = accfull + 2, *done = accfull + 4,
           *wfull = accfull + 5;
  uint32_t *slot = (uint32_t *)(accfull + 6);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int segs = W / TC_BM;
  const int x0 = (blockIdx.x % segs) * TC_BM, n0 = (blockIdx.x / segs) * BN;
  const int y0 = blockIdx.y * TC_SEGS, img = blockIdx.z;
  const int G = TC_SEGS * nch;  // halo loads of this block, segment-major
  if (tid == 0) {
    for (int i = 0; i < 2 * TC3M_MAX_STAGES; i++) mb_init(&bars[i], 1);
    mb_init(&accfull[0], 1);
    mb_init(&accfull[1], 1);
    mb_init(&accfree[0], TC_BM);
    mb_init(&accfree[1], TC_BM);
    mb_init(done, 1);
    mb_init(wfull, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    fence_async_smem();
  }
  __syncwarp();
  if (tid < 32) tm_alloc(slot, 2 * BN);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *slot;
  bool ok = true;
  if (warp == 4) {
    if (lane == 0) {
      const uint32_t idesc = tc_idesc(BN, 0, 0);
      int issued = 0, consumed = 0;  // halo loads issued / landed
      bool wlanded = false;
      auto issue = [&](int g, int st) {
        const int seg = g / nch, kc = g - seg * nch;
        mb_expect_tx(&full[st], TH_A_BYTES);
        tma_load_5d(saddr(sm + st * TH_A_SLOT), &mapA, &full[st], 0, x0 - 1, kc * 4, y0 + seg - 1,
                    img);
        issued = g + 1;
      };
      mb_expect_tx(wfull, nch * M::B_CHUNK);
      for (int kc = 0; kc < nch; kc++)
        tma_load_4d(saddr(wts + kc * M::B_CHUNK), &mapB, wfull, 0, n0, kc * 4, 0);
      for (int i = 0; i < S && i < G; i++) issue(i, i);
      ok = mb_wait(wfull, 0);
      wlanded = ok;
      for (int g = 0; g < G && ok; g++) {
        const int seg = g / nch, kc = g - seg * nch, st = g % S, acc = seg & 1;
        // the accumulator of segment seg - 2 must have been read out
        if (kc == 0 && seg >= 2 && !mb_wait(&accfree[acc], (uint32_t)((seg - 2) >> 1) & 1u)) {
          ok = false;
          break;
        }
        if (!mb_wait(&full[st], (uint32_t)(g / S) & 1u)) {
          ok = false;
          break;
        }
        consumed = g + 1;
        tc_fence_after();
        const uint32_t a = saddr(sm + st * TH_A_SLOT), b = saddr(wts + kc * M::B_CHUNK);
        const uint32_t d = tmem + (uint32_t)(acc * BN);
        // the taps are start-address offsets, added to the descriptors'
        // address field (16-byte units, no carry: shared addresses < 2^18)
        const uint64_t da = tc_desc(a, 2080, 128), db = tc_desc(b, BN * 16, 128);
#pragma unroll
        for (int tap = 0; tap < 9; tap++) {
          const int dy = tap / 3, dx = tap % 3;  // offsets + 1
#pragma unroll
          for (int k2 = 0; k2 < 2; k2++)
            tc_mma(d, da + (uint64_t)((dy * (4 * 2080) + (2 * k2) * 2080 + dx * 16) >> 4),
                   db + (uint64_t)((tap * (4 * BN * 16) + (2 * k2) * (BN * 16)) >> 4), idesc,
                   (kc | tap | k2) != 0);
        }
        tc_commit(&empty[st]);
        if (kc == nch - 1) tc_commit(&accfull[acc]);
        // refill the stage the previous halo used: its MMAs complete ahead
        // of the ones just issued
        if (g >= 1 && g - 1 + S < G) {
          const int pst = (g - 1) % S;
          if (!mb_wait(&empty[pst], (uint32_t)((g - 1) / S) & 1u)) {
            ok = false;
            break;
          }
          issue(g - 1 + S, pst);
        }
      }
      tc_commit(done);  // arrives when every MMA issued above is complete
      if (!ok) {
        // loads still in flight land in this block's shared memory: wait for
        // them (bounded) before the block may exit
        if (!wlanded) mb_wait(wfull, 0);
        for (int g = consumed; g < issued; g++) mb_wait(&full[g % S], (uint32_t)(g / S) & 1u);
      }
      if (!mb_wait(done, 0)) ok = false;
    }
    __syncwarp();
  } else {
    // epilogue: this thread's pixel of each segment, from the segment's accumulator
    for (int seg = 0; seg < TC_SEGS; seg++) {
      const int acc = seg & 1;
      const bool landed = __all_sync(0xffffffffu, mb_wait(&accfull[acc], (uint32_t)(seg >> 1) & 1u));
      tc_fence_after();
      if (landed && ok) {
        const long long row = ((long long)img * H + y0 + seg) * W + x0 + warp * 32 + lane;
        bf16 *o = out + row * N + n0;
#pragma unroll
        for (int c0 = 0; c0 < BN; c0 += 16) {
          float v[16];
          tm_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(acc * BN + c0), v);
          uint32_t w[8];
#pragma unroll
          for (int j = 0; j < 16; j += 2) {
            float v0 = v[j], v1 = v[j + 1];
            if (EPI != TC_PLAIN) {
              v0 += bias[n0 + c0 + j];
              v1 += bias[n0 + c0 + j + 1];
            }
            if (EPI == TC_BIAS_RELU) {
              v0 = fmaxf(v0, 0.f);
              v1 = fmaxf(v1, 0.f);
            }
            const __nv_bfloat162 h = __floats2bfloat162_rn(v0, v1);
            memcpy(&w[j / 2], &h, 4);
          }
          *(uint4 *)(o + c0) = make_uint4(w[0], w[1], w[2], w[3]);
          *(uint4 *)(o + c0 + 8) = make_uint4(w[4], w[5], w[6], w[7]);
        }
      } else {
        ok = false;
      }
      tc_fence_before();
      mb_arrive(&accfree[acc]);
    }
  }
  ok = __syncthreads_and(ok) != 0;
  if (!ok && tid == 0) atomicExch(err, 1);
  tc_fence_before();
  __syncthreads();
  __syncwarp();
  if (tid < 32) tm_free(tmem, 2 * BN);
}

// Weight gradient of a 3x3 convolution (pad 1, W a multiple of 128, C a
// multiple of 32) in the halo-tile form: dW[n][tap][c] = sum over pixels p of
// dZ[p][n] X[p + offset(tap)][c], as nine products D_tap[n][c] (M = 128
// output channels, N = 32 input channels of one chunk, K = pixels) that stay
// in tensor memory (9 x 32 columns) while the block walks its range of
// 128-pixel row segments.  Per segment one TMA load stages the X halo exactly
// as k_tc_conv3h does (its rows are the B operand, MN-major: pixels 16 bytes
// apart, so tap (dy, dx) is a start-address offset), and one TMA load stages
// dZ as [output group][pixel][8 outputs] (the A operand, MN-major).  FP32
// atomics add the block's nine tiles into dW at the end.
//   mapX:  as k_tc_conv3h's mapA
//   mapDZ: dims (8, W, N/8, H, images), strides (N*2, 16, W*N*2, H*W*N*2),
//          box (8, 128, min(16, N/8), 1, 1)
// Stages: TH_WS of TcHaloW::STAGE bytes (one block per SM: the nine tiles
// take 512 tensor-memory columns).
constexpr int TH_WS = 3;
struct TcHaloW {
  static constexpr int DZ_SLOT = 128 * 128 * 2;  // 16 groups x 128 pixels x 16 bytes
  static constexpr int STAGE = TH_A_SLOT + DZ_SLOT;
  static constexpr int BYTES = TH_WS * STAGE + 64 + 1024;
};

__global__ void __launch_bounds__(TC_THREADS) k_tc_wgrad3h(const __grid_constant__ CUtensorMap mapX,
                                                           const __grid_constant__ CUtensorMap mapDZ,
                                                           int H, int W, int C, int N, int nseg,
                                                           int seg_per_block, float *__restrict__ dW,
                                                           int ldw, int *err) {
  using T = TcHaloW;
  constexpr int S = TH_WS;
  uint8_t *sm = tc_smem_base();
  uint64_t *bars = (uint64_t *)(sm + S * T::STAGE);  // full[S], empty[S], done
  uint64_t *full = bars, *empty = bars + S, *done = bars + 2 * S;
  uint32_t *slot = (uint32_t *)(bars + 2 * S + 1);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int c0 = blockIdx.x * 32, n0 = blockIdx.y * 128;
  const int sbeg = blockIdx.z * seg_per_block, send = min(nseg, sbeg + seg_per_block);
  const int ns = send > sbeg ? send - sbeg : 0;
  const int groups = min(16, (N - n0) / 8);
  const uint32_t tx_bytes = TH_A_BYTES + 8 * 128 * groups * 2;
  const int segs_per_row = W / TC_BM;
  // two threads issue the MMAs, lane 0 of warp 0 (taps 0-4, and the loads)
  // and lane 0 of warp 1 (taps 5-8): one thread alone could not issue the
  // 72 MMAs of a segment as fast as the tensor pipe runs them.  empty[] and
  // done take one tcgen05.commit from each.
  if (tid == 0) {
    for (int i = 0; i < S; i++) mb_init(&bars[i], 1);
    for (int i = S; i < 2 * S + 1; i++) mb_init(&bars[i], 2);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    fence_async_smem();
  }
  __syncwarp();
  if (tid < 32) tm_alloc(slot, 512);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *slot;
  bool ok = true;
  // the other lanes of warps 0 and 1 wait at __syncwarp instead of polling
  // the mbarriers beside the issuing lanes
  if (warp < 2) {
    if (lane == 0) {
      const int role = warp;  // 0: taps 0-4 and the loads; 1: taps 5-8
      const uint32_t idesc = tc_idesc(32, 1, 1);
      int issued = 0, consumed = 0;
      auto issue = [&](int i, int st) {
        const int sg = sbeg + i;
        const int xs = sg % segs_per_row, row = sg / segs_per_row;
        const int y = row % H, img = row / H, x0 = xs * TC_BM;
        const uint32_t a = saddr(sm + st * T::STAGE), d = a + TH_A_SLOT;
        mb_expect_tx(&full[st], tx_bytes);
        tma_load_5d(a, &mapX, &full[st], 0, x0 - 1, c0 / 8, y - 1, img);
        tma_load_5d(d, &mapDZ, &full[st], 0, x0, n0 / 8, y, img);
        issued = i + 1;
      };
      if (role == 0)
        for (int i = 0; i < S && i < ns; i++) issue(i, i);
      for (int i = 0; i < ns && ok; i++) {
        const int st = i % S;
        const uint32_t ph = (uint32_t)(i / S) & 1u;
        if (!mb_wait(&full[st], ph)) {
          ok = false;
          break;
        }
        consumed = i + 1;
        tc_fence_after();
        const uint32_t xa = saddr(sm + st * T::STAGE), za = xa + TH_A_SLOT;
        // one descriptor per operand and stage; every tap and K step is a
        // start-address offset, added to the descriptor's address field
        // (16-byte units; shared addresses stay below 2^18, so no carry
        // leaves the field), and the 72 MMAs are unrolled: the issuing
        // thread spends a few instructions per MMA
        const uint64_t da = tc_desc(za, 128, 2048), db = tc_desc(xa, 128, 2080);
  #pragma unroll
        for (int tap = 0; tap < 9; tap++) {
          const int dy = tap / 3, dx = tap % 3;  // offsets + 1
          if ((tap < 5) != (role == 0)) continue;
  #pragma unroll
          for (int kk = 0; kk < 8; kk++)
            tc_mma(tmem + tap * 32, da + (uint64_t)((kk * 256) >> 4),
                   db + (uint64_t)((dy * (4 * 2080) + (16 * kk + dx) * 16) >> 4), idesc,
                   (i | kk) != 0);
        }
        tc_commit(&empty[st]);
        // refill the stage the previous segment used (see k_tc_conv3h)
        if (role == 0 && i >= 1 && i - 1 + S < ns) {
          const int pst = (i - 1) % S;
          if (!mb_wait(&empty[pst], (uint32_t)((i - 1) / S) & 1u)) {
            ok = false;
            break;
          }
          issue(i - 1 + S, pst);
        }
      }
      tc_commit(done);
      if (!ok && role == 0)
        for (int i = consumed; i < issued; i++) mb_wait(&full[i % S], (uint32_t)(i / S) & 1u);
    }
    __syncwarp();
  }
  if (!mb_wait(done, 0)) ok = false;
  ok = __syncthreads_and(ok) != 0;
  __syncwarp();
  tc_fence_after();
  if (!ok) {
    if (tid == 0) atomicExch(err, 1);
  } else if (ns > 0) {
    const int n = n0 + warp * 32 + lane;  // this thread's tensor-memory lane
#pragma unroll 1
    for (int tap = 0; tap < 9; tap++) {
#pragma unroll
      for (int h = 0; h < 2; h++) {
        float v[16];
        tm_ld16(tmem + ((uint32_t)(warp * 32) << 16) + tap * 32 + h * 16, v);
        if (n < N) {
          float *row = dW + (size_t)n * ldw + tap * C + c0 + h * 16;
#pragma unroll
          for (int j = 0; j < 16; j++) atomicAdd(row + j, v[j]);
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  __syncwarp();
  if (tid < 32) tm_free(tmem, 512);
}

}  // namespace sgtc
