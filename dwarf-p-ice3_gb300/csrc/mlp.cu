// mlp.cu — BF16 tensor-core (tcgen05) GEMM with fused epilogues, and the
// per-point MLP of the slow-process surrogate built on it (forward,
// hand-written backward, Adam).
//
// tc_gemm_kernel: one CTA (4 warps) computes a 128 x N tile (N <= 256) of
//   C[m][n] = sum_k A(m, k) B(n, k),  A(m, k) = A[m*sam + k*sak],  B(n, k) = B[n*sbn + k*sbk]
// in FP32 in TMEM.  K is walked in chunks of 64: the CTA stages the A and B
// chunks into shared memory in the K-major core-matrix layout (16-byte
// vector loads when K is the contiguous index, element loads otherwise,
// which also transposes), one thread issues the K/16 tcgen05.mma and commits
// to an mbarrier, and all threads wait (bounded) before the next chunk.
// Rows >= M and k >= K are staged as zeros.  The epilogue reads the tile
// back with tcgen05.ld (warp w: rows 32w..32w+31) and applies:
//   EPI_STORE     C -> f32 (split-K partials at C + split * M * ldc)
//   EPI_BIAS_GELU Z = C + bias -> f32 Zout (optional), H = GELU(Z) -> bf16
//   EPI_BIAS      Y = C + bias -> f32
//   EPI_DGELU     dZ = C * GELU'(Zin) -> bf16 H and f32 C
// On a barrier timeout the kernel sets *err, stops issuing and frees its
// TMEM after a second bounded wait.
#include <cuda_bf16.h>
#include <math.h>

#include "ice3gb_kernels.h"
#include "tc_sm103.cuh"

namespace {

constexpr int KC = 64;                 // K chunk per stage
constexpr long WAIT_ITERS = 1L << 22;  // bounded mbarrier wait (about a second at most)

// GELU in its tanh form, 0.5 z (1 + tanh(sqrt(2/pi) (z + 0.044715 z^3)))
// (Hendrycks & Gimpel 2016), with the hardware tanh.approx.f32: one MUFU
// operation and five FP32 operations per activation, the same function in
// training and inference.
__device__ __forceinline__ float tanh_hw(float x)
{
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float gelu(float z)
{
  const float u = z * fmaf(0.035677408136300125f, z * z, 0.7978845608028654f);
  const float h = 0.5f * z;
  return fmaf(h, tanh_hw(u), h);
}
__device__ __forceinline__ float dgelu(float z)
{
  const float z2 = z * z;
  const float th = tanh_hw(z * fmaf(0.035677408136300125f, z2, 0.7978845608028654f));
  const float du = fmaf(0.10703222440890037f, z2, 0.7978845608028654f);
  return 0.5f * (1.0f + th) + 0.5f * z * (1.0f - th * th) * du;
}

__global__ void __launch_bounds__(128) tc_gemm_kernel(const TcGemmArgs a)
{
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __nv_bfloat16 *sA = reinterpret_cast<__nv_bfloat16 *>(smem_raw);               // 128 x KC
  __nv_bfloat16 *sB = sA + 128 * KC;                                            // 256 x KC
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int np = (a.N + 15) & ~15;
  const uint32_t ncols = np <= 32 ? 32u : np <= 64 ? 64u : np <= 128 ? 128u : 256u;
  const long m0 = (long)blockIdx.x * 128;
  // K range of this split
  const int kpad = (a.K + 15) & ~15;
  const int ksplit = ((kpad / 16 + a.k_split - 1) / a.k_split) * 16;
  const int kbeg = blockIdx.y * ksplit;
  const int kend = min(kpad, kbeg + ksplit);
  if (tid == 0) tc::mbar_init(&mbar, 1);
  if (warp == 0) tc::tmem_alloc(&tmem_base, ncols);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tmem_base;
  const uint32_t idesc = tc::idesc_bf16_f32(128, np);
  const bool a_vec = a.sak == 1 && (a.sam % 8) == 0 && (((uintptr_t)a.A) & 15) == 0;
  const bool b_vec = a.sbk == 1 && (a.sbn % 8) == 0 && (((uintptr_t)a.B) & 15) == 0;
  bool ok = true, issued = false;
  uint32_t phase = 0;
  for (int k0 = kbeg; k0 < kend && ok; k0 += KC) {
    const int kc = min(KC, kend - k0);
    // ---- stage A (128 x kc) and B (np x kc)
    if (a_vec && (a.K % 8) == 0) {
      for (int i = tid; i < 128 * (kc >> 3); i += 128) {
        const int r = i / (kc >> 3), q = i % (kc >> 3);
        const long m = m0 + r;
        const int k = k0 + 8 * q;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (m < a.M && k < a.K) v = __ldg(reinterpret_cast<const uint4 *>(a.A + m * a.sam + k));
        *reinterpret_cast<uint4 *>(sA + tc::core_off(r, 8 * q, kc)) = v;
      }
    } else {
      for (int i = tid; i < 128 * kc; i += 128) {
        int r, kk;
        if (a.sam == 1) { r = i % 128; kk = i / 128; } else { r = i / kc; kk = i % kc; }
        const long m = m0 + r;
        const int k = k0 + kk;
        __nv_bfloat16 v = __float2bfloat16(0.0f);
        if (m < a.M && k < a.K) v = a.A[m * a.sam + (long)k * a.sak];
        sA[tc::core_off(r, kk, kc)] = v;
      }
    }
    if (b_vec && (a.K % 8) == 0) {
      for (int i = tid; i < np * (kc >> 3); i += 128) {
        const int r = i / (kc >> 3), q = i % (kc >> 3);
        const int k = k0 + 8 * q;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (r < a.N && k < a.K) v = __ldg(reinterpret_cast<const uint4 *>(a.B + (long)r * a.sbn + k));
        *reinterpret_cast<uint4 *>(sB + tc::core_off(r, 8 * q, kc)) = v;
      }
    } else {
      for (int i = tid; i < np * kc; i += 128) {
        int r, kk;
        if (a.sbn == 1) { r = i % np; kk = i / np; } else { r = i / kc; kk = i % kc; }
        const int k = k0 + kk;
        __nv_bfloat16 v = __float2bfloat16(0.0f);
        if (r < a.N && k < a.K) v = a.B[(long)r * a.sbn + (long)k * a.sbk];
        sB[tc::core_off(r, kk, kc)] = v;
      }
    }
    tc::fence_async_smem();
    __syncthreads();
    // ---- MMAs of the chunk
    if (tid == 0) {
      tc::fence_after();
      const uint32_t sbo = (uint32_t)(kc >> 3) * 128u;
      for (int ks = 0; ks < kc / 16; ++ks) {
        const uint64_t da = tc::desc(tc::smem_u32(sA) + ks * 256, 128u, sbo);
        const uint64_t db = tc::desc(tc::smem_u32(sB) + ks * 256, 128u, sbo);
        tc::mma_bf16(tmem, da, db, idesc, issued || ks > 0);
      }
      issued = true;
      tc::commit(&mbar);
    }
    issued = true;
    // block-uniform: every warp must take the same path into tcgen05.ld
    ok = __syncthreads_and(tc::mbar_wait(&mbar, phase, WAIT_ITERS) ? 1 : 0) != 0;
    phase ^= 1u;
    tc::fence_after();
  }
  if (!ok) {
    if (tid == 0) atomicExch(a.err, 1);
    tc::mbar_wait(&mbar, phase ^ 1u, WAIT_ITERS);     // let MMAs in flight finish before freeing TMEM
  }
  // ---- epilogue
  if (ok) {
    const long m = m0 + warp * 32 + lane;
    for (int c0 = 0; c0 < np; c0 += 16) {
      float v[16];
      if (issued) tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      else
        for (int j = 0; j < 16; ++j) v[j] = 0.0f;
      if (m >= a.M) continue;
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int n = c0 + j;
        if (n >= a.N) continue;
        float x = v[j];
        switch (a.epi) {
          case EPI_STORE:
            a.C[(long)blockIdx.y * a.M * a.ldc + m * a.ldc + n] = x;
            break;
          case EPI_BIAS_GELU: {
            const float z = x + a.bias[n];
            if (a.Zout) a.Zout[m * a.ldz + n] = z;
            a.H[m * a.ldh + n] = __float2bfloat16(gelu(z));
            break;
          }
          case EPI_BIAS:
            a.C[m * a.ldc + n] = x + a.bias[n];
            break;
          default: {  // EPI_DGELU
            const float dz = x * dgelu(a.Zin[m * a.ldz + n]);
            a.H[m * a.ldh + n] = __float2bfloat16(dz);
            if (a.C) a.C[m * a.ldc + n] = dz;
            break;
          }
        }
      }
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

// ---------------------------------------------------------------------------
// Fused inference of the surrogate's MLP shape (16 -> 256 -> 256 -> 256 ->
// n_out <= 16, GELU): one persistent CTA per SM walks 128-row tiles.  Per
// tile the 128 x 256 FP32 accumulators of consecutive layers alternate
// between the two halves of TMEM (columns 0-255 and 256-511), the BF16
// activations sit in shared memory (64 KB, K-major core matrices), W1 and
// the output layer stay resident in shared memory, and W2 / W3 stream from
// L2 as eight 32 KB K-chunks (pre-packed in the core-matrix layout) through
// a four-stage ring filled by bulk asynchronous copies.  Thread 0 issues the
// copies and the tcgen05.mma; all 16 warps run the epilogues (tcgen05.ld,
// bias, GELU, BF16 pack into the activation tile) in two halves of 128
// columns: the MMAs of the next layer's first two K-chunks (the first
// half's activations) run while the warps form the second half.
constexpr int FZ_NST = 4;                               // weight ring stages (3: 5.14, 4: 4.98 ms on 8.4 M rows)
constexpr int FZ_THREADS = 512;                         // 16 warps: 4 row groups x 4 column quarters
constexpr uint32_t FZ_CHUNK_BYTES = 256 * 64 * 2;       // one K-chunk of W2 / W3
constexpr int FZ_OFF_H = 0, FZ_OFF_STAGE = 65536, FZ_OFF_W1 = FZ_OFF_STAGE + FZ_NST * 32768;
constexpr int FZ_OFF_W4 = FZ_OFF_W1 + 8192, FZ_OFF_X = FZ_OFF_W4 + 8192, FZ_OFF_B = FZ_OFF_X + 4096;
constexpr int FZ_SMEM = FZ_OFF_B + (3 * 256 + 16) * 4;

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b)
{
  const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t *>(&v);
}

// Bias + GELU of 32 accumulator columns (from cb0) of one row into the
// activation tile.  In an epilogue half h, warp w holds TMEM lanes
// 32 (w % 4) .. + 31 (its rows) and the columns 128 h + 32 (w / 4) .. + 31;
// the load of the second half is in flight while the first half's GELU runs
// (the MUFU tanh is the epilogue's bound); the biases are read four at a
// time (the same address for the whole warp).
__device__ __forceinline__ void fz_gelu_half(const uint32_t r[32], const float *bias, int cb0, int row,
                                             __nv_bfloat16 *sH)
{
#pragma unroll
  for (int g = 0; g < 4; ++g) {
    const int cb = cb0 + 8 * g;
    const float4 b0 = *reinterpret_cast<const float4 *>(bias + cb);
    const float4 b1 = *reinterpret_cast<const float4 *>(bias + cb + 4);
    const float bb[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
    uint32_t w[4];
#pragma unroll
    for (int j = 0; j < 4; ++j)
      w[j] = pack_bf16x2(gelu(__uint_as_float(r[8 * g + 2 * j]) + bb[2 * j]),
                         gelu(__uint_as_float(r[8 * g + 2 * j + 1]) + bb[2 * j + 1]));
    *reinterpret_cast<uint4 *>(sH + tc::core_off(row, cb, 256)) = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

__global__ void __launch_bounds__(FZ_THREADS, 1) mlp_fused_kernel(const MlpFusedArgs a)
{
  extern __shared__ __align__(1024) unsigned char smem[];
  __nv_bfloat16 *sH = reinterpret_cast<__nv_bfloat16 *>(smem + FZ_OFF_H);
  __nv_bfloat16 *sW1 = reinterpret_cast<__nv_bfloat16 *>(smem + FZ_OFF_W1);
  __nv_bfloat16 *sW4 = reinterpret_cast<__nv_bfloat16 *>(smem + FZ_OFF_W4);
  __nv_bfloat16 *sX = reinterpret_cast<__nv_bfloat16 *>(smem + FZ_OFF_X);
  float *sB = reinterpret_cast<float *>(smem + FZ_OFF_B);
  __shared__ __align__(8) uint64_t bar_mma, bar_full[FZ_NST], bar_free[FZ_NST];
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x, warp = tid >> 5;
  const long ntiles = (a.n + 127) / 128;
  const long my_tiles = blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  const long total_chunks = 8 * my_tiles;
  // resident operands: W1 (256 x 16), output layer (16 x 256), biases
  for (int i = tid; i < 4096 / 8; i += FZ_THREADS) {
    reinterpret_cast<uint4 *>(sW1)[i] = __ldg(reinterpret_cast<const uint4 *>(a.w1) + i);
    reinterpret_cast<uint4 *>(sW4)[i] = __ldg(reinterpret_cast<const uint4 *>(a.w4) + i);
  }
  for (int i = tid; i < 256; i += FZ_THREADS) {
    sB[i] = a.b1[i];
    sB[256 + i] = a.b2[i];
    sB[512 + i] = a.b3[i];
  }
  if (tid < 16) sB[768 + tid] = tid < a.n_out ? a.b4[tid] : 0.0f;
  if (tid == 0) {
    tc::mbar_init(&bar_mma, 1);
    for (int s = 0; s < FZ_NST; ++s) {
      tc::mbar_init(&bar_full[s], 1);
      tc::mbar_init(&bar_free[s], 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tc::tmem_alloc(&tmem_base, 512);
  tc::fence_async_smem();
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tmem_base;
  const uint32_t id256 = tc::idesc_bf16_f32(128, 256), id16 = tc::idesc_bf16_f32(128, 16);
  const uint32_t aH = tc::smem_u32(sH), aX = tc::smem_u32(sX), aW1 = tc::smem_u32(sW1), aW4 = tc::smem_u32(sW4);
  long issued = 0, consumed = 0;       // weight chunks (thread 0's bookkeeping)
  uint32_t mma_phase = 0;
  bool ok = true;
  // chunk g of the stream: W2 chunks 0..3, then W3 chunks 0..3, per tile
  auto issue = [&](long g) -> bool {
    const int s = (int)(g % FZ_NST);
    if (g >= FZ_NST && !tc::mbar_wait(&bar_free[s], (uint32_t)((g / FZ_NST - 1) & 1), WAIT_ITERS)) return false;
    const int j = (int)(g % 8);
    const __nv_bfloat16 *src = (j < 4 ? a.w2 : a.w3) + (long)(j & 3) * (256 * 64);
    tc::mbar_expect_tx(&bar_full[s], FZ_CHUNK_BYTES);
    tc::bulk_g2s(smem + FZ_OFF_STAGE + s * 32768, src, FZ_CHUNK_BYTES, &bar_full[s]);
    ++issued;
    return true;
  };
  if (tid == 0)
    for (long g = 0; g < FZ_NST - 1 && g < total_chunks && ok; ++g) ok = issue(g);
  // Accumulators: the layers alternate between TMEM columns 0-255 (A) and
  // 256-511 (B), so that the MMAs of a layer's first K half (activation
  // columns 0-127, written by the first half of the previous epilogue) run
  // while the warps form the second half of that epilogue.
  const uint32_t tA = tmem, tB = tmem + 256u;
  const int lane = tid & 31, q4 = warp & 3, row = 32 * q4 + lane;
  auto ld_half = [&](uint32_t tacc, int h, uint32_t r[32]) {
    tc::tmem_ld32_nowait(tacc + ((uint32_t)(32 * q4) << 16) + (uint32_t)(128 * h + 32 * (warp >> 2)), r);
  };
  auto gelu_half = [&](const uint32_t r[32], const float *bias, int h) {
    fz_gelu_half(r, bias, 128 * h + 32 * (warp >> 2), row, sH);
  };
  auto sync_async = [&]() {     // activation writes visible to the tensor core; TMEM accesses ordered
    tc::fence_async_smem();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
  };
  long n_commit = 0;            // commits to bar_mma (thread 0)
  bool uncommitted = false;     // MMAs issued after the last commit to bar_mma (thread 0)
  // thread 0: the MMAs of K-chunks c0, c0 + 1 of a hidden layer into tacc
  auto mma_chunks = [&](uint32_t tacc, int c0) -> bool {
    for (int c = c0; c < c0 + 2; ++c) {
      const long g = consumed;
      const int s = (int)(g % FZ_NST);
      if (!tc::mbar_wait(&bar_full[s], (uint32_t)((g / FZ_NST) & 1), WAIT_ITERS)) return false;
      tc::fence_after();
      const uint32_t aS = tc::smem_u32(smem + FZ_OFF_STAGE + s * 32768);
#pragma unroll
      for (int j = 0; j < 4; ++j)
        tc::mma_bf16(tacc, tc::desc(aH + (uint32_t)(c * 8 + 2 * j) * 128u, 128u, 4096u),
                     tc::desc(aS + (uint32_t)(2 * j) * 128u, 128u, 1024u), id256, c > 0 || j > 0);
      uncommitted = true;
      tc::commit(&bar_free[s]);
      ++consumed;
      const long gn = g + FZ_NST - 1;
      if (gn < total_chunks && gn >= issued && !issue(gn)) return false;
    }
    return true;
  };
  auto commit_mma = [&]() {
    tc::commit(&bar_mma);
    ++n_commit;
    uncommitted = false;
  };
  // all threads: wait for the last commit to bar_mma
  auto wait_mma = [&]() -> bool {
    ok = __syncthreads_and(ok && tc::mbar_wait(&bar_mma, mma_phase, WAIT_ITERS)) != 0;
    mma_phase ^= 1u;
    tc::fence_after();
    return ok;
  };
  long tile = blockIdx.x;
  for (long it = 0; it < my_tiles; ++it, tile += gridDim.x) {
    const long r0 = tile * 128;
    // ---- input rows -> BF16 tile (threads 0..127, one row each)
    if (tid < 128) {
      const long rw = r0 + tid;
      float x[16];
      if (rw < a.n) {
        const float4 *xp = reinterpret_cast<const float4 *>(a.x + rw * 16);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float4 v = __ldg(xp + q);
          x[4 * q] = v.x; x[4 * q + 1] = v.y; x[4 * q + 2] = v.z; x[4 * q + 3] = v.w;
        }
      } else {
#pragma unroll
        for (int q = 0; q < 16; ++q) x[q] = 0.0f;
      }
      *reinterpret_cast<uint4 *>(sX + tc::core_off(tid, 0, 16)) =
          make_uint4(pack_bf16x2(x[0], x[1]), pack_bf16x2(x[2], x[3]), pack_bf16x2(x[4], x[5]), pack_bf16x2(x[6], x[7]));
      *reinterpret_cast<uint4 *>(sX + tc::core_off(tid, 8, 16)) =
          make_uint4(pack_bf16x2(x[8], x[9]), pack_bf16x2(x[10], x[11]), pack_bf16x2(x[12], x[13]),
                     pack_bf16x2(x[14], x[15]));
    }
    sync_async();
    // ---- layer 1: K = 16, one MMA into A
    if (tid == 0) {
      tc::mma_bf16(tA, tc::desc(aX, 128u, 256u), tc::desc(aW1, 128u, 256u), id256, false);
      commit_mma();
    }
    if (!wait_mma()) break;
    // ---- layers 2 (into B) and 3 (into A): K = 256 in four chunks; the
    // first two chunks start after the first half of the previous epilogue
    for (int layer = 0; layer < 2 && ok; ++layer) {
      const uint32_t tprev = layer == 0 ? tA : tB, tcur = layer == 0 ? tB : tA;
      const float *bprev = sB + 256 * layer;
      uint32_t rh0[32], rh1[32];
      ld_half(tprev, 0, rh0);
      tc::tmem_wait_ld();
      ld_half(tprev, 1, rh1);                   // in flight during the first half
      gelu_half(rh0, bprev, 0);
      sync_async();
      if (tid == 0) ok = mma_chunks(tcur, 0);
      tc::tmem_wait_ld();
      gelu_half(rh1, bprev, 1);
      sync_async();
      if (tid == 0) {
        if (ok) ok = mma_chunks(tcur, 2);
        commit_mma();
      }
      if (!wait_mma()) break;
    }
    if (!ok) break;
    // ---- epilogue of layer 3 (A), both halves, then the output layer
    // (N = 16, K = 256) into B
    {
      uint32_t rh0[32], rh1[32];
      ld_half(tA, 0, rh0);
      tc::tmem_wait_ld();
      ld_half(tA, 1, rh1);
      gelu_half(rh0, sB + 512, 0);
      tc::tmem_wait_ld();
      gelu_half(rh1, sB + 512, 1);
    }
    sync_async();
    if (tid == 0) {
#pragma unroll
      for (int j = 0; j < 16; ++j)
        tc::mma_bf16(tB, tc::desc(aH + (uint32_t)(2 * j) * 128u, 128u, 4096u),
                     tc::desc(aW4 + (uint32_t)(2 * j) * 128u, 128u, 4096u), id16, j > 0);
      commit_mma();
    }
    if (!wait_mma()) break;
    if (warp < 4) {                  // output columns 0..15: the first column quarter's warps
      float v[16];
      tc::tmem_ld16(tB + ((uint32_t)(warp * 32) << 16), v);
      const long rw = r0 + tid;
      if (rw < a.n) {
#pragma unroll
        for (int j = 0; j < 16; ++j)
          if (j < a.n_out) a.y[rw * a.n_out + j] = v[j] + sB[768 + j];
      }
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
  }
  if (!ok) {
    if (tid == 0) atomicExch(a.err, 1);
    // let the tensor core and the copies in flight finish before the
    // shared memory and TMEM are released: one more commit covers every MMA
    // issued so far; its phase is the parity of the commit count
    if (tid == 0) {
      if (uncommitted) commit_mma();
      if (n_commit > 0) tc::mbar_wait(&bar_mma, (uint32_t)((n_commit - 1) & 1), WAIT_ITERS);
      for (long g = consumed; g < issued; ++g)
        tc::mbar_wait(&bar_full[g % FZ_NST], (uint32_t)((g / FZ_NST) & 1), WAIT_ITERS);
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 512);
}

// FP32 master weights -> the fused kernel's BF16 layouts: W1 [256][16] and
// the output layer [16][256] (rows >= n_out zero) as K-major core-matrix
// tiles, W2 / W3 [256][256] as four K-chunks of 256 x 64 each.
__global__ void mlp_pack_kernel(const float *__restrict__ p, long w1, long w2, long w3, long w4, int n_out,
                                __nv_bfloat16 *__restrict__ out)
{
  const long total = 4096 + 65536 + 65536 + 4096;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    float v;
    long dst;
    if (i < 4096) {                                   // W1: n = i / 16, k = i % 16
      const int n = (int)(i / 16), k = (int)(i % 16);
      v = p[w1 + i];
      dst = tc::core_off(n, k, 16);
    } else if (i < 4096 + 131072) {                   // W2 / W3: n, k in 256 x 256
      const long j = i - 4096;
      const int l = (int)(j / 65536);
      const int n = (int)((j % 65536) / 256), k = (int)(j % 256);
      v = p[(l == 0 ? w2 : w3) + (long)n * 256 + k];
      dst = 4096 + (long)l * 65536 + (long)(k / 64) * (256 * 64) + tc::core_off(n, k % 64, 64);
    } else {                                          // output layer: n < 16, k < 256
      const long j = i - 4096 - 131072;
      const int n = (int)(j / 256), k = (int)(j % 256);
      v = n < n_out ? p[w4 + (long)n * 256 + k] : 0.0f;
      dst = 4096 + 131072 + tc::core_off(n, k, 256);
    }
    out[dst] = __float2bfloat16(v);
  }
}

// Sum of the split-K partials in a fixed order: out[i] = sum_s part[s * n + i].
__global__ void sum_splits_kernel(const float *__restrict__ part, float *__restrict__ out, long n, int splits)
{
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    float s = 0.0f;
    for (int j = 0; j < splits; ++j) s += part[(long)j * n + i];
    out[i] = s;
  }
}

// Column sums (bias gradients): out[n] = sum_m x[m * ld + n], fixed order.
__global__ void col_sum_kernel(const float *__restrict__ x, float *__restrict__ out, int rows, int cols, long ld)
{
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= cols) return;
  float s = 0.0f;
  for (int m = 0; m < rows; ++m) s += x[(long)m * ld + n];
  out[n] = s;
}

// Loss of the surrogate head: per rate r, y[2r] is the logit of "the rate is
// nonzero" (binary cross-entropy against act), y[2r+1] the transformed rate
// (squared error against val where the rate is nonzero).  Writes dY
// ([rows][16], mean over the batch) in bf16 for the GEMMs and in f32 for the
// output-bias gradient, and accumulates the loss.
__global__ void surrogate_loss_kernel(const float *__restrict__ y, const float *__restrict__ tgt, int rows, int nrates,
                                      __nv_bfloat16 *__restrict__ dy, float *__restrict__ dyf, float *__restrict__ loss)
{
  __shared__ float red[128];
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.0f;
  if (m < rows) {
    const float inv = 1.0f / (float)rows;
    for (int r = 0; r < nrates; ++r) {
      const float logit = y[(long)m * 16 + 2 * r], pred = y[(long)m * 16 + 2 * r + 1];
      const float act = tgt[(long)m * 16 + 2 * r], val = tgt[(long)m * 16 + 2 * r + 1];
      const float p = 1.0f / (1.0f + expf(-logit));
      l += -(act * logf(fmaxf(p, 1e-12f)) + (1.0f - act) * logf(fmaxf(1.0f - p, 1e-12f)));
      const float e = act > 0.5f ? pred - val : 0.0f;
      l += e * e;
      const float g0 = (p - act) * inv, g1 = 2.0f * e * inv;
      dy[(long)m * 16 + 2 * r] = __float2bfloat16(g0);
      dy[(long)m * 16 + 2 * r + 1] = __float2bfloat16(g1);
      dyf[(long)m * 16 + 2 * r] = g0;
      dyf[(long)m * 16 + 2 * r + 1] = g1;
    }
    for (int j = 2 * nrates; j < 16; ++j) {
      dy[(long)m * 16 + j] = __float2bfloat16(0.0f);
      dyf[(long)m * 16 + j] = 0.0f;
    }
  }
  red[threadIdx.x] = l;
  __syncthreads();
  for (int s = 64; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(loss, red[0] / (float)rows);
}

// Adam on FP32 master weights; refreshes the BF16 copy used by the GEMMs.
__global__ void adam_kernel(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m1,
                            float *__restrict__ m2, __nv_bfloat16 *__restrict__ w16, long n, float lr, float b1,
                            float b2, float eps, float c1, float c2)
{
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float a = b1 * m1[i] + (1.0f - b1) * gi, b = b2 * m2[i] + (1.0f - b2) * gi * gi;
    m1[i] = a;
    m2[i] = b;
    const float wi = w[i] - lr * (a * c1) / (sqrtf(b * c2) + eps);
    w[i] = wi;
    if (w16) w16[i] = __float2bfloat16(wi);
  }
}

__global__ void to_bf16_kernel(const float *__restrict__ x, __nv_bfloat16 *__restrict__ y, long n)
{
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    y[i] = __float2bfloat16(x[i]);
}

}  // namespace

// Operand staging needs (128 + 256) x KC BF16 = 48 KB; the request is
// padded to 96 KB so that at most two CTAs (2 x 256 TMEM columns, the SM's
// 512) are resident per SM and no tcgen05.alloc has to wait for columns.
size_t tc_gemm_smem_bytes() { return (size_t)96 * 1024; }

cudaError_t launch_tc_gemm(const TcGemmArgs &a, cudaStream_t s)
{
  if (a.N < 1 || a.N > 256 || a.M < 1 || a.K < 1 || a.k_split < 1) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)tc_gemm_smem_bytes());
  if (e != cudaSuccess) return e;
  dim3 grid((unsigned)((a.M + 127) / 128), (unsigned)a.k_split);
  tc_gemm_kernel<<<grid, 128, tc_gemm_smem_bytes(), s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_mlp_pack(const float *p, long w1, long w2, long w3, long w4, int n_out, __nv_bfloat16 *out,
                            cudaStream_t s)
{
  mlp_pack_kernel<<<136, 1024, 0, s>>>(p, w1, w2, w3, w4, n_out, out);
  return cudaGetLastError();
}

cudaError_t launch_mlp_fused(const MlpFusedArgs &a, int num_sms, cudaStream_t s)
{
  cudaError_t e = cudaFuncSetAttribute(mlp_fused_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, FZ_SMEM);
  if (e != cudaSuccess) return e;
  const long tiles = (a.n + 127) / 128;
  long blocks = num_sms;
  if (blocks > tiles) blocks = tiles;
  if (blocks < 1) return cudaSuccess;
  mlp_fused_kernel<<<(unsigned)blocks, FZ_THREADS, FZ_SMEM, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_sum_splits(const float *part, float *out, long n, int splits, cudaStream_t s)
{
  long blocks = (n + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  sum_splits_kernel<<<(unsigned)blocks, 256, 0, s>>>(part, out, n, splits);
  return cudaGetLastError();
}

cudaError_t launch_col_sum(const float *x, float *out, int rows, int cols, long ld, cudaStream_t s)
{
  col_sum_kernel<<<(unsigned)((cols + 127) / 128), 128, 0, s>>>(x, out, rows, cols, ld);
  return cudaGetLastError();
}

cudaError_t launch_surrogate_loss(const float *y, const float *tgt, int rows, int nrates, __nv_bfloat16 *dy,
                                  float *dyf, float *loss, cudaStream_t s)
{
  surrogate_loss_kernel<<<(unsigned)((rows + 127) / 128), 128, 0, s>>>(y, tgt, rows, nrates, dy, dyf, loss);
  return cudaGetLastError();
}

cudaError_t launch_adam(float *w, const float *g, float *m1, float *m2, __nv_bfloat16 *w16, long n, float lr, float b1,
                        float b2, float eps, int step, cudaStream_t s)
{
  const float c1 = 1.0f / (1.0f - powf(b1, (float)step)), c2 = 1.0f / (1.0f - powf(b2, (float)step));
  long blocks = (n + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  adam_kernel<<<(unsigned)blocks, 256, 0, s>>>(w, g, m1, m2, w16, n, lr, b1, b2, eps, c1, c2);
  return cudaGetLastError();
}

cudaError_t launch_to_bf16(const float *x, __nv_bfloat16 *y, long n, cudaStream_t s)
{
  long blocks = (n + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  to_bf16_kernel<<<(unsigned)blocks, 256, 0, s>>>(x, y, n);
  return cudaGetLastError();
}
