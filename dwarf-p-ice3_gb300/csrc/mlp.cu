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
constexpr long WAIT_ITERS = 1L << 26;  // bounded mbarrier wait (~seconds)

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float dgelu(float z)
{
  return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
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
