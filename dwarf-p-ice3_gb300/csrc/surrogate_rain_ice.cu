// surrogate_rain_ice.cu — the learned surrogate of the ICE4_SLOW rates in
// the rain_ice step.
//
// surrogate_sample_kernel: per grid point, the 16 features of a micro point
//   at its first hard pass (and, for training, the plain kernel's slow rates
//   as targets); with a normalisation it standardises the features and
//   checks them against the training envelope.  Accepted points get a row of
//   a compacted [rows][16] matrix (warp-aggregated atomics; a point's row
//   number does not change its result), the others row -1.
// rain_ice_surrogate_kernel: the rain_ice point loop of rain_ice.cu where a
//   point with a row takes its first hard pass's slow rates from the
//   network's output row, then passes a fix-up check (finite sources,
//   non-negative hydrometeor sources, vapour not driven below its input or
//   zero, total water conserved to 1e-12 of the water sources); a point that
//   fails it is recomputed by the plain path in the same launch, as are
//   points without a row.
#include "ice3gb_device.cuh"
#include "ice3gb_kernels.h"
#include "surrogate_point.cuh"

// One block of RI_THREADS per SM, as the plain rain_ice kernel.
#ifndef RI_BLOCKS_PER_SM
#define RI_BLOCKS_PER_SM 1
#endif

namespace {
using namespace ice3pt;
using namespace ice3sur;

constexpr int SAMPLE_THREADS = 256;

__device__ __forceinline__ void warp_add(unsigned long long *ctr, bool pred)
{
  const unsigned m = __ballot_sync(0xffffffffu, pred);
  if ((threadIdx.x & 31) == 0 && m) atomicAdd(ctr, (unsigned long long)__popc(m));
}

// RATES: also the plain slow rates (training targets), which need the
// lookup tables in shared memory; without, only the features.
template <bool RATES>
__global__ void __launch_bounds__(SAMPLE_THREADS) surrogate_sample_kernel(const __grid_constant__ Cst c,
                                                                          const __grid_constant__ SurSampleArgs a)
{
  extern __shared__ double lut[];
  __shared__ Derived dsh;
  if (RATES)
    for (int i = threadIdx.x; i < LUT_N; i += blockDim.x) lut[i] = a.luts[i];
  if (threadIdx.x == 0) make_derived(c, dsh);
  __syncthreads();
  const long n = (long)a.nij * a.nk;
  const unsigned lane = threadIdx.x & 31u;
  __shared__ unsigned wrows[SAMPLE_THREADS / 32];
  __shared__ unsigned long long block_base;
  // uniform trip count: whole warps reach the ballots, whole blocks the barriers
  const long stride = (long)gridDim.x * blockDim.x;
  for (long p0 = (long)blockIdx.x * blockDim.x; p0 < n; p0 += stride) {
    const long p = p0 + threadIdx.x;
    float x[NFEAT];
    double r[NRATE];
    bool micro = false, ok = false;
    if (p < n) micro = sample_point<RATES>(c, dsh, lut, a.f, p, a.dt, x, r);
    float xf[NFEAT];
    if (micro) {
      ok = true;
#pragma unroll
      for (int j = 0; j < NFEAT; ++j) {
        float v = x[j];
        if (a.norm_on) {
          v = (v - a.norm.mean[j]) * a.norm.inv_std[j];
          ok = ok && v >= a.norm.lo[j] && v <= a.norm.hi[j];   // false for NaN
        }
        xf[j] = v;
      }
    }
    // rows handed out per block (one atomic per block: a per-warp atomic on
    // the one counter serialised the kernel at the L2)
    const unsigned m = __ballot_sync(0xffffffffu, ok);
    const unsigned warp = threadIdx.x >> 5;
    if (lane == 0) wrows[warp] = (unsigned)__popc(m);
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned tot = 0;
      for (int w = 0; w < SAMPLE_THREADS / 32; ++w) {
        const unsigned cw = wrows[w];
        wrows[w] = tot;
        tot += cw;
      }
      block_base = tot ? atomicAdd(a.count, (unsigned long long)tot) : 0ull;
    }
    __syncthreads();
    const long row = ok ? (long)(block_base + wrows[warp] + __popc(m & ((1u << lane) - 1u))) : -1;
    __syncthreads();                  // wrows and block_base are rewritten by the next iteration
    const bool kept = ok && row < a.cap;
    if (kept) {
      float4 *fr = reinterpret_cast<float4 *>(a.feat + row * ROW);
#pragma unroll
      for (int j = 0; j < NFEAT; j += 4) fr[j / 4] = make_float4(xf[j], xf[j + 1], xf[j + 2], xf[j + 3]);
      if (RATES) {
        float t[ROW];
        encode_targets(r, t);
        float4 *tr = reinterpret_cast<float4 *>(a.targets + row * ROW);
#pragma unroll
        for (int j = 0; j < ROW; j += 4) tr[j / 4] = make_float4(t[j], t[j + 1], t[j + 2], t[j + 3]);
      }
      if (a.point_of_row) a.point_of_row[row] = (long long)p;
    }
    if (p < n && a.row_of_point) a.row_of_point[p] = kept ? (int)row : -1;
    warp_add(a.stats + 0, micro);
    warp_add(a.stats + 1, micro && !ok);
    warp_add(a.stats + 2, ok && !kept);
  }
}

__device__ __forceinline__ void warp_key_max(unsigned int *key_max, unsigned int key)
{
  const unsigned int m = __reduce_max_sync(0xffffffffu, key);
  if ((threadIdx.x & 31) == 0 && m != 0u) atomicMax(key_max, m);
}

__device__ __forceinline__ bool finite_(double x) { return (fm::bits_(x) & 0x7ff0000000000000LL) != 0x7ff0000000000000LL; }

__global__ void __launch_bounds__(RI_THREADS, RI_BLOCKS_PER_SM)
    rain_ice_surrogate_kernel(const __grid_constant__ Cst c, const __grid_constant__ SurRainIceArgs sa)
{
  extern __shared__ double lut[];
  __shared__ Derived dsh;
  // the in-out fields a point starts from, for the fall-back to the plain
  // path: kept in shared memory rather than in registers across the point
  // code (fewer spills of the large point kernel)
  __shared__ double s_in[8][RI_THREADS];
  __shared__ double s_sur[RI_THREADS][NRATE];          // the decoded learned rates of a thread's point
  const RainIceArgs &a = sa.ri;
  for (int i = threadIdx.x; i < LUT_N; i += blockDim.x) lut[i] = a.luts[i];
  if (threadIdx.x == 0) make_derived(c, dsh);
  __shared__ unsigned int chunk;
  __syncthreads();
  const Ice3gbRainIceFields &f = a.f;
  const long n = (long)a.nij * a.nk;
  const double dt = a.dt;
  bool any_capped = false;
  for (;;) {
    if (threadIdx.x == 0) chunk = atomicAdd(a.scr.chunk_counter, 1u);
    __syncthreads();
    const long base = (long)chunk * blockDim.x;
    __syncthreads();
    if (base >= n) break;
    const long slot = base + threadIdx.x;
    unsigned int key = 0u;
    bool used = false, fell_back = false;
    if (slot < n) {
      const long p = a.order ? (long)__ldg(a.order + slot) : slot;
      const int row = __ldg(sa.row_of_point + p);
      const double *use = nullptr;
      if (row >= 0) {
        decode_rates(sa.y + (long)row * sa.ldy, s_sur[threadIdx.x]);
        use = s_sur[threadIdx.x];
      }
      double *in0 = &s_in[0][threadIdx.x];                        // element k at in0[k * RI_THREADS]
      in0[0 * RI_THREADS] = f.ths[p]; in0[1 * RI_THREADS] = f.rvs[p]; in0[2 * RI_THREADS] = f.rcs[p];
      in0[3 * RI_THREADS] = f.rrs[p]; in0[4 * RI_THREADS] = f.ris[p]; in0[5 * RI_THREADS] = f.rss[p];
      in0[6 * RI_THREADS] = f.rgs[p]; in0[7 * RI_THREADS] = f.cit[p];
      for (int attempt = 0; attempt < 2; ++attempt) {
        bool capped;
        key = rain_ice_point<true>(c, dsh, lut, f, p, dt, a.max_passes, capped, use);
        if (!use) { any_capped |= capped; break; }
        // fix-up check of the surrogate-assisted point
        const double o_th = f.ths[p], o_v = f.rvs[p], o_c = f.rcs[p], o_r = f.rrs[p], o_i = f.ris[p];
        const double o_s = f.rss[p], o_g = f.rgs[p];
        double in[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) in[k] = in0[k * RI_THREADS];
        const double w_in = in[1] + in[2] + in[3] + in[4] + in[5] + in[6];
        const double w_out = o_v + o_c + o_r + o_i + o_s + o_g;
        const double w_abs = fabs(in[1]) + fabs(in[2]) + fabs(in[3]) + fabs(in[4]) + fabs(in[5]) + fabs(in[6]);
        const bool ok = finite_(o_th) && finite_(w_out) && !negd(o_c) && !negd(o_r) && !negd(o_i) && !negd(o_s) &&
                        !negd(o_g) && (!negd(o_v) || o_v >= in[1]) && fabs(w_out - w_in) <= 1e-12 * w_abs;
        if (ok) { used = true; any_capped |= capped; break; }
        // restore the in-out fields and take the plain path
        f.ths[p] = in[0]; f.rvs[p] = in[1]; f.rcs[p] = in[2]; f.rrs[p] = in[3]; f.ris[p] = in[4];
        f.rss[p] = in[5]; f.rgs[p] = in[6]; f.cit[p] = in[7];
        use = nullptr;
        fell_back = true;
      }
      a.scr.keys[p] = key;
    }
    warp_key_max(a.scr.key_max, key);
    warp_add(sa.stats + 3, used);
    warp_add(sa.stats + 4, fell_back);
  }
  if (any_capped) atomicOr(a.scr.status, ICE3GB_DEV_PASS_CAP);
}

size_t lut_smem_bytes() { return sizeof(double) * LUT_N; }

}  // namespace

cudaError_t launch_surrogate_sample(const Cst &c, const SurSampleArgs &a, int num_sms, cudaStream_t s)
{
  const bool rates = a.targets != nullptr;
  const size_t smem = rates ? lut_smem_bytes() : 0;
  cudaError_t e = cudaFuncSetAttribute(surrogate_sample_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)lut_smem_bytes());
  if (e != cudaSuccess) return e;
  const long n = (long)a.nij * a.nk;
  long blocks = (n + SAMPLE_THREADS - 1) / SAMPLE_THREADS;
  const long cap = (long)num_sms * (rates ? 2 : 8);      // resident blocks per SM
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  if (rates) surrogate_sample_kernel<true><<<(unsigned)blocks, SAMPLE_THREADS, smem, s>>>(c, a);
  else surrogate_sample_kernel<false><<<(unsigned)blocks, SAMPLE_THREADS, smem, s>>>(c, a);
  return cudaGetLastError();
}

cudaError_t launch_rain_ice_surrogate(const Cst &c, const SurRainIceArgs &a, int num_sms, cudaStream_t s)
{
  cudaError_t e = cudaFuncSetAttribute(rain_ice_surrogate_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)lut_smem_bytes());
  if (e != cudaSuccess) return e;
  const long n = (long)a.ri.nij * a.ri.nk;
  long chunks = (n + RI_THREADS - 1) / RI_THREADS;
  long blocks = (long)num_sms * RI_BLOCKS_PER_SM;
  if (blocks > chunks) blocks = chunks;
  if (blocks < 1) blocks = 1;
  rain_ice_surrogate_kernel<<<(unsigned)blocks, RI_THREADS, lut_smem_bytes(), s>>>(c, a);
  return cudaGetLastError();
}
