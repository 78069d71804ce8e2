// rain_ice.cu — ICE4 one-moment microphysics step, one grid point per thread.
//
// Restates, per grid point, PHYEX RAIN_ICE (PHYEX-IAL_CY50T1/micro/
// rain_ice.F90:334-652 and its disabled tail :758-790), ICE4_PACK
// (mode_ice4_pack.F90), ICE4_STEPPING (mode_ice4_stepping.F90:139-518),
// ICE4_TENDENCIES (mode_ice4_tendencies.F90:150-717) and the processes it
// calls (nucleation, rrhong, rimltc, compute_pdf, slow, warm, fast_rs,
// fast_rg, fast_ri), then the total tendencies and ICE4_CORRECT_NEGATIVITIES.
//
// GB300 mapping:
//  * the ICE4 collection-kernel tables (GAMINC_RIM1/2/4, KER_RACCSS/RACCS/
//    SACCRG, KER_RDRYG, KER_SDRYG; 78,720 B FP64) are staged once per block
//    in shared memory; blocks are persistent (one of 512 threads per SM) and
//    pull 1-point-per-thread chunks from a global counter, which balances the
//    data-dependent number of sub-steps across SMs; the chunk barrier keeps
//    the warps of a block in step through the (large) point code;
//  * every per-point quantity that is fixed over the sub-steps (log rho and
//    the rho powers) is computed once; real powers are fm::fexp(a*log x) with the
//    logarithms of the slope parameters shared by all processes;
//  * points are processed in regime order: a first kernel sorts each tile of
//    131,072 points by which hydrometeors are present, whether T < TT and
//    whether the air is supersaturated over ice (the masks that decide which
//    process branches and how many sub-steps a point takes), so a warp's
//    lanes take the same branches instead of the union of all regimes; the
//    tile keeps the gathered accesses within a window of 1 MB per field
//    (tiles of 32,768 / 65,536 / 131,072 points: rain_ice 171.6 / 170.6 /
//    170.2 ms at 1024x1024x90, fewer part-filled warps at the regime
//    boundaries).  Results do not depend on the order;
//  * with a PRFR option a column kernel first forms the precipitation
//    fraction the sub-stepping starts from (prfr_column);
//  * the only cross-point coupling of the Fortran stepping (PRREVAV taken
//    after the last pass of the call, mode_ice4_stepping.F90:514-516) is
//    kept with a per-point pass key and a warp-reduced atomicMax, resolved by
//    a second small kernel.
#include "ice3gb_device.cuh"
#include "ice3gb_kernels.h"
#include "rain_ice_kernel.cuh"

namespace {
using namespace ice3pt;
using namespace ice3ri;

// OCND2: level heights and droplet concentrations, one thread per column.
__global__ void rain_ice_ocnd2_column_kernel(const __grid_constant__ Cst c, const __grid_constant__ RainIceArgs a)
{
  const long col = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (col < a.nij) ocnd2_column(c, a.f, a.nij, a.nk, col, a.ocs, a.ocs + (long)a.nij * a.nk);
}

template <bool H>
__global__ void rain_ice_prfr_kernel(const __grid_constant__ Cst c, const __grid_constant__ RainIceArgs a)
{
  const long col = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (col < a.nij) prfr_column<H>(c, a.f, a.nij, a.nk, col);
}

// Processing order: per tile of ORDER_TILE points, a counting sort by regime
// (bit 0..4: cloud, rain, ice, snow, graupel above XRTMIN; bit 5: T < TT;
// bit 6: supersaturation over ice, from an FP32 estimate of e_si(T)).  The
// last bit decides the costly branches that few points of a regime take: the
// nucleation (ice4_nucleation.func.h:40-89) and the Bergeron process
// (mode_ice4_fast_ri.F90:60-75), exp / log / divisions that a warp otherwise
// runs for one or two of its lanes.  Warp-aggregated shared-memory atomics
// give each point its slot in the tile; the order inside a regime follows the
// atomics and does not matter.  The tile's keys (one byte per point) sit in
// dynamic shared memory.
#ifndef ICE3GB_ORDER_TILE
#define ICE3GB_ORDER_TILE 131072
#endif
constexpr int ORDER_TILE = ICE3GB_ORDER_TILE, ORDER_THREADS = 1024, ORDER_BINS = 128;
static_assert(ORDER_BINS % 32 == 0 && ORDER_BINS <= 256, "bins per lane in the scan; one-byte keys");

// rv > e_si (EPSILO + rv) / p, i.e. ice supersaturation, in FP32 (a sort key
// only: the rounding of the estimate does not reach the results)
__device__ __forceinline__ bool ice_supersat_est(const Cst &c, double t, double p, double rv)
{
  const float tf = (float)t, pf = (float)p, rvf = (float)rv;
  const float esi = expf((float)c.ALPI - (float)c.BETAI / tf - (float)c.GAMI * logf(tf));
  return rvf * pf > esi * ((float)c.EPSILO + rvf);
}

__global__ void __launch_bounds__(ORDER_THREADS) rain_ice_order_kernel(const __grid_constant__ Cst c,
                                                                       const __grid_constant__ RainIceArgs a)
{
  extern __shared__ unsigned char key[];   // [ORDER_TILE]
  __shared__ unsigned int cnt[ORDER_BINS];
  const Ice3gbRainIceFields &f = a.f;
  const long n = (long)a.nij * a.nk;
  const long base = (long)blockIdx.x * ORDER_TILE;
  const int m = (int)((n - base) < ORDER_TILE ? (n - base) : ORDER_TILE);
  const unsigned lane = threadIdx.x & 31u;
  if (threadIdx.x < ORDER_BINS) cnt[threadIdx.x] = 0u;
  __syncthreads();
  for (int i0 = 0; i0 < m; i0 += ORDER_THREADS) {       // uniform trip count: full warps in the collectives
    const int i = i0 + (int)threadIdx.x;
    unsigned k = 0xffu;
    if (i < m) {
      const long p = base + i;
      const double t = ld1(f.tht, p) * ld1(f.exn, p);
      k = (gtp(ld1(f.rct, p), c.C_RTMIN) ? 1u : 0u) | (gtp(ld1(f.rrt, p), c.R_RTMIN) ? 2u : 0u) |
          (gtp(ld1(f.rit, p), c.I_RTMIN) ? 4u : 0u) | (gtp(ld1(f.rst, p), c.S_RTMIN) ? 8u : 0u) |
          (gtp(ld1(f.rgt, p), c.G_RTMIN) ? 16u : 0u) | (ltp(t, c.TT) ? 32u : 0u) |
          (ice_supersat_est(c, t, ld1(f.pabs, p), ld1(f.rvt, p)) ? 64u : 0u);
      key[i] = (unsigned char)k;
    }
    const unsigned peers = __match_any_sync(0xffffffffu, k);
    if (k != 0xffu && lane == (unsigned)(__ffs(peers) - 1)) atomicAdd(&cnt[k], (unsigned)__popc(peers));
  }
  __syncthreads();
  if (threadIdx.x < 32) {                               // exclusive scan of the counts, BPL per lane
    constexpr int BPL = ORDER_BINS / 32;
    unsigned own[BPL], s = 0u;
#pragma unroll
    for (int j = 0; j < BPL; ++j) { own[j] = cnt[BPL * lane + j]; s += own[j]; }
    const unsigned tot = s;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const unsigned t = __shfl_up_sync(0xffffffffu, s, d);
      if (lane >= (unsigned)d) s += t;
    }
    unsigned excl = s - tot;
#pragma unroll
    for (int j = 0; j < BPL; ++j) { cnt[BPL * lane + j] = excl; excl += own[j]; }
  }
  __syncthreads();
  for (int i0 = 0; i0 < m; i0 += ORDER_THREADS) {
    const int i = i0 + (int)threadIdx.x;
    const unsigned k = i < m ? (unsigned)key[i] : 0xffu;
    const unsigned peers = __match_any_sync(0xffffffffu, k);
    const unsigned leader = (unsigned)(__ffs(peers) - 1);
    unsigned first = 0u;
    if (k != 0xffu && lane == leader) first = atomicAdd(&cnt[k], (unsigned)__popc(peers));
    first = __shfl_sync(0xffffffffu, first, (int)leader);
    if (k != 0xffu) {
      const unsigned rank = (unsigned)__popc(peers & ((1u << lane) - 1u));
      a.order[base + first + rank] = (unsigned int)(base + i);
    }
  }
}

// PRREVAV after the last pass of the call: zero evap3d on micro points that
// were not active in that pass (mode_ice4_stepping.F90:514-516).
__global__ void rain_ice_evap_fixup_kernel(double *__restrict__ evap3d, const unsigned int *__restrict__ keys,
                                           const unsigned int *__restrict__ key_max, long n)
{
  const unsigned int kmax = *key_max;
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < n; p += (long)gridDim.x * blockDim.x) {
    const unsigned int k = keys[p];
    if (k != 0u && k != kmax) evap3d[p] = 0.0;
  }
}

}  // namespace

size_t rain_ice_smem_bytes() { return sizeof(double) * LUT_N; }

cudaError_t launch_rain_ice_points(const Cst &c, const RainIceArgs &a, int num_sms, cudaStream_t s)
{
  const bool subg = (int)c.SUBG_RC_RR_ACCR != 0 || (int)c.SUBG_RR_EVAP != 0;
  const bool hail = (int)c.NRR == 7;
  if (c.MRSTEP != 0.0 || c.TSTEP_TS != 0.0) return launch_rain_ice_points_ts(c, a, num_sms, s);
  void (*kern)(const Cst, const RainIceArgs) =
      c.OCND2 != 0.0
          ? (hail ? (subg ? rain_ice_points_kernel<true, true, true> : rain_ice_points_kernel<false, true, true>)
                  : (subg ? rain_ice_points_kernel<true, false, true> : rain_ice_points_kernel<false, false, true>))
      : hail ? (subg ? rain_ice_points_kernel<true, true> : rain_ice_points_kernel<false, true>)
             : (subg ? rain_ice_points_kernel<true, false> : rain_ice_points_kernel<false, false>);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rain_ice_smem_bytes());
  if (e != cudaSuccess) return e;
  const long n = (long)a.nij * a.nk;
  long chunks = (n + RI_THREADS - 1) / RI_THREADS;
  long blocks = (long)num_sms * RI_BLOCKS_PER_SM;
  if (blocks > chunks) blocks = chunks;
  if (blocks < 1) blocks = 1;
  kern<<<(unsigned)blocks, RI_THREADS, rain_ice_smem_bytes(), s>>>(c, a);
  return cudaGetLastError();
}

cudaError_t launch_rain_ice_ocnd2_columns(const Cst &c, const RainIceArgs &a, cudaStream_t s)
{
  rain_ice_ocnd2_column_kernel<<<(unsigned)((a.nij + 127) / 128), 128, 0, s>>>(c, a);
  return cudaGetLastError();
}

cudaError_t launch_rain_ice_prfr(const Cst &c, const RainIceArgs &a, cudaStream_t s)
{
  if ((int)c.NRR == 7) rain_ice_prfr_kernel<true><<<(unsigned)((a.nij + 127) / 128), 128, 0, s>>>(c, a);
  else rain_ice_prfr_kernel<false><<<(unsigned)((a.nij + 127) / 128), 128, 0, s>>>(c, a);
  return cudaGetLastError();
}

cudaError_t launch_rain_ice_order(const Cst &c, const RainIceArgs &a, cudaStream_t s)
{
  const long n = (long)a.nij * a.nk;
  const long tiles = (n + ORDER_TILE - 1) / ORDER_TILE;
  cudaError_t e = cudaFuncSetAttribute(rain_ice_order_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, ORDER_TILE);
  if (e != cudaSuccess) return e;
  rain_ice_order_kernel<<<(unsigned)tiles, ORDER_THREADS, ORDER_TILE, s>>>(c, a);
  return cudaGetLastError();
}

cudaError_t launch_rain_ice_evap_fixup(const RainIceArgs &a, cudaStream_t s)
{
  const long n = (long)a.nij * a.nk;
  long blocks = (n + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  rain_ice_evap_fixup_kernel<<<(unsigned)blocks, 256, 0, s>>>(a.f.evap3d, a.scr.keys, a.scr.key_max, n);
  return cudaGetLastError();
}
