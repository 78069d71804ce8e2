// rain_ice_kernel.cuh — the rain_ice point kernel template (persistent
// blocks, lookup tables staged in shared memory, chunked work counter, pass
// keys for the PRREVAV fixup), instantiated in rain_ice.cu and, for the
// MRSTEP / TSTEP_TS time splitting, in rain_ice_ts.cu (compiled in parallel).
#pragma once

#include "ice3gb_device.cuh"
#include "ice3gb_kernels.h"
#include "rain_ice_point.cuh"

// Resident blocks of rain_ice_points_kernel per SM: one block of RI_THREADS
// = 512 threads (128 registers per thread, one copy of the 78.7 KB lookup
// tables per SM, the rest of the shared memory left to L1 for the register
// spills).  The chunk barrier keeps the 16 warps in step through the (large)
// point code; warps that pull their own chunks drift apart and run it from
// the instruction cache's misses (305 instead of 177 ms at 1024x1024x90).
// 512 x 1 measured 172.5 ms against 176.7 ms for 256 x 2.
#ifndef RI_BLOCKS_PER_SM
#define RI_BLOCKS_PER_SM 1
#endif

namespace ice3ri {
using namespace ice3pt;

__device__ __forceinline__ void warp_key_max(unsigned int *key_max, unsigned int key)
{
  const unsigned int m = __reduce_max_sync(0xffffffffu, key);
  if ((threadIdx.x & 31) == 0 && m != 0u) atomicMax(key_max, m);
}

// SUBG: the subgrid warm-process options (SUBG_RC_RR_ACCR / SUBG_RR_EVAP
// other than NONE); the NONE instantiation carries none of their code.
// H: hail (NRR = 7), the hail kernels read from the global copy of the tables.
// O: OCND2 (NRR = 6, warm options NONE), with a.tw and the column fields a.ocs.
// TS: the MRSTEP / TSTEP_TS time splitting.
template <bool SUBG, bool H = false, bool O = false, bool TS = false>
__global__ void __launch_bounds__(RI_THREADS, RI_BLOCKS_PER_SM) rain_ice_points_kernel(const __grid_constant__ Cst c,
                                                                         const __grid_constant__ RainIceArgs a)
{
  extern __shared__ double lut[];
  __shared__ Derived dsh;
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
    if (slot < n) {
      const long p = a.order ? (long)__ldg(a.order + slot) : slot;
      bool capped;
      if (O)
        key = rain_ice_point<false, SUBG, H, true, TS>(c, dsh, lut, f, p, dt, a.max_passes, capped, nullptr,
                                                           a.luts, a.tw, a.ocs, a.ocs + n);
      else
        key = rain_ice_point<false, SUBG, H, false, TS>(c, dsh, lut, f, p, dt, a.max_passes, capped, nullptr, a.luts);
      any_capped |= capped;
      a.scr.keys[p] = key;
    }
    warp_key_max(a.scr.key_max, key);
  }
  if (any_capped) atomicOr(a.scr.status, ICE3GB_DEV_PASS_CAP);
}

// The precipitation fraction of a call with a PRFR option, one thread per
// column (prfr_column); runs before the point kernel, which starts from it.

}  // namespace ice3ri
