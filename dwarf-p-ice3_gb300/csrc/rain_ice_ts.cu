// rain_ice_ts.cu — the rain_ice point kernel with the MRSTEP / TSTEP_TS time
// splitting of ICE4_STEPPING (mode_ice4_stepping.F90:191-197, :387-453), any
// warm-process option, with or without hail, or with OCND2; a separate
// translation unit so that it compiles beside rain_ice.cu.
#include "ice3gb_device.cuh"
#include "ice3gb_kernels.h"
#include "rain_ice_kernel.cuh"

using namespace ice3ri;

cudaError_t launch_rain_ice_points_ts(const Cst &c, const RainIceArgs &a, int num_sms, cudaStream_t s)
{
  const bool subg = (int)c.SUBG_RC_RR_ACCR != 0 || (int)c.SUBG_RR_EVAP != 0;
  const bool hail = (int)c.NRR == 7;
  void (*kern)(const Cst, const RainIceArgs) =
      c.OCND2 != 0.0
          ? (hail ? (subg ? rain_ice_points_kernel<true, true, true, true> : rain_ice_points_kernel<false, true, true, true>)
                  : (subg ? rain_ice_points_kernel<true, false, true, true> : rain_ice_points_kernel<false, false, true, true>))
      : hail ? (subg ? rain_ice_points_kernel<true, true, false, true> : rain_ice_points_kernel<false, true, false, true>)
             : (subg ? rain_ice_points_kernel<true, false, false, true> : rain_ice_points_kernel<false, false, false, true>);
  const size_t smem = sizeof(double) * LUT_N;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const long n = (long)a.nij * a.nk;
  long chunks = (n + RI_THREADS - 1) / RI_THREADS;
  long blocks = (long)num_sms * RI_BLOCKS_PER_SM;
  if (blocks > chunks) blocks = chunks;
  if (blocks < 1) blocks = 1;
  kern<<<(unsigned)blocks, RI_THREADS, smem, s>>>(c, a);
  return cudaGetLastError();
}
