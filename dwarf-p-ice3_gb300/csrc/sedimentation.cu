// sedimentation.cu — statistical sedimentation, one column sweep per thread.
//
// Restates ICE4_SEDIMENTATION_STAT (PHYEX-IAL_CY50T1/micro/
// mode_ice4_sedimentation_stat.F90:143-229) and the reference JAX
// sedimentation_stat (src/ice3/jax/stencils/sedimentation.py:58-352), the two
// differing in the cloud mean-radius factor and the flux-divergence scaling
// (selected by `fortran`).  A thread owns one column and walks k from the top
// level to the surface with the five species side by side, keeping each
// species' incoming flux F_{k+1} in a register; consecutive threads own
// consecutive columns, so every level access is coalesced.  What the species
// share at a level (rho, dz, rho dz, dt/(rho dz) and log rho, computed only
// when a species sediments there) is computed once; threshold tests and
// clamps run on the integer pipe (GB300's FP64 pipe is the bound).
#include "ice3gb_device.cuh"
#include "ice3gb_kernels.h"
#include "sedimentation_point.cuh"

namespace {
using namespace ice3sed;

__global__ void __launch_bounds__(128) sedimentation_kernel(const __grid_constant__ Cst c, SedArgs a)
{
  const long col = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (col >= a.nij) return;
  // PHYEX skips the cloud species when LSEDIC is off
  const bool skip_c = a.fortran && c.LSEDIC == 0.0;
  if (skip_c) {
    if (a.fpr[0])
      for (int k = 0; k < a.nk; ++k) a.fpr[0][(long)k * a.nij + col] = 0.0;
    a.inpr[0][col] = 0.0;
  }
  const bool has_st = a.sea != nullptr && a.town != nullptr;
  const double sea = a.sea ? a.sea[col] : 0.0, town = a.town ? a.town[col] : 0.0;
  const CloudPar cp = cloud_params(c, a.fortran, has_st, sea, town);
  SedColumnIO io;
  io.rhodref = a.rhodref; io.dzz = a.dzz; io.pabs = a.pabs; io.tht = a.tht;
  for (int s = 0; s < 5; ++s) {
    io.src_in[s] = a.src[s];
    io.src_out[s] = a.src[s];
    io.fpr[s] = a.fpr[s];
    io.inpr[s] = a.inpr[s];
  }
  io.nij = a.nij;
  io.nk = a.nk;
  sed_column_forward(c, a.fortran, skip_c, cp, a.dt, io, col);
  // hail (NRR = 7), an independent species: its own sweep of the column
  if (a.hsrc) sed_hail_column(c, a.dt, a.rhodref, a.dzz, a.hsrc, a.hfpr, a.hinpr, a.nij, a.nk, col);
}

// Fog deposition on the lowest level (rain_ice.F90:876-895).
// SEDIM = SPLI: one column per thread (sed_split_column).
__global__ void __launch_bounds__(128) sedimentation_split_kernel(const __grid_constant__ Cst c,
                                                                  const __grid_constant__ SplitArgs a)
{
  const long col = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (col >= a.sed.nij) return;
  const bool has_st = a.sed.sea != nullptr && a.sed.town != nullptr;
  const double sea = has_st ? a.sed.sea[col] : 0.0, town = has_st ? a.sed.town[col] : 0.0;
  const CloudPar cp = cloud_params(c, true, has_st, sea, town);
  const long n = (long)a.sed.nij * a.sed.nk;
  SplitColumnIO io;
  io.rhodref = a.sed.rhodref; io.dzz = a.sed.dzz; io.pabs = a.sed.pabs; io.tht = a.sed.tht; io.exn = a.exn;
  io.rvt = a.rvt; io.rvs = a.rvs; io.ths = a.ths;
  for (int s = 0; s < 5; ++s) {
    io.rt[s] = a.rt[s];
    io.src[s] = a.sed.src[s];
    io.fpr[s] = a.sed.fpr[s];
    io.inpr[s] = a.sed.inpr[s];
  }
  io.nsp = a.rht ? 6 : 5;
  io.rt[5] = a.rht;
  io.src[5] = a.sed.hsrc;
  io.fpr[5] = a.sed.hfpr;
  io.inpr[5] = a.sed.hinpr;
  io.rtmp = a.scratch;
  io.ext = a.scratch + n;
  io.nij = a.sed.nij;
  io.nk = a.sed.nk;
  if (!sed_split_column(c, cp, a.sed.dt, io, col, a.max_iter)) atomicOr(a.status, ICE3GB_DEV_SED_CAP);
}

__global__ void fog_deposition_kernel(const __grid_constant__ Cst c, FogArgs a)
{
  const long col = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (col >= a.nij) return;
  if (a.enabled) {
    const double rct = a.rct[col];
    const double indep = c.VDEPOSC * rct * a.rhodref[col] / c.RHOLW;
    a.rcs[col] -= c.VDEPOSC * rct / a.dzz[col];
    a.inprc[col] += indep;
    if (a.indep) a.indep[col] = indep;
  } else if (a.indep) {
    a.indep[col] = 0.0;
  }
}

}  // namespace

cudaError_t launch_sedimentation(const Cst &c, const SedArgs &a, cudaStream_t s)
{
  const long n = a.nij;
  const int threads = 128;
  sedimentation_kernel<<<(unsigned)((n + threads - 1) / threads), threads, 0, s>>>(c, a);
  return cudaGetLastError();
}

cudaError_t launch_sedimentation_split(const Cst &c, const SplitArgs &a, cudaStream_t s)
{
  const long n = a.sed.nij;
  const int threads = 128;
  sedimentation_split_kernel<<<(unsigned)((n + threads - 1) / threads), threads, 0, s>>>(c, a);
  return cudaGetLastError();
}

cudaError_t launch_fog_deposition(const Cst &c, const FogArgs &a, cudaStream_t s)
{
  const int threads = 256;
  fog_deposition_kernel<<<(unsigned)((a.nij + threads - 1) / threads), threads, 0, s>>>(c, a);
  return cudaGetLastError();
}
